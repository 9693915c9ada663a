// fw_step_detailed_lr91_f64.cu -- plain form and ionic pass of ModelLR91, double.
#include "fw_step_detailed.cuh"

FW_DETAILED_UNIT(ModelLR91, double, lr91_f64)
