// fw_step_detailed_tp06_f64.cu -- plain form and ionic pass of ModelTP06, double.
#include "fw_step_detailed.cuh"

FW_DETAILED_UNIT(ModelTP06, double, tp06_f64)
