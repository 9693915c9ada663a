// fw_step_detailed_lr91_f32.cu -- plain form and ionic pass of ModelLR91, float.
#include "fw_step_detailed.cuh"

FW_DETAILED_UNIT(ModelLR91, float, lr91_f32)
