// fw_step_detailed_tp06_f32.cu -- plain form and ionic pass of ModelTP06, float.
#include "fw_step_detailed.cuh"

FW_DETAILED_UNIT(ModelTP06, float, tp06_f32)
