// fw_step_detailed_crn_f32.cu -- plain form and ionic pass of ModelCRN, float.
#include "fw_step_detailed.cuh"

FW_DETAILED_UNIT(ModelCRN, float, crn_f32)
