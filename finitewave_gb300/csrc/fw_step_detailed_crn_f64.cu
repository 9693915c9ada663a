// fw_step_detailed_crn_f64.cu -- plain form and ionic pass of ModelCRN, double.
#include "fw_step_detailed.cuh"

FW_DETAILED_UNIT(ModelCRN, double, crn_f64)
