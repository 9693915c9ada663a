// fw_fused.cu -- placeholder for the temporally blocked FP32 form.
#include "fw_internal.cuh"

namespace fw {

int step_fused(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
               cudaStream_t stream)
{
    (void)a; (void)n_begin; (void)n_steps; (void)stream;
    set_error("fw_step: FW_FORM_FUSED not available for this configuration");
    return FW_ERR_UNSUPPORTED;
}

}  // namespace fw
