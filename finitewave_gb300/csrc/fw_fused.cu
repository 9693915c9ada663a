// fw_fused.cu -- entry of the fused, temporally blocked FP32 form: checks
// that the configuration has a fused kernel and dispatches per model (the
// kernels are in fw_fused_kernel.cuh, instantiated in fw_fused_{ap,ms,fk}.cu).
#include "fw_internal.cuh"

namespace fw {

int step_fused(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
               cudaStream_t stream)
{
    if (a->precision != FW_F32) {
        set_error("fw_step (fused): float32 only");
        return FW_ERR_UNSUPPORTED;
    }
    if (a->ni > (1 << 30) || a->nj > (1 << 30)) {
        set_error("fw_step (fused): grid too large");
        return FW_ERR_ARG;
    }
    switch (a->model) {
    case FW_MODEL_AP: return step_fused_ap(a, n_begin, n_steps, stream);
    case FW_MODEL_MS: return step_fused_ms(a, n_begin, n_steps, stream);
    case FW_MODEL_FK: return step_fused_fk(a, n_begin, n_steps, stream);
    }
    set_error("fw_step (fused): model %d has no fused form", a->model);
    return FW_ERR_UNSUPPORTED;
}

}  // namespace fw
