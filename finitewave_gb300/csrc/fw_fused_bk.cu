// fw_fused_bk.cu -- instantiations of the fused FP32 kernel for ModelBK
// (one translation unit per model so that they compile in parallel).
#include "fw_fused_march.cuh"

namespace fw {

int step_fused_bk(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                  cudaStream_t stream)
{
    return fused::fused_model<ModelBK>(a, n_begin, n_steps, stream);
}

}  // namespace fw
