// fw_fused.cu -- entry of the fused, temporally blocked FP32 form: checks
// that the configuration has a fused kernel and dispatches per model (the
// kernels are in fw_fused_kernel.cuh and fw_fused_tma.cuh, instantiated in
// fw_fused_{ap,ms,fk}.cu), and the weight repacking for the TMA kernel.
#include "fw_internal.cuh"

namespace fw {

namespace {

// out[p * NWO + q] = w[plane(q) * n + p], plane(q) skipping the centre.
template <int NWO, int CENTRE>
__global__ void k_pack(const float *__restrict__ w, int64_t n,
                       float *__restrict__ out)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x) {
        float v[NWO];
#pragma unroll
        for (int q = 0; q < NWO; ++q) v[q] = w[(int64_t)(q < CENTRE ? q : q + 1) * n + p];
        float4 *o = reinterpret_cast<float4 *>(out + p * NWO);
#pragma unroll
        for (int q = 0; q < NWO / 4; ++q)
            o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
}

}  // namespace

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
    case FW_MODEL_BK: return step_fused_bk(a, n_begin, n_steps, stream);
    }
    set_error("fw_step (fused): model %d has no fused form", a->model);
    return FW_ERR_UNSUPPORTED;
}

int pack_weights(int32_t stencil, const float *w, int64_t n, float *out,
                 cudaStream_t stream)
{
    if (!w || !out || n <= 0) {
        set_error("fw_pack_weights: null pointer or empty grid");
        return FW_ERR_ARG;
    }
    if (((uintptr_t)out & 15) != 0) {
        set_error("fw_pack_weights: output must be 16-byte aligned");
        return FW_ERR_ARG;
    }
    const int threads = 256;
    const int blocks = grid_for(n, threads);
    if (stencil == FW_STENCIL_ISO5)
        k_pack<4, 2><<<blocks, threads, 0, stream>>>(w, n, out);
    else if (stencil == FW_STENCIL_ANISO9)
        k_pack<8, 4><<<blocks, threads, 0, stream>>>(w, n, out);
    else {
        set_error("fw_pack_weights: 2D stencils only");
        return FW_ERR_UNSUPPORTED;
    }
    FW_CHECK_LAUNCH("k_pack");
    return FW_OK;
}

}  // namespace fw
