// fw_internal.cuh -- shared definitions of the fwgpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fwgpu.h"

namespace fw {

// Error reporting: set by the entry points, read by fw_last_error().
void set_error(const char *fmt, ...);
int cuda_error(cudaError_t e, const char *what);

#define FW_CUDA_CHECK(call)                                  \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return fw::cuda_error(e_, #call); \
    } while (0)

// Counts every kernel launch of the library (fw_launch_count()).
void count_launch();

#define FW_CHECK_LAUNCH(what)                                \
    do {                                                     \
        fw::count_launch();                                  \
        cudaError_t e_ = cudaGetLastError();                 \
        if (e_ != cudaSuccess) return fw::cuda_error(e_, what); \
    } while (0)

inline int stencil_nw(int st)
{
    switch (st) {
    case FW_STENCIL_ISO5: return 5;
    case FW_STENCIL_ANISO9: return 9;
    case FW_STENCIL_ISO7: return 7;
    case FW_STENCIL_ANISO19: return 19;
    case FW_STENCIL_SYM9: return 9;
    case FW_STENCIL_ANISO19_XY: return 19;
    }
    return 0;
}

inline int stencil_dim(int st)
{
    return (st == FW_STENCIL_ISO5 || st == FW_STENCIL_ANISO9 ||
            st == FW_STENCIL_SYM9) ? 2 : 3;
}

// Grid strides of the axes i and j (k has stride 1).  In 2D the reference's
// j axis is the contiguous one, so si = nj and sj = 1.
struct Grid {
    int64_t ni, nj, nk, n;
    int64_t si, sj;
};

inline Grid make_grid(int64_t ni, int64_t nj, int64_t nk, int dim)
{
    Grid g;
    g.ni = ni;
    g.nj = nj;
    g.nk = dim == 2 ? 1 : nk;
    g.n = ni * nj * g.nk;
    if (dim == 2) {
        g.si = nj;
        g.sj = 1;
    } else {
        g.si = nj * nk;
        g.sj = nk;
    }
    return g;
}

// Diffusion sum for one node, weight-major weights, the reference's term
// order (left-to-right sum of products).  Callers compile this with FMA
// contraction disabled where bitwise parity is required.
template <int ST, class T>
__device__ __forceinline__ T diffuse_node(const T *__restrict__ u,
                                          const T *__restrict__ w, int64_t p,
                                          int64_t n, int64_t si, int64_t sj)
{
    if constexpr (ST == FW_STENCIL_ISO5) {
        // isotropic_stencil_2d.py:126-130
        return u[p - si] * w[p] + u[p - 1] * w[n + p] + u[p] * w[2 * n + p] +
               u[p + 1] * w[3 * n + p] + u[p + si] * w[4 * n + p];
    } else if constexpr (ST == FW_STENCIL_ANISO9) {
        // asymmetric_stencil_2d.py:192-200
        return u[p - si - 1] * w[p] + u[p - si] * w[n + p] +
               u[p - si + 1] * w[2 * n + p] + u[p - 1] * w[3 * n + p] +
               u[p] * w[4 * n + p] + u[p + 1] * w[5 * n + p] +
               u[p + si - 1] * w[6 * n + p] + u[p + si] * w[7 * n + p] +
               u[p + si + 1] * w[8 * n + p];
    } else if constexpr (ST == FW_STENCIL_ISO7) {
        // isotropic_stencil_3d.py:101-107
        return u[p - si] * w[p] + u[p - sj] * w[n + p] + u[p - 1] * w[2 * n + p] +
               u[p] * w[3 * n + p] + u[p + 1] * w[4 * n + p] +
               u[p + sj] * w[5 * n + p] + u[p + si] * w[6 * n + p];
    } else if constexpr (ST == FW_STENCIL_ANISO19_XY) {
        // asymmetric_stencil_3d.py:140-158 without the terms of planes 9,
        // 10 and 13-18, which are zero for in-plane fibers (adding them
        // changes no sum), in the same order
        return u[p - si - sj] * w[p] + u[p - si] * w[n + p] +
               u[p - si + sj] * w[2 * n + p] + u[p - sj] * w[3 * n + p] +
               u[p] * w[4 * n + p] + u[p + sj] * w[5 * n + p] +
               u[p + si - sj] * w[6 * n + p] + u[p + si] * w[7 * n + p] +
               u[p + si + sj] * w[8 * n + p] + u[p - 1] * w[11 * n + p] +
               u[p + 1] * w[12 * n + p];
    } else {
        // asymmetric_stencil_3d.py:140-158
        return u[p - si - sj] * w[p] + u[p - si] * w[n + p] +
               u[p - si + sj] * w[2 * n + p] + u[p - sj] * w[3 * n + p] +
               u[p] * w[4 * n + p] + u[p + sj] * w[5 * n + p] +
               u[p + si - sj] * w[6 * n + p] + u[p + si] * w[7 * n + p] +
               u[p + si + sj] * w[8 * n + p] + u[p - sj - 1] * w[9 * n + p] +
               u[p - sj + 1] * w[10 * n + p] + u[p - 1] * w[11 * n + p] +
               u[p + 1] * w[12 * n + p] + u[p + sj - 1] * w[13 * n + p] +
               u[p + sj + 1] * w[14 * n + p] + u[p - si - 1] * w[15 * n + p] +
               u[p + si - 1] * w[16 * n + p] + u[p - si + 1] * w[17 * n + p] +
               u[p + si + 1] * w[18 * n + p];
    }
}

// The in-plane 3D sum of diffuse_node<FW_STENCIL_ANISO19_XY> with the
// node's weights taken from a row of 12 values (planes 0-8, 11, 12 and a
// pad) of a table of distinct rows: the same products in the same order.
template <class T>
__device__ __forceinline__ T diffuse_row_xy(const T *__restrict__ u,
                                            const T *__restrict__ row, int64_t p,
                                            int64_t si, int64_t sj)
{
    T w[12];
    if constexpr (sizeof(T) == 4) {
        const float4 *r = reinterpret_cast<const float4 *>(row);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float4 v = __ldg(r + q);
            w[4 * q] = v.x;
            w[4 * q + 1] = v.y;
            w[4 * q + 2] = v.z;
            w[4 * q + 3] = v.w;
        }
    } else {
        const double2 *r = reinterpret_cast<const double2 *>(row);
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const double2 v = __ldg(r + q);
            w[2 * q] = v.x;
            w[2 * q + 1] = v.y;
        }
    }
    return u[p - si - sj] * w[0] + u[p - si] * w[1] + u[p - si + sj] * w[2] +
           u[p - sj] * w[3] + u[p] * w[4] + u[p + sj] * w[5] +
           u[p + si - sj] * w[6] + u[p + si] * w[7] + u[p + si + sj] * w[8] +
           u[p - 1] * w[9] + u[p + 1] * w[10];
}

// Launch helpers ------------------------------------------------------------

inline int grid_for(int64_t n, int threads, int max_blocks = 152 * 16)
{
    int64_t b = (n + threads - 1) / threads;
    if (b > max_blocks) b = max_blocks;
    if (b < 1) b = 1;
    return (int)b;
}

// Entry points implemented in the translation units.
int build_weights(int32_t stencil, int32_t precision, const int8_t *mesh,
                  const double *cond, double cond_scalar, const double *fibers,
                  double D_al, double D_ac, double D_model, double dt,
                  double dr2, int64_t ni, int64_t nj, int64_t nk, void *w_out,
                  cudaStream_t stream);
int diffuse(int32_t stencil, int32_t precision, void *u_new, const void *u,
            const void *w, const int64_t *idx, int64_t n_idx, int64_t ni,
            int64_t nj, int64_t nk, cudaStream_t stream);
int ionic(int32_t model, int32_t precision, void *u_new, const void *u,
          void *const *state, const int64_t *idx, int64_t n_idx, double dt,
          const double *params, cudaStream_t stream);
int step_plain(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
               cudaStream_t stream);
int ecg(int32_t stencil, int32_t precision, const void *u, const void *w,
        const int8_t *myo, int64_t ni, int64_t nj, int64_t nk,
        const double *coords, int32_t n_leads, double dr, double *out,
        cudaStream_t stream);
int step_fused(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
               cudaStream_t stream);
int pack_weights(int32_t stencil, const float *w, int64_t n, float *out,
                 cudaStream_t stream);
int step_fused_ap(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                  cudaStream_t stream);
int step_fused_ms(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                  cudaStream_t stream);
int step_fused_fk(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                  cudaStream_t stream);
int step_fused_bk(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                  cudaStream_t stream);

int batch_plan_size(const fw_step_args *const *tissues, int32_t n,
                    int64_t *bytes);
int batch_plan(const fw_step_args *const *tissues, int32_t n,
               const int64_t *n_begin, void *plan, int64_t plan_bytes,
               fw_batch *out, cudaStream_t stream);
int batch_run(const fw_batch *b, uint32_t *scratch, int64_t offset,
              int64_t n_steps, cudaStream_t stream);
constexpr int64_t kBatchScratchBytes = 256;
int batch_run_noalloc(const fw_batch *b, int64_t offset, int64_t n_steps,
                      cudaStream_t stream);

// Detailed models, one translation unit per model x precision
// (fw_step_detailed_*.cu).
#define FW_DECLARE_DETAILED(NAME)                                             \
    int plain_##NAME(const fw_step_args *a, int64_t n_begin, int64_t n_steps, \
                     cudaStream_t stream);                                    \
    int ionic_##NAME(void *u_new, const void *u, void *const *state,          \
                     const int64_t *idx, int64_t n_idx, double dt,            \
                     const double *params, cudaStream_t stream);
FW_DECLARE_DETAILED(tp06_f64)
FW_DECLARE_DETAILED(tp06_f32)
FW_DECLARE_DETAILED(crn_f64)
FW_DECLARE_DETAILED(crn_f32)
FW_DECLARE_DETAILED(lr91_f64)
FW_DECLARE_DETAILED(lr91_f32)
#undef FW_DECLARE_DETAILED

}  // namespace fw
