// fw_step.cu -- the plain form for the phenomenological models
// (Aliev-Panfilov, Mitchell-Schaeffer, Fenton-Karma), the stand-alone
// diffusion pass, and the dispatch of the plain form and the ionic pass to
// the detailed models' translation units (fw_step_detailed_*.cu).
//
// Built with --fmad=false: the stencil sum and the ionic updates keep the
// reference's operation order without FMA contraction, so FP64 runs of the
// +,-,*,/-only models are bitwise equal to the reference's float64 path.
#include <stdio.h>

#include "fw_model_dispatch.cuh"
#include "fw_plain.cuh"

namespace fw {

int step_plain(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
               cudaStream_t stream)
{
    const bool f64 = a->precision == FW_F64;
    if (a->model == FW_MODEL_TP06)
        return f64 ? plain_tp06_f64(a, n_begin, n_steps, stream)
                   : plain_tp06_f32(a, n_begin, n_steps, stream);
    if (a->model == FW_MODEL_CRN)
        return f64 ? plain_crn_f64(a, n_begin, n_steps, stream)
                   : plain_crn_f32(a, n_begin, n_steps, stream);
    if (a->model == FW_MODEL_LR91)
        return f64 ? plain_lr91_f64(a, n_begin, n_steps, stream)
                   : plain_lr91_f32(a, n_begin, n_steps, stream);
    PlainDispatch d{a, n_begin, n_steps, stream};
    return dispatch_model_stencil(a->model, a->stencil, a->precision, d);
}

int ionic(int32_t model, int32_t precision, void *u_new, const void *u,
          void *const *state, const int64_t *idx, int64_t n_idx, double dt,
          const double *params, cudaStream_t stream)
{
    if ((model == FW_MODEL_TP06 || model == FW_MODEL_CRN ||
         model == FW_MODEL_LR91) &&
        precision != FW_F64 && precision != FW_F32) {
        set_error("unknown precision %d", precision);
        return FW_ERR_ARG;
    }
    const bool f64 = precision == FW_F64;
    if (model == FW_MODEL_TP06)
        return (f64 ? ionic_tp06_f64 : ionic_tp06_f32)(
            u_new, u, state, idx, n_idx, dt, params, stream);
    if (model == FW_MODEL_CRN)
        return (f64 ? ionic_crn_f64 : ionic_crn_f32)(
            u_new, u, state, idx, n_idx, dt, params, stream);
    if (model == FW_MODEL_LR91)
        return (f64 ? ionic_lr91_f64 : ionic_lr91_f32)(
            u_new, u, state, idx, n_idx, dt, params, stream);
    IonicDispatch d{u_new, u, state, idx, n_idx, dt, params, stream};
    return dispatch_model(model, precision, d);
}

int ecg(int32_t stencil, int32_t precision, const void *u, const void *w,
        const int8_t *myo, int64_t ni, int64_t nj, int64_t nk,
        const double *coords, int32_t n_leads, double dr, double *out,
        cudaStream_t stream)
{
    if (!stencil_nw(stencil) || !u || !w || !myo || !coords || !out) {
        set_error("fw_ecg: bad stencil or null pointer");
        return FW_ERR_ARG;
    }
    if (precision != FW_F64 && precision != FW_F32) {
        set_error("fw_ecg: unknown precision %d", precision);
        return FW_ERR_ARG;
    }
    {
        // the lead coordinates are read on the host: refuse device memory
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, coords) == cudaSuccess &&
            at.type == cudaMemoryTypeDevice) {
            set_error("fw_ecg: coords must be host memory");
            return FW_ERR_ARG;
        }
        cudaGetLastError();
    }
    const int dim = stencil_dim(stencil);
    Grid g = make_grid(ni, nj, nk, dim);
    const double(*xyz)[3] = reinterpret_cast<const double(*)[3]>(coords);
#define ECG_CASE(ST)                                                          \
    case ST:                                                                  \
        return precision == FW_F64                                            \
                   ? launch_ecg<ST, double>((const double *)u,                \
                                            (const double *)w, myo, g, dim,   \
                                            xyz, n_leads, dr, out, stream)    \
                   : launch_ecg<ST, float>((const float *)u, (const float *)w, \
                                           myo, g, dim, xyz, n_leads, dr, out, \
                                           stream);
    switch (stencil) {
        ECG_CASE(FW_STENCIL_ISO5)
        ECG_CASE(FW_STENCIL_ANISO9)
        ECG_CASE(FW_STENCIL_ISO7)
        ECG_CASE(FW_STENCIL_ANISO19)
        ECG_CASE(FW_STENCIL_ANISO19_XY)
    }
#undef ECG_CASE
    return FW_ERR_ARG;
}

int diffuse(int32_t stencil, int32_t precision, void *u_new, const void *u,
            const void *w, const int64_t *idx, int64_t n_idx, int64_t ni,
            int64_t nj, int64_t nk, cudaStream_t stream)
{
    int nw = stencil_nw(stencil);
    if (!nw || !u_new || !u || !w || (n_idx > 0 && !idx)) {
        set_error("fw_diffuse: bad stencil or null pointer");
        return FW_ERR_ARG;
    }
    Grid g = make_grid(ni, nj, nk, stencil_dim(stencil));
    if (n_idx <= 0) return FW_OK;
    int blocks = grid_for(n_idx, kThreads);
#define LAUNCH(ST)                                                             \
    if (precision == FW_F64)                                                   \
        k_diffuse<ST, double><<<blocks, kThreads, 0, stream>>>(               \
            (double *)u_new, (const double *)u, (const double *)w, idx, n_idx, \
            g.n, g.si, g.sj);                                                  \
    else                                                                       \
        k_diffuse<ST, float><<<blocks, kThreads, 0, stream>>>(                \
            (float *)u_new, (const float *)u, (const float *)w, idx, n_idx,    \
            g.n, g.si, g.sj);
    switch (stencil) {
    case FW_STENCIL_ISO5: LAUNCH(FW_STENCIL_ISO5); break;
    case FW_STENCIL_ANISO9: LAUNCH(FW_STENCIL_ANISO9); break;
    case FW_STENCIL_ISO7: LAUNCH(FW_STENCIL_ISO7); break;
    case FW_STENCIL_ANISO19: LAUNCH(FW_STENCIL_ANISO19); break;
    case FW_STENCIL_ANISO19_XY: LAUNCH(FW_STENCIL_ANISO19_XY); break;
    }
#undef LAUNCH
    FW_CHECK_LAUNCH("k_diffuse");
    return FW_OK;
}

}  // namespace fw
