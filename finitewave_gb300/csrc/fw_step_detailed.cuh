// fw_step_detailed.cuh -- the plain form and the ionic pass of the detailed
// models (TP06, Courtemanche) at one fixed precision.  Each model x precision
// pair is its own translation unit (fw_step_detailed_*.cu): the expression
// trees are large, so splitting keeps the build parallel, and the float64
// units are compiled without FMA contraction (closest to the reference's
// evaluation order) while the float32 units use FMA and fast division.
#pragma once

#include "fw_models_big.cuh"
#include "fw_plain.cuh"

namespace fw {

template <class M, class T>
int plain_detailed(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                   cudaStream_t stream)
{
    switch (a->stencil) {
    case FW_STENCIL_ISO5:
        return run_plain<M, FW_STENCIL_ISO5, T>(a, n_begin, n_steps, stream);
    case FW_STENCIL_ANISO9:
        return run_plain<M, FW_STENCIL_ANISO9, T>(a, n_begin, n_steps, stream);
    case FW_STENCIL_ISO7:
        return run_plain<M, FW_STENCIL_ISO7, T>(a, n_begin, n_steps, stream);
    case FW_STENCIL_ANISO19:
        return run_plain<M, FW_STENCIL_ANISO19, T>(a, n_begin, n_steps, stream);
    case FW_STENCIL_ANISO19_XY:
        return run_plain<M, FW_STENCIL_ANISO19_XY, T>(a, n_begin, n_steps, stream);
    }
    set_error("unknown stencil %d", a->stencil);
    return FW_ERR_ARG;
}

}  // namespace fw

// Defines fw::plain_<NAME> and fw::ionic_<NAME> for model M at precision T.
#define FW_DETAILED_UNIT(M, T, NAME)                                          \
    namespace fw {                                                            \
    int plain_##NAME(const fw_step_args *a, int64_t n_begin, int64_t n_steps, \
                     cudaStream_t stream)                                     \
    {                                                                         \
        return plain_detailed<M, T>(a, n_begin, n_steps, stream);             \
    }                                                                         \
    int ionic_##NAME(void *u_new, const void *u, void *const *state,          \
                     const int64_t *idx, int64_t n_idx, double dt,            \
                     const double *params, cudaStream_t stream)               \
    {                                                                         \
        return run_ionic<M, T>(u_new, u, state, idx, n_idx, dt, params,       \
                               stream);                                       \
    }                                                                         \
    }
