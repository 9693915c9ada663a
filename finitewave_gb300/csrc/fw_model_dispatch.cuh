// fw_model_dispatch.cuh -- map runtime (model, stencil, precision) enums to
// template instantiations.
#pragma once

#include "fw_internal.cuh"
#include "fw_models.cuh"

namespace fw {

template <class F>
int dispatch_model(int32_t model, int32_t precision, const F &f)
{
#define FW_MODEL_CASE(ID, M)                                        \
    case ID:                                                        \
        return precision == FW_F64 ? f.template run<M, double>()    \
                                   : f.template run<M, float>();
    if (precision != FW_F64 && precision != FW_F32) {
        set_error("unknown precision %d", precision);
        return FW_ERR_ARG;
    }
    switch (model) {
        FW_MODEL_CASE(FW_MODEL_AP, ModelAP)
        FW_MODEL_CASE(FW_MODEL_MS, ModelMS)
        FW_MODEL_CASE(FW_MODEL_FK, ModelFK)
        FW_MODEL_CASE(FW_MODEL_BK, ModelBK)
        FW_MODEL_CASE(FW_MODEL_BO, ModelBO)
    }
#undef FW_MODEL_CASE
    set_error("model %d not supported", model);
    return FW_ERR_UNSUPPORTED;
}

template <class M, class F>
int dispatch_stencil(int32_t stencil, int32_t precision, const F &f)
{
#define FW_ST_CASE(ST)                                                   \
    case ST:                                                             \
        return precision == FW_F64 ? f.template run<M, ST, double>()     \
                                   : f.template run<M, ST, float>();
    switch (stencil) {
        FW_ST_CASE(FW_STENCIL_ISO5)
        FW_ST_CASE(FW_STENCIL_ANISO9)
        FW_ST_CASE(FW_STENCIL_ISO7)
        FW_ST_CASE(FW_STENCIL_ANISO19)
        FW_ST_CASE(FW_STENCIL_ANISO19_XY)
    }
#undef FW_ST_CASE
    set_error("unknown stencil %d", stencil);
    return FW_ERR_ARG;
}

template <class F>
int dispatch_model_stencil(int32_t model, int32_t stencil, int32_t precision,
                           const F &f)
{
    if (precision != FW_F64 && precision != FW_F32) {
        set_error("unknown precision %d", precision);
        return FW_ERR_ARG;
    }
    switch (model) {
    case FW_MODEL_AP: return dispatch_stencil<ModelAP>(stencil, precision, f);
    case FW_MODEL_MS: return dispatch_stencil<ModelMS>(stencil, precision, f);
    case FW_MODEL_FK: return dispatch_stencil<ModelFK>(stencil, precision, f);
    case FW_MODEL_BK: return dispatch_stencil<ModelBK>(stencil, precision, f);
    case FW_MODEL_BO: return dispatch_stencil<ModelBO>(stencil, precision, f);
    }
    set_error("model %d not supported", model);
    return FW_ERR_UNSUPPORTED;
}

}  // namespace fw
