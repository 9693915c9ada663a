// fw_capi.cu -- the extern "C" entry points declared in include/fwgpu.h:
// argument validation, error reporting and dispatch to the kernels.
#include <stdarg.h>
#include <stdio.h>

#include <atomic>

#include "fw_internal.cuh"
#include "fw_model_dispatch.cuh"
#include "fw_models_big.cuh"

namespace fw {

static thread_local char g_err[512] = "";
static std::atomic<int64_t> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

int cuda_error(cudaError_t e, const char *what)
{
    set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    return FW_ERR_CUDA;
}

namespace {

struct Info {
    int ns, np;
};

Info model_info(int32_t model)
{
    switch (model) {
    case FW_MODEL_AP: return {ModelAP::NS, ModelAP::NP};
    case FW_MODEL_MS: return {ModelMS::NS, ModelMS::NP};
    case FW_MODEL_FK: return {ModelFK::NS, ModelFK::NP};
    case FW_MODEL_TP06: return {ModelTP06::NS, ModelTP06::NP};
    case FW_MODEL_CRN: return {ModelCRN::NS, ModelCRN::NP};
    case FW_MODEL_BK: return {ModelBK::NS, ModelBK::NP};
    case FW_MODEL_BO: return {ModelBO::NS, ModelBO::NP};
    case FW_MODEL_LR91: return {ModelLR91::NS, ModelLR91::NP};
    }
    return {-1, -1};
}

bool valid_window(const fw_window &w) { return w.stride > 0; }

int check_step_args(const fw_step_args *a, int64_t n_steps)
{
    if (!a) {
        set_error("fw_step: args is NULL");
        return FW_ERR_ARG;
    }
    Info mi = model_info(a->model);
    if (mi.ns < 0) {
        set_error("fw_step: model %d not supported", a->model);
        return FW_ERR_UNSUPPORTED;
    }
    int nw = stencil_nw(a->stencil);
    if (!nw) {
        set_error("fw_step: unknown stencil %d", a->stencil);
        return FW_ERR_ARG;
    }
    if (a->precision != FW_F64 && a->precision != FW_F32) {
        set_error("fw_step: unknown precision %d", a->precision);
        return FW_ERR_ARG;
    }
    if (a->form != FW_FORM_PLAIN && a->form != FW_FORM_FUSED) {
        set_error("fw_step: unknown form %d", a->form);
        return FW_ERR_ARG;
    }
    int dim = stencil_dim(a->stencil);
    if (a->ni < 3 || a->nj < 3 || (dim == 3 ? a->nk < 3 : a->nk != 1)) {
        set_error("fw_step: grid (%lld,%lld,%lld) does not fit a %dD stencil",
                  (long long)a->ni, (long long)a->nj, (long long)a->nk, dim);
        return FW_ERR_ARG;
    }
    if (a->ni * a->nj * a->nk > (int64_t)1 << 40) {
        set_error("fw_step: grid too large");
        return FW_ERR_ARG;
    }
    if (n_steps < 0 || n_steps > ((int64_t)1 << 31)) {
        set_error("fw_step: n_steps %lld out of range", (long long)n_steps);
        return FW_ERR_ARG;
    }
    if (a->pitch != 0 && a->pitch != a->nj) {
        set_error("fw_step: a row pitch other than nj is for batches only");
        return FW_ERR_UNSUPPORTED;
    }
    if (!a->mesh || !a->myo || !a->weights || !a->u[0] || !a->u[1] ||
        a->u[0] == a->u[1]) {
        set_error("fw_step: mesh/myo/weights/u buffers missing or aliased");
        return FW_ERR_ARG;
    }
    for (int i = 0; i < mi.ns; ++i)
        if (!a->state[i]) {
            set_error("fw_step: state variable %d is NULL", i);
            return FW_ERR_ARG;
        }
    if (a->n_stims < 0 || a->n_stims > FW_MAX_STIMS || a->n_at < 0 ||
        a->n_at > FW_MAX_AT || a->n_lat < 0 || a->n_lat > FW_MAX_LAT ||
        a->n_probe < 0 || a->n_probe > FW_MAX_PROBE) {
        set_error("fw_step: too many stimuli or trackers");
        return FW_ERR_ARG;
    }
    for (int i = 0; i < a->n_stims; ++i) {
        const fw_stim &s = a->stims[i];
        if (s.kind != FW_STIM_VOLTAGE && s.kind != FW_STIM_CURRENT) {
            set_error("fw_step: stimulus %d has unknown kind %d", i, s.kind);
            return FW_ERR_ARG;
        }
    }
    for (int i = 0; i < a->n_at; ++i)
        if (!valid_window(a->at[i].win) || !a->at[i].act_step) {
            set_error("fw_step: activation tracker %d invalid", i);
            return FW_ERR_ARG;
        }
    for (int i = 0; i < a->n_lat; ++i) {
        const fw_lat_tracker &L = a->lat[i];
        if (!valid_window(L.win) || !L.activated || !L.cross_count ||
            (L.capacity > 0 && !L.cross_steps) || L.capacity < 0) {
            set_error("fw_step: local activation tracker %d invalid", i);
            return FW_ERR_ARG;
        }
    }
    for (int i = 0; i < a->n_probe; ++i) {
        const fw_probe_tracker &P = a->probe[i];
        if (!valid_window(P.win) || P.n_cells < 1 || !P.cells || !P.out ||
            P.n_vars < 1 || P.n_vars > FW_MAX_PROBE_VARS || P.capacity < 0 ||
            P.sample_offset < 0) {
            set_error("fw_step: probe tracker %d invalid", i);
            return FW_ERR_ARG;
        }
        for (int v = 0; v < P.n_vars; ++v)
            if (P.var_ids[v] < 0 || P.var_ids[v] > mi.ns) {
                set_error("fw_step: probe tracker %d var id %d out of range", i,
                          P.var_ids[v]);
                return FW_ERR_ARG;
            }
    }
    if (a->n_ecg < 0 || a->n_ecg > FW_MAX_ECG) {
        set_error("fw_step: n_ecg %d out of range (0..%d)", a->n_ecg,
                  FW_MAX_ECG);
        return FW_ERR_ARG;
    }
    for (int i = 0; i < a->n_ecg; ++i) {
        const fw_ecg_tracker &E = a->ecg[i];
        if (!valid_window(E.win) || E.n_leads < 1 ||
            E.n_leads > FW_MAX_ECG_LEADS || !E.out || E.capacity < 0 ||
            E.sample_offset < 0) {
            set_error("fw_step: ECG tracker %d invalid", i);
            return FW_ERR_ARG;
        }
    }
    if (a->n_tip < 0 || a->n_tip > FW_MAX_TIP) {
        set_error("fw_step: n_tip %d out of range (0..%d)", a->n_tip,
                  FW_MAX_TIP);
        return FW_ERR_ARG;
    }
    for (int i = 0; i < a->n_tip; ++i) {
        const fw_tip_tracker &P = a->tip[i];
        if (!valid_window(P.win) || !P.u_prev || !P.out || !P.count ||
            P.capacity < 0 || P.capacity > INT32_MAX || P.sample_offset < 0) {
            set_error("fw_step: spiral tip tracker %d invalid", i);
            return FW_ERR_ARG;
        }
    }
    if ((a->n_ecg > 0 || a->n_tip > 0) && a->form == FW_FORM_FUSED) {
        set_error("fw_step: ECG and spiral tip trackers run in the plain "
                  "form only");
        return FW_ERR_UNSUPPORTED;
    }
    return FW_OK;
}

}  // namespace
}  // namespace fw

extern "C" {

int fw_version(void) { return 100; }

size_t fw_struct_size(int32_t which)
{
    switch (which) {
    case 0: return sizeof(fw_step_args);
    case 1: return sizeof(fw_stim);
    case 2: return sizeof(fw_at_tracker);
    case 3: return sizeof(fw_lat_tracker);
    case 4: return sizeof(fw_probe_tracker);
    case 5: return sizeof(fw_window);
    case 6: return sizeof(fw_batch);
    case 7: return sizeof(fw_ecg_tracker);
    case 8: return sizeof(fw_tip_tracker);
    case 9: return sizeof(fw_tip);
    }
    return 0;
}

const char *fw_last_error(void) { return fw::g_err; }

int64_t fw_launch_count(void) { return fw::g_launches.load(); }

int fw_model_info(int32_t model, int32_t *n_state, int32_t *n_params)
{
    fw::Info mi = fw::model_info(model);
    if (mi.ns < 0) {
        fw::set_error("fw_model_info: model %d not supported", model);
        return FW_ERR_UNSUPPORTED;
    }
    if (n_state) *n_state = mi.ns;
    if (n_params) *n_params = mi.np;
    return FW_OK;
}

int fw_state_is_f64(int32_t model, int32_t precision, int32_t index)
{
    (void)model;
    (void)index;
    return precision == FW_F64 ? 1 : 0;
}

int fw_state_is_pair(int32_t model, int32_t precision, int32_t index)
{
    if (precision != FW_F32) return 0;
    switch (model) {
    case FW_MODEL_TP06: return fw::ModelTP06::is_conc(index) ? 1 : 0;
    case FW_MODEL_CRN: return fw::ModelCRN::is_conc(index) ? 1 : 0;
    case FW_MODEL_LR91: return fw::ModelLR91::is_conc(index) ? 1 : 0;
    default: return 0;
    }
}

int fw_build_weights(int32_t stencil, int32_t precision, const int8_t *mesh,
                     const double *cond, double cond_scalar,
                     const double *fibers, double D_al, double D_ac,
                     double D_model, double dt, double dr2, int64_t ni,
                     int64_t nj, int64_t nk, void *w_out, void *stream)
{
    return fw::build_weights(stencil, precision, mesh, cond, cond_scalar,
                             fibers, D_al, D_ac, D_model, dt, dr2, ni, nj, nk,
                             w_out, (cudaStream_t)stream);
}

int fw_diffuse(int32_t stencil, int32_t precision, void *u_new, const void *u,
               const void *w, const int64_t *idx, int64_t n_idx, int64_t ni,
               int64_t nj, int64_t nk, void *stream)
{
    return fw::diffuse(stencil, precision, u_new, u, w, idx, n_idx, ni, nj, nk,
                       (cudaStream_t)stream);
}

int fw_ionic(int32_t model, int32_t precision, void *u_new, const void *u,
             void *const *state, const int64_t *idx, int64_t n_idx,
             double dt, const double *params, void *stream)
{
    fw::Info mi = fw::model_info(model);
    if (mi.ns < 0) {
        fw::set_error("fw_ionic: model %d not supported", model);
        return FW_ERR_UNSUPPORTED;
    }
    if (!u_new || !u || !state || !params || (n_idx > 0 && !idx)) {
        fw::set_error("fw_ionic: null pointer");
        return FW_ERR_ARG;
    }
    for (int i = 0; i < mi.ns; ++i)
        if (!state[i]) {
            fw::set_error("fw_ionic: state variable %d is NULL", i);
            return FW_ERR_ARG;
        }
    return fw::ionic(model, precision, u_new, u, state, idx, n_idx, dt, params,
                     (cudaStream_t)stream);
}

int fw_pack_weights(int32_t stencil, const float *w, int64_t n, float *out,
                    void *stream)
{
    return fw::pack_weights(stencil, w, n, out, (cudaStream_t)stream);
}

int fw_step(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
            void *stream)
{
    int rc = fw::check_step_args(a, n_steps);
    if (rc) return rc;
    if (n_steps == 0) return FW_OK;
    if (a->form == FW_FORM_FUSED)
        return fw::step_fused(a, n_begin, n_steps, (cudaStream_t)stream);
    return fw::step_plain(a, n_begin, n_steps, (cudaStream_t)stream);
}

int fw_ecg(int32_t stencil, int32_t precision, const void *u, const void *w,
           const int8_t *myo, int64_t ni, int64_t nj, int64_t nk,
           const double *coords, int32_t n_leads, double dr, double *out,
           void *stream)
{
    return fw::ecg(stencil, precision, u, w, myo, ni, nj, nk, coords, n_leads,
                   dr, out, (cudaStream_t)stream);
}

int fw_batch_plan_size(const fw_step_args *const *tissues, int32_t n,
                       int64_t *plan_bytes)
{
    return fw::batch_plan_size(tissues, n, plan_bytes);
}

int fw_batch_plan(const fw_step_args *const *tissues, int32_t n,
                  const int64_t *n_begin, void *plan, int64_t plan_bytes,
                  fw_batch *out, void *stream)
{
    return fw::batch_plan(tissues, n, n_begin, plan, plan_bytes, out,
                          (cudaStream_t)stream);
}

int fw_batch_scratch_size(int64_t *bytes)
{
    if (!bytes) {
        fw::set_error("fw_batch_scratch_size: NULL output");
        return FW_ERR_ARG;
    }
    *bytes = fw::kBatchScratchBytes;
    return FW_OK;
}

int fw_batch_run(const fw_batch *b, void *scratch, int64_t offset,
                 int64_t n_steps, void *stream)
{
    return fw::batch_run(b, (uint32_t *)scratch, offset, n_steps,
                         (cudaStream_t)stream);
}

int fw_batch_run_noalloc(const fw_batch *b, int64_t offset, int64_t n_steps,
                         void *stream)
{
    return fw::batch_run_noalloc(b, offset, n_steps, (cudaStream_t)stream);
}

}  // extern "C"
