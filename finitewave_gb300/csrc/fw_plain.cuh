// fw_plain.cuh -- kernels and host loop of the plain form of the monodomain
// step (one launch per time step) and of the stand-alone ionic pass, as
// templates over the model M, the stencil ST and the precision T.  Each
// translation unit that instantiates them picks its own FMA policy: the
// float64 path of the reference's +,-,*,/-only models is compiled with
// --fmad=false so that it is bitwise the reference's.
//
// Per time step n (core/model/cardiac_model.py:164-178):
//   1. k_stim      once per stimulus whose step window contains n, on u_cur
//   2. k_step      all nodes: trackers read u_cur (after stimuli, before the
//                  update, as tracker_next does after the kernels but before
//                  the swap); myocytes get u_nxt = diffusion + ionic
//   3. k_probe     when a probe tracker is active at n: u_cur and the state
//                  variables (already advanced, as the reference's trackers
//                  see them)
//   the caller's buffers then swap roles.
#pragma once

#include "fw_internal.cuh"
#include "fw_models.cuh"

namespace fw {
namespace {


constexpr int kThreads = 256;

template <class T>
struct StimK {
    const int8_t *mesh;
    const int8_t *mask;
    T *u;
    int64_t lo[3], ext[3];
    int64_t stride[3];
    int64_t count;
    double value, u_max;
    int kind, has_umax;
};

// StimVoltage*/StimCurrent* .stimulate (cpuwave2D/stimulation/*.py) over the
// stimulus box, restricted to mesh == 1 and the optional mask.
template <class T>
__global__ void k_stim(StimK<T> s)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
         t < s.count; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t c2 = t % s.ext[2];
        int64_t r = t / s.ext[2];
        int64_t c1 = r % s.ext[1];
        int64_t c0 = r / s.ext[1];
        int64_t p = (s.lo[0] + c0) * s.stride[0] + (s.lo[1] + c1) * s.stride[1] +
                    (s.lo[2] + c2) * s.stride[2];
        if (s.mesh[p] != 1) continue;
        if (s.mask && !s.mask[p]) continue;
        if (s.kind == FW_STIM_VOLTAGE) {
            s.u[p] = (T)s.value;
        } else {
            T x = s.u[p] + (T)s.value;
            if (s.has_umax && x > (T)s.u_max) x = (T)s.u_max;
            s.u[p] = x;
        }
    }
}

// Thresholds, parameters and dt are held in the kernel's precision T,
// rounded on the host: a float32 kernel then does no float64 conversions
// (GB300's float64 pipe is a small fraction of its float32 rate).
template <class T>
struct AtK {
    T thr;
    int32_t *act;
};

template <class T>
struct LatK {
    T thr;
    uint8_t *activated;
    int32_t *steps;
    int32_t *count;
    int32_t cap;
};

template <class T>
struct StepK {
    const int8_t *myo;
    const T *w;
    // FW_STENCIL_ANISO19_XY: the weights as distinct rows of 12 values
    // (planes 0-8, 11, 12, padding) and each node's row, or NULL
    const T *wrow;
    const int32_t *widx;
    const T *u;
    T *un;
    void *state[FW_MAX_STATE];
    T params[FW_MAX_PARAMS];
    T dt;
    int64_t n, si, sj;
    int64_t step;
    int32_t n_at, n_lat;
    AtK<T> at[FW_MAX_AT];
    LatK<T> lat[FW_MAX_LAT];
    int32_t *status;
};

template <class T>
__device__ __forceinline__ void track(const StepK<T> &k, int64_t p, T uc)
{
    for (int a = 0; a < k.n_at; ++a) {
        // (act_t < 0) & (u > threshold)  (activation_time_2d_tracker.py:61-63)
        if (uc > k.at[a].thr && k.at[a].act[p] < 0)
            k.at[a].act[p] = (int32_t)k.step;
    }
    for (int l = 0; l < k.n_lat; ++l) {
        // cross_threshold (local_activation_time_2d_tracker.py:71-89)
        const LatK<T> &L = k.lat[l];
        uint8_t act = L.activated[p];
        if (uc >= L.thr && !act) {
            L.activated[p] = 1;
            int32_t c = L.count[p];
            if (c < L.cap)
                L.steps[(int64_t)c * k.n + p] = (int32_t)k.step;
            else if (k.status)
                atomicOr(k.status, FW_DEV_LAT_OVERFLOW);
            L.count[p] = c + 1;
        } else if (uc < L.thr && act) {
            L.activated[p] = 0;
        }
    }
}

// Minimum resident CTAs per SM asked of the compiler for the float32
// k_step: models may set M::kMinBlocksF32 (the detailed models trade
// registers for the occupancy their memory latency needs); 1 otherwise.
template <class M, class T, class = void>
struct MinBlocks {
    static constexpr int value = 1;
};
template <class M>
struct MinBlocks<M, float, decltype(void(M::kMinBlocksF32))> {
    static constexpr int value = M::kMinBlocksF32;
};

template <class M, int ST, class T>
__global__ void __launch_bounds__(kThreads, (MinBlocks<M, T>::value))
    k_step(StepK<T> k)
{
    const Params<T, M::NP> P = load_params<T, M::NP>(k.params);
    const T dt = k.dt;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < k.n;
         p += (int64_t)gridDim.x * blockDim.x) {
        T uc = k.u[p];
        if (k.n_at | k.n_lat) track(k, p, uc);
        if (!k.myo[p]) continue;
        T un;
        if constexpr (ST == FW_STENCIL_ANISO19_XY) {
            if (k.wrow)
                un = diffuse_row_xy<T>(k.u, k.wrow + (int64_t)k.widx[p] * 12, p,
                                       k.si, k.sj);
            else
                un = diffuse_node<ST, T>(k.u, k.w, p, k.n, k.si, k.sj);
        } else {
            un = diffuse_node<ST, T>(k.u, k.w, p, k.n, k.si, k.sj);
        }
        auto st = M::template load<T>(k.state, p);
        un = M::template update<T>(uc, un, st, P, dt);
        M::template store<T>(k.state, p, st);
        k.un[p] = un;
        if (!isfinite(un) && k.status) atomicOr(k.status, FW_DEV_NONFINITE);
    }
}

struct ProbeOne {
    const int64_t *cells;
    double *out;
    int64_t sample;
    int64_t capacity;
    int32_t n_cells, n_vars;
    int32_t var_ids[FW_MAX_PROBE_VARS];
};

template <class T>
struct ProbeK {
    const T *u;
    void *state[FW_MAX_STATE];
    uint32_t f64_mask;
    uint32_t pair_mask;
    int32_t n;
    ProbeOne pr[FW_MAX_PROBE];
    int32_t *status;
};

template <class T>
__global__ void k_probe(ProbeK<T> k)
{
    for (int t = 0; t < k.n; ++t) {
        const ProbeOne &P = k.pr[t];
        if (P.sample >= P.capacity) {
            if (threadIdx.x == 0 && k.status)
                atomicOr(k.status, FW_DEV_PROBE_OVERFLOW);
            continue;
        }
        int total = P.n_cells * P.n_vars;
        for (int q = threadIdx.x; q < total; q += blockDim.x) {
            int v = q / P.n_cells, c = q % P.n_cells;
            int64_t p = P.cells[c];
            int id = P.var_ids[v];
            double x;
            if (id == 0)
                x = (double)k.u[p];
            else if ((k.f64_mask >> (id - 1)) & 1u)
                x = ((const double *)k.state[id - 1])[p];
            else if ((k.pair_mask >> (id - 1)) & 1u) {
                const float2 c = ((const float2 *)k.state[id - 1])[p];
                x = (double)c.x + (double)c.y;
            }
            else
                x = (double)((const T *)k.state[id - 1])[p];
            P.out[(P.sample * P.n_vars + v) * (int64_t)P.n_cells + c] = x;
        }
    }
}

// ECG leads (ecg_2d_tracker.py:114-153, ecg_3d_tracker.py:99-140): per
// myocyte the diffusion increment diffuse(u) - u weighted by 1 / (d dr),
// d the squared distance to the lead; per-thread partial sums in T, a block
// reduction in float64, one float64 atomic add per block and lead.
template <class T>
struct EcgK {
    const T *u;
    const T *w;
    const int8_t *myo;
    int64_t n, si, sj, nj, nk;
    int32_t dim, n_leads;
    T xyz[FW_MAX_ECG_LEADS][3];
    T dr;
    double *out;
};

template <int ST, class T>
__global__ void __launch_bounds__(kThreads) k_ecg(EcgK<T> k)
{
    T acc[FW_MAX_ECG_LEADS];
#pragma unroll
    for (int c = 0; c < FW_MAX_ECG_LEADS; ++c) acc[c] = (T)0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < k.n;
         p += (int64_t)gridDim.x * blockDim.x) {
        if (!k.myo[p]) continue;
        const T diff = diffuse_node<ST, T>(k.u, k.w, p, k.n, k.si, k.sj) - k.u[p];
        T fi, fj, fk;
        if (k.dim == 2) {
            fi = (T)(p / k.nj);
            fj = (T)(p % k.nj);
            fk = (T)0;
        } else {
            const int64_t plane = k.nj * k.nk, r = p % plane;
            fi = (T)(p / plane);
            fj = (T)(r / k.nk);
            fk = (T)(r % k.nk);
        }
#pragma unroll
        for (int c = 0; c < FW_MAX_ECG_LEADS; ++c) {
            if (c >= k.n_leads) break;
            const T dx = k.xyz[c][0] - fi, dy = k.xyz[c][1] - fj,
                    dz = k.xyz[c][2] - fk;
            const T d = dx * dx + dy * dy + dz * dz;
            if (d > (T)0) acc[c] += diff / (d * k.dr);
        }
    }
    __shared__ double red[FW_MAX_ECG_LEADS][kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < FW_MAX_ECG_LEADS; ++c) {
        double v = (double)acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[c][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < FW_MAX_ECG_LEADS && (int)threadIdx.x < k.n_leads) {
        double v = 0.0;
        for (int q = 0; q < kThreads / 32; ++q) v += red[threadIdx.x][q];
        atomicAdd(&k.out[threadIdx.x], v);
    }
}

template <int ST, class T>
int launch_ecg(const T *u, const T *w, const int8_t *myo, const Grid &g,
               int dim, const double (*coords)[3], int n_leads, double dr,
               double *out, cudaStream_t stream)
{
    if (n_leads < 1 || n_leads > FW_MAX_ECG_LEADS) {
        set_error("ECG: %d leads (1..%d)", n_leads, FW_MAX_ECG_LEADS);
        return FW_ERR_ARG;
    }
    EcgK<T> k;
    k.u = u;
    k.w = w;
    k.myo = myo;
    k.n = g.n;
    k.si = g.si;
    k.sj = g.sj;
    k.nj = g.nj;
    k.nk = g.nk;
    k.dim = dim;
    k.n_leads = n_leads;
    for (int c = 0; c < FW_MAX_ECG_LEADS; ++c)
        for (int a = 0; a < 3; ++a)
            k.xyz[c][a] = c < n_leads ? (T)coords[c][a] : (T)0;
    k.dr = (T)dr;
    k.out = out;
    k_ecg<ST, T><<<grid_for(g.n, kThreads, 152 * 8), kThreads, 0, stream>>>(k);
    FW_CHECK_LAUNCH("k_ecg");
    return FW_OK;
}

// Spiral-wave tips (spiral_wave_core_2d_tracker.py:88-249): the cell
// (i, j)-(i+1, j+1) holds a tip when the threshold isoline crosses it in
// both the previous and the current potential; the tip is the intersection
// of the two bilinear isolines inside the cell (_correct_tip_pos), found in
// float64.
template <class T>
struct TipK {
    const T *u_prev;
    const T *u;
    int64_t ni, nj, nk;   // slice (i, j) planes; k the z index (nk = 1 in 2D)
    double thr;
    fw_tip *out;
    int32_t *count;
    int64_t capacity;
    int32_t sample;
    int32_t *status;
};

template <class T>
__global__ void __launch_bounds__(kThreads) k_tips(TipK<T> k)
{
    const int64_t di = k.ni - 10, dj = k.nj - 10;
    if (di <= 0 || dj <= 0) return;
    const int64_t cells = di * dj * k.nk;
    const T thr = (T)k.thr;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
         t < cells; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kk = t % k.nk;
        const int64_t r = t / k.nk;
        const int64_t j = 5 + r % dj, i = 5 + r / dj;
        // element (i, j) of z layer kk; rows of a layer are nj * nk apart
        const int64_t si = k.nj * k.nk, sj = k.nk;
        const int64_t p = i * si + j * sj + kk;
        // neighbours: (i+1, j) = p + si, (i, j+1) = p + sj
        const T *up = k.u_prev, *uc = k.u;
        auto crosses = [&](const T *u) {
            const T a = u[p], b = u[p + si], c = u[p + sj], d = u[p + si + sj];
            if (a >= thr && (b < thr || c < thr || d < thr)) return 1;
            if (a < thr && (b >= thr || c >= thr || d >= thr)) return 1;
            return 0;
        };
        int counter = crosses(up);
        if (counter == 1) counter += crosses(uc);
        if (counter != 2) continue;
        // _correct_tip_pos (spiral_wave_core_2d_tracker.py:98-146)
        const double u00 = up[p], u01 = up[p + sj], u10 = up[p + si],
                     u11 = up[p + si + sj];
        const double n00 = uc[p], n01 = uc[p + sj], n10 = uc[p + si],
                     n11 = uc[p + si + sj];
        const double th = k.thr;
        const double AC = u00 - u01 + u11 - u10;
        const double GC = u01 - u00;
        const double BC = u10 - u00;
        const double DC = u00 - th;
        const double AD = n00 - n01 + n11 - n10;
        const double GD = n01 - n00;
        const double BD = n10 - n00;
        const double DD = n00 - th;
        const double Q = BC * AD - BD * AC;
        const double R = GC * AD - GD * AC;
        const double S = DC * AD - DD * AC;
        const double QOnR = Q / R;
        const double SOnR = S / R;
        const double Tq = AC * QOnR;
        const double U = AC * SOnR - BC + GC * QOnR;
        const double V = GC * SOnR - DC;
        const double disc = U * U - 4. * Tq * V;
        if (disc < 0) continue;
        const double T2 = 2. * Tq;
        if (T2 == 0.) continue;
        const double sq = sqrt(disc);
        const double xn = (-U - sq) / T2, xp = (-U + sq) / T2;
        const double yn = -QOnR * xn - SOnR, yp = -QOnR * xp - SOnR;
        double cx, cy;
        if (0 <= xn && xn <= 1 && 0 <= yn && yn <= 1) {
            cx = xn;
            cy = yn;
        } else if (0 <= xp && xp <= 1 && 0 <= yp && yp <= 1) {
            cx = xp;
            cy = yp;
        } else {
            continue;
        }
        const int32_t slot = atomicAdd(k.count, 1);
        if (slot < k.capacity) {
            fw_tip &o = k.out[slot];
            o.sample = k.sample;
            o.k = (int32_t)kk;
            o.i = (int32_t)i;
            o.j = (int32_t)j;
            o.x = (double)j + cy;
            o.y = (double)i + cx;
        } else if (k.status) {
            atomicOr(k.status, FW_DEV_TIP_OVERFLOW);
        }
    }
}

template <int ST, class T>
__global__ void k_diffuse(T *un, const T *u, const T *w, const int64_t *idx,
                          int64_t n_idx, int64_t n, int64_t si, int64_t sj)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_idx;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t p = idx[t];
        un[p] = diffuse_node<ST, T>(u, w, p, n, si, sj);
    }
}

template <class M, class T>
struct IonicK {
    T *un;
    const T *u;
    void *state[FW_MAX_STATE];
    T params[FW_MAX_PARAMS];
    T dt;
    const int64_t *idx;
    int64_t n_idx;
};

template <class M, class T>
__global__ void k_ionic(IonicK<M, T> k)
{
    const Params<T, M::NP> P = load_params<T, M::NP>(k.params);
    const T dt = k.dt;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
         t < k.n_idx; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t p = k.idx[t];
        auto st = M::template load<T>(k.state, p);
        k.un[p] = M::template update<T>(k.u[p], k.un[p], st, P, dt);
        M::template store<T>(k.state, p, st);
    }
}

bool in_window(const fw_window &w, int64_t n)
{
    return w.stride > 0 && n >= w.first && n <= w.last && n % w.stride == 0;
}

template <class T>
int launch_stim(const fw_step_args *a, const fw_stim &s, T *u,
                cudaStream_t stream)
{
    StimK<T> k;
    int dim = stencil_dim(a->stencil);
    Grid g = make_grid(a->ni, a->nj, a->nk, dim);
    int64_t shape[3] = {g.ni, g.nj, g.nk};
    k.mesh = a->mesh;
    k.mask = s.mask;
    k.u = u;
    k.count = 1;
    for (int d = 0; d < 3; ++d) {
        int64_t lo = d < dim ? s.lo[d] : 0, hi = d < dim ? s.hi[d] : 1;
        if (lo < 0) lo = 0;
        if (hi > shape[d]) hi = shape[d];
        if (hi <= lo) return FW_OK;
        k.lo[d] = lo;
        k.ext[d] = hi - lo;
        k.count *= hi - lo;
    }
    k.stride[0] = g.si;
    k.stride[1] = dim == 2 ? 1 : g.sj;
    k.stride[2] = 1;
    k.value = s.value;
    k.u_max = s.u_max;
    k.kind = s.kind;
    k.has_umax = s.has_umax;
    k_stim<T><<<grid_for(k.count, kThreads), kThreads, 0, stream>>>(k);
    FW_CHECK_LAUNCH("k_stim");
    return FW_OK;
}

template <class M, int ST, class T>
int run_plain(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
              cudaStream_t stream)
{
    int dim = stencil_dim(ST);
    Grid g = make_grid(a->ni, a->nj, a->nk, dim);
    StepK<T> k;
    k.myo = a->myo;
    k.w = (const T *)a->weights;
    k.wrow = (const T *)a->weight_rows;
    k.widx = a->weight_row_index;
    if (k.wrow && (ST != FW_STENCIL_ANISO19_XY || !k.widx ||
                   ((uintptr_t)k.wrow & 15) != 0)) {
        set_error("fw_step: weight_rows needs FW_STENCIL_ANISO19_XY, a row "
                  "index and 16-byte aligned rows");
        return FW_ERR_ARG;
    }
    for (int i = 0; i < FW_MAX_STATE; ++i) k.state[i] = a->state[i];
    for (int i = 0; i < FW_MAX_PARAMS; ++i) k.params[i] = (T)a->params[i];
    k.dt = (T)a->dt;
    k.n = g.n;
    k.si = g.si;
    k.sj = g.sj;
    k.status = a->status;

    ProbeK<T> pk;
    pk.status = a->status;
    for (int i = 0; i < FW_MAX_STATE; ++i) pk.state[i] = a->state[i];
    pk.f64_mask = pk.pair_mask = 0;
    for (int i = 0; i < M::NS; ++i) {
        if (fw_state_is_f64(a->model, a->precision, i)) pk.f64_mask |= 1u << i;
        if (fw_state_is_pair(a->model, a->precision, i)) pk.pair_mask |= 1u << i;
    }

    const int blocks = grid_for(g.n, kThreads, 152 * 8);
    for (int64_t s = 0; s < n_steps; ++s) {
        const int64_t n = n_begin + s;
        T *cur = (T *)a->u[s & 1];
        T *nxt = (T *)a->u[(s + 1) & 1];
        for (int i = 0; i < a->n_stims; ++i) {
            const fw_stim &st = a->stims[i];
            if (n >= st.first && n <= st.last) {
                int rc = launch_stim<T>(a, st, cur, stream);
                if (rc) return rc;
            }
        }
        k.u = cur;
        k.un = nxt;
        k.step = n;
        k.n_at = 0;
        for (int i = 0; i < a->n_at; ++i)
            if (in_window(a->at[i].win, n))
                k.at[k.n_at++] = AtK<T>{(T)a->at[i].threshold,
                                        a->at[i].act_step};
        k.n_lat = 0;
        for (int i = 0; i < a->n_lat; ++i)
            if (in_window(a->lat[i].win, n)) {
                const fw_lat_tracker &L = a->lat[i];
                k.lat[k.n_lat++] = LatK<T>{(T)L.threshold, L.activated,
                                        L.cross_steps, L.cross_count,
                                        L.capacity};
            }
        k_step<M, ST, T><<<blocks, kThreads, 0, stream>>>(k);
        FW_CHECK_LAUNCH("k_step");
        pk.n = 0;
        for (int i = 0; i < a->n_probe; ++i) {
            const fw_probe_tracker &P = a->probe[i];
            if (!in_window(P.win, n)) continue;
            ProbeOne &o = pk.pr[pk.n++];
            o.cells = P.cells;
            o.out = P.out;
            o.sample = P.sample_offset + (n - P.win.first) / P.win.stride;
            o.capacity = P.capacity;
            o.n_cells = P.n_cells;
            o.n_vars = P.n_vars;
            for (int v = 0; v < FW_MAX_PROBE_VARS; ++v) o.var_ids[v] = P.var_ids[v];
        }
        if (pk.n) {
            pk.u = cur;
            k_probe<T><<<1, 128, 0, stream>>>(pk);
            FW_CHECK_LAUNCH("k_probe");
        }
        for (int i = 0; i < a->n_ecg; ++i) {
            const fw_ecg_tracker &E = a->ecg[i];
            if (!in_window(E.win, n)) continue;
            const int64_t smp = E.sample_offset + (n - E.win.first) / E.win.stride;
            if (smp < 0 || smp >= E.capacity) {
                set_error("fw_step: ECG sample %lld outside its capacity %lld",
                          (long long)smp, (long long)E.capacity);
                return FW_ERR_ARG;
            }
            int rc = launch_ecg<ST, T>(cur, k.w, a->myo, g, dim, E.coords,
                                       E.n_leads, E.dr,
                                       E.out + smp * E.n_leads, stream);
            if (rc) return rc;
        }
        for (int i = 0; i < a->n_tip; ++i) {
            const fw_tip_tracker &P = a->tip[i];
            if (!in_window(P.win, n)) continue;
            TipK<T> tk;
            tk.u_prev = (const T *)P.u_prev;
            tk.u = cur;
            tk.ni = g.ni;
            tk.nj = g.nj;
            tk.nk = g.nk;
            tk.thr = P.threshold;
            tk.out = P.out;
            tk.count = P.count;
            tk.capacity = P.capacity;
            tk.sample = (int32_t)(P.sample_offset + (n - P.win.first) / P.win.stride);
            tk.status = a->status;
            const int64_t cells = (g.ni > 10 && g.nj > 10)
                                      ? (g.ni - 10) * (g.nj - 10) * g.nk : 0;
            if (cells > 0) {
                k_tips<T><<<grid_for(cells, kThreads, 152 * 8), kThreads, 0,
                            stream>>>(tk);
                FW_CHECK_LAUNCH("k_tips");
            }
            FW_CUDA_CHECK(cudaMemcpyAsync(P.u_prev, cur, g.n * sizeof(T),
                                          cudaMemcpyDeviceToDevice, stream));
        }
    }
    return FW_OK;
}

template <class M, class T>
int run_ionic(void *u_new, const void *u, void *const *state,
              const int64_t *idx, int64_t n_idx, double dt,
              const double *params, cudaStream_t stream)
{
    IonicK<M, T> k;
    k.un = (T *)u_new;
    k.u = (const T *)u;
    for (int i = 0; i < FW_MAX_STATE; ++i) k.state[i] = i < M::NS ? state[i] : nullptr;
    for (int i = 0; i < FW_MAX_PARAMS; ++i)
        k.params[i] = i < M::NP ? (T)params[i] : (T)0;
    k.dt = (T)dt;
    k.idx = idx;
    k.n_idx = n_idx;
    if (n_idx > 0) k_ionic<M, T><<<grid_for(n_idx, kThreads), kThreads, 0, stream>>>(k);
    FW_CHECK_LAUNCH("k_ionic");
    return FW_OK;
}

struct PlainDispatch {
    const fw_step_args *a;
    int64_t n_begin, n_steps;
    cudaStream_t stream;
    template <class M, int ST, class T>
    int run() const { return run_plain<M, ST, T>(a, n_begin, n_steps, stream); }
};

struct IonicDispatch {
    void *u_new;
    const void *u;
    void *const *state;
    const int64_t *idx;
    int64_t n_idx;
    double dt;
    const double *params;
    cudaStream_t stream;
    template <class M, class T>
    int run() const
    {
        return run_ionic<M, T>(u_new, u, state, idx, n_idx, dt, params, stream);
    }
};

}  // namespace
}  // namespace fw
