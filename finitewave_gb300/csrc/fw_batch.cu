// fw_batch.cu -- many independent 2D float32 tissues advanced together by one
// persistent kernel over a ragged tile list.
//
// Each tissue is described by the same fw_step_args as a single-tissue run
// (Aliev-Panfilov, Mitchell-Schaeffer or Fenton-Karma; 5- or 9-point
// stencil; any size).  fw_batch_plan turns the tissues into a device
// descriptor table plus a list of (tissue, tile) pairs covering every tissue
// with the fused form's temporally blocked regions; fw_batch_run then
// advances all tissues by K time steps per launch.  The CTAs of a launch are
// persistent (a few per SM) and take tiles from a shared counter in a small
// caller-provided scratch buffer, so tissues of different models and sizes
// balance across the GPU; the last CTA to finish resets the counters, so the
// scratch stays zero between launches.
//
// A tile is the fused form's region (fw_fused_kernel.cuh): the off-centre
// weights and the potential staged with cp.async into shared memory, the
// ionic state and centre weights of each thread's strip in registers, K
// sub-steps on chip with the fused kernels' FMA chain (so a batched tissue
// is bitwise the same as the tissue run alone), the interior written back.  Stimulus and tracker windows are evaluated on the
// device from each tissue's step windows, so a launch needs no per-launch
// host data beyond the step offset.  Per sub-step, in the reference's order
// (core/model/cardiac_model.py:164-178): stimuli, activation / local
// activation trackers on u after the stimuli, diffusion + ionic update.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "fw_fused_kernel.cuh"

namespace fw {
namespace batch {

constexpr int kMaxState = 2;    // AP, MS: 1; FK: 2
constexpr int kMaxParams = 12;  // FK: 11
constexpr int KMAX = 4;         // time steps per launch (fixed per build)
constexpr int LW = 64, LH = 32, R = 8;
constexpr int NT = LW * (LH / R);
constexpr int TI = LH - 2 * KMAX, TJ = LW - 2 * KMAX;

struct BStim {
    int64_t first, last;
    int32_t kind, has_umax;
    float value, u_max;
    int32_t lo0, hi0, lo1, hi1;
    const int8_t *mask;
};

struct BWin {
    int64_t first, last, stride;
};

// Per-tissue scalars and pointers, staged into shared memory at the start
// of each tile (so that the sub-step loops read them without reloading
// from global memory around their own global stores).
struct BHead {
    const float *w;
    const int8_t *myo;
    float *u[2];
    void *state[kMaxState];
    float params[kMaxParams];
    float dt;
    int32_t model, stencil;
    int32_t ni, nj, tiles_j;
    int32_t n_stims, has_at, has_lat;
    int64_t n, step_base;
    BWin at_win;
    float at_thr;
    int32_t *at_act;
    BWin lat_win;
    float lat_thr;
    int32_t lat_cap;
    uint8_t *lat_activated;
    int32_t *lat_steps;
    int32_t *lat_count;
    int32_t *status;
};

struct BTissue {
    BHead h;
    BStim stims[FW_MAX_STIMS];
};

struct BTile {
    int32_t tissue, tile;
};

struct BSmem {
    float4 w[2][LH][LW];
    float u[2][LH + 2][LW + 2];
    BHead h;
    uint32_t stim_on[FW_MAX_STIMS];
    uint32_t any_stim, at_on, lat_on;
    int next;
};
static_assert(sizeof(BHead) % 4 == 0, "BHead is staged in 4-byte words");

// Sub-steps s < ks of a launch starting at tissue step n0 that fall inside
// [first, last] and on a multiple of stride.
__device__ __forceinline__ uint32_t window_bits(int64_t n0, int ks,
                                                int64_t first, int64_t last,
                                                int64_t stride)
{
    uint32_t m = 0;
    for (int s = 0; s < ks; ++s) {
        const int64_t n = n0 + s;
        if (n >= first && n <= last && (stride == 1 || n % stride == 0))
            m |= 1u << s;
    }
    return m;
}

__device__ __noinline__ void lat_append(const BHead &T, int64_t p, int64_t n)
{
    const int32_t c = T.lat_count[p];
    if (c < T.lat_cap)
        T.lat_steps[(int64_t)c * T.n + p] = (int32_t)n;
    else if (T.status)
        atomicOr(T.status, FW_DEV_LAT_OVERFLOW);
    T.lat_count[p] = c + 1;
}

// One tile of a tissue: K sub-steps from tissue step n0, input buffer
// u[in_buf].  The tissue's head and the per-sub-step event bits are in S
// (staged before the call, visible after the staging barrier below); its
// stimuli are read from `stims` in global memory.
template <class M, int ST>
__device__ __forceinline__ void run_tile(const BStim *stims, int tile,
                                         int64_t n0, int ks, int in_buf,
                                         BSmem &S)
{
    const BHead &T = S.h;
    constexpr int NWO = fused::Stencil2D<ST>::NWO;
    constexpr int CEN = fused::Stencil2D<ST>::CENTRE;
    const int tid = threadIdx.x;
    const int col = tid % LW;
    const int r0 = (tid / LW) * R;
    const int bi = tile / T.tiles_j, bj = tile % T.tiles_j;
    const int oi = bi * TI - KMAX;
    const int oj = bj * TJ - KMAX;
    const int gj = oj + col;
    const bool col_in = gj >= 0 && gj < T.nj;
    const bool col_interior = col >= KMAX && col < KMAX + TJ;
    const float *u_in = T.u[in_buf];
    float *u_out = T.u[in_buf ^ 1];

    {
        constexpr int ROWS = NT / LW, PER = LH / ROWS;
        const int lr0 = tid / LW;
        const float *wbase[NWO];
#pragma unroll
        for (int q = 0; q < NWO; ++q)
            wbase[q] = T.w + (int64_t)(q < CEN ? q : q + 1) * T.n;
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const int lr = lr0 + i * ROWS;
            const int gi = oi + lr;
            const bool in = col_in && gi >= 0 && gi < T.ni;
            const int64_t p = in ? (int64_t)gi * T.nj + gj : 0;
            fused::cp_async4(&S.u[0][lr + 1][col + 1], u_in + p, in);
#pragma unroll
            for (int q = 0; q < NWO; ++q)
                fused::cp_async4(
                    reinterpret_cast<float *>(&S.w[q >> 2][lr][col]) + (q & 3),
                    wbase[q] + p, in);
        }
    }
    typename M::template St<float> st[R];
    float wcen[R];
    uint32_t myo_bits = 0, own = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int lr = r0 + r, gi = oi + lr;
        const bool in = col_in && gi >= 0 && gi < T.ni;
        const int64_t p = in ? (int64_t)gi * T.nj + gj : 0;
        const int8_t m = T.myo[p];
        st[r] = M::template load<float>(T.state, p);
        wcen[r] = T.w[(int64_t)CEN * T.n + p];
        if (in && m) myo_bits |= 1u << r;
        if (in && col_interior && lr >= KMAX && lr < KMAX + TI) own |= 1u << r;
    }
    for (int i = tid; i < 2 * (LW + 2); i += NT) {
        const int b = i / (LW + 2), c = i % (LW + 2);
        S.u[b][0][c] = 0.f;
        S.u[b][LH + 1][c] = 0.f;
    }
    for (int i = tid; i < 2 * LH; i += NT) {
        const int b = i / LH, rr = i % LH + 1;
        S.u[b][rr][0] = 0.f;
        S.u[b][rr][LW + 1] = 0.f;
    }
    uint32_t lat_act = 0, at_done = 0;
    if (T.has_lat) {
#pragma unroll
        for (int r = 0; r < R; ++r)
            if ((own >> r) & 1u) {
                const int64_t p = (int64_t)(oi + r0 + r) * T.nj + gj;
                if (T.lat_activated[p]) lat_act |= 1u << r;
            }
    }
    fused::cp_async_wait_all();
    __syncthreads();

    Params<float, M::NP> P;
#pragma unroll
    for (int i = 0; i < M::NP; ++i) P.v[i] = T.params[i];
    const float dt = T.dt;
    uint32_t upd = 0;
    if (col > 0 && col < LW - 1) {
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (r0 + r > 0 && r0 + r < LH - 1) upd |= 1u << r;
    }
    upd &= myo_bits;
    const uint32_t any_stim = S.any_stim, at_on = S.at_on, lat_on = S.lat_on;
    const float at_thr = T.at_thr, lat_thr = T.lat_thr;

    for (int s = 0; s < ks; ++s) {
        const int64_t n = n0 + s;
        const int cb = s & 1;
        float(*cur)[LW + 2] = S.u[cb];
        float(*nxt)[LW + 2] = S.u[cb ^ 1];

        if ((any_stim >> s) & 1u) {
            for (int i = 0; i < T.n_stims; ++i) {
                if (!((S.stim_on[i] >> s) & 1u)) continue;
                const BStim &F = stims[i];
                if (gj < F.lo1 || gj >= F.hi1) continue;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (!((myo_bits >> r) & 1u)) continue;
                    const int lr = r0 + r, gi = oi + lr;
                    if (gi < F.lo0 || gi >= F.hi0) continue;
                    if (F.mask && !F.mask[(int64_t)gi * T.nj + gj]) continue;
                    float x = cur[lr + 1][col + 1];
                    if (F.kind == FW_STIM_VOLTAGE) {
                        x = F.value;
                    } else {
                        x = x + F.value;
                        if (F.has_umax && x > F.u_max) x = F.u_max;
                    }
                    cur[lr + 1][col + 1] = x;
                }
            }
            __syncthreads();
        }

        float wl[R + 2], wc[R + 2], wr[R + 2];
#pragma unroll
        for (int i = 0; i < R + 2; ++i) {
            wl[i] = cur[r0 + i][col];
            wc[i] = cur[r0 + i][col + 1];
            wr[i] = cur[r0 + i][col + 2];
        }

        if (own) {
            float mx = wc[1];
#pragma unroll
            for (int r = 1; r < R; ++r) mx = fmaxf(mx, wc[r + 1]);
            // the strip's maximum first (fmaxf skips NaN rows, which never
            // cross): most sub-steps cross nowhere
            if (((at_on >> s) & 1u) && mx > at_thr) {
                // first crossing = smallest step; "never" (-1) is the largest
                // unsigned value (activation_time_2d_tracker.py:61-63)
                const uint32_t hit =
                    fused::rows_gt<R>(wc, at_thr) & own & ~at_done;
                if (hit) {
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        if (!((hit >> r) & 1u)) continue;
                        const int64_t p = (int64_t)(oi + r0 + r) * T.nj + gj;
                        atomicMin(reinterpret_cast<unsigned *>(T.at_act) + p,
                                  (unsigned)n);
                    }
                    at_done |= hit;
                }
            }
            if ((lat_on >> s) & 1u) {
                // cross_threshold (local_activation_time_2d_tracker.py:71-89)
                const uint32_t rise =
                    fused::rows_ge<R>(wc, lat_thr) & own & ~lat_act;
                const uint32_t fall =
                    fused::rows_lt<R>(wc, lat_thr) & own & lat_act;
                lat_act ^= rise | fall;
                if (rise) {
#pragma unroll
                    for (int r = 0; r < R; ++r)
                        if ((rise >> r) & 1u)
                            lat_append(T, (int64_t)(oi + r0 + r) * T.nj + gj, n);
                }
            }
        }

#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float b1 = wc[r + 1];
            const int lr = r0 + r;
            const float4 wa = S.w[0][lr][col];
            const float4 wb = NWO == 8 ? S.w[1][lr][col] : wa;
            const float un = fused::stencil_fma<ST>(wcen[r], b1, wa, wb, wl[r], wc[r],
                                                    wr[r], wl[r + 1], wr[r + 1],
                                                    wl[r + 2], wc[r + 2], wr[r + 2]);
            const float uu = M::template update<float>(b1, un, st[r], P, dt);
            nxt[lr + 1][col + 1] = ((upd >> r) & 1u) ? uu : b1;
        }
        __syncthreads();
    }

    const int fb = ks & 1;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (!((own >> r) & 1u)) continue;
        const int lr = r0 + r;
        const int64_t p = (int64_t)(oi + lr) * T.nj + gj;
        if ((myo_bits >> r) & 1u) {
            const float uo = S.u[fb][lr + 1][col + 1];
            u_out[p] = uo;
            if (!isfinite(uo) && T.status) atomicOr(T.status, FW_DEV_NONFINITE);
            M::template store<float>(T.state, p, st[r]);
        }
        if (T.has_lat) T.lat_activated[p] = (lat_act >> r) & 1u;
    }
}

// Persistent kernel: CTAs take tiles from scratch[0] until the list is
// exhausted; the last CTA to leave (counted in scratch[1]) zeroes both.
__global__ void __launch_bounds__(NT, 2)
    k_batch(const BTissue *__restrict__ tissues, const BTile *__restrict__ tiles,
            int32_t n_tiles, int32_t n_tissues, int64_t offset, int32_t ks,
            int32_t in_buf, uint32_t *scratch)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BSmem &S = *reinterpret_cast<BSmem *>(smem_raw);
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) S.next = (int)atomicAdd(&scratch[0], 1u);
        __syncthreads();
        const int t = S.next;
        if (t >= n_tiles) break;
        const BTile bt = tiles[t];
        if (bt.tissue < 0 || bt.tissue >= n_tissues) {
            // a corrupted plan: report it on the first tissue's status word
            // and skip the tile
            if (tid == 0 && tissues[0].h.status)
                atomicOr(tissues[0].h.status, FW_DEV_BATCH_FAULT);
            __syncthreads();
            continue;
        }
        const BTissue *Tg = tissues + bt.tissue;
        {
            // stage the tissue's head into shared memory
            const uint32_t *src = reinterpret_cast<const uint32_t *>(&Tg->h);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&S.h);
            for (int i = tid; i < (int)(sizeof(BHead) / 4); i += NT)
                dst[i] = src[i];
        }
        __syncthreads();
        const BHead &T = S.h;
        const int64_t n0 = T.step_base + offset;
        // event bits of this launch for the tissue (uniform per CTA)
        if (tid < FW_MAX_STIMS) {
            uint32_t b = 0;
            if (tid < T.n_stims)
                b = window_bits(n0, ks, Tg->stims[tid].first,
                                Tg->stims[tid].last, 1);
            S.stim_on[tid] = b;
        } else if (tid == FW_MAX_STIMS) {
            S.at_on = T.has_at ? window_bits(n0, ks, T.at_win.first,
                                             T.at_win.last, T.at_win.stride)
                               : 0u;
        } else if (tid == FW_MAX_STIMS + 1) {
            S.lat_on = T.has_lat ? window_bits(n0, ks, T.lat_win.first,
                                               T.lat_win.last, T.lat_win.stride)
                                 : 0u;
        }
        __syncthreads();
        if (tid == 0) {
            uint32_t any = 0;
            for (int i = 0; i < FW_MAX_STIMS; ++i) any |= S.stim_on[i];
            S.any_stim = any;
        }
        // S.any_stim is read after the staging barrier inside run_tile
        const int key = T.model * 8 + T.stencil;
        const BStim *stims = Tg->stims;
        switch (key) {
        case FW_MODEL_AP * 8 + FW_STENCIL_ISO5:
            run_tile<ModelAP, FW_STENCIL_ISO5>(stims, bt.tile, n0, ks, in_buf, S);
            break;
        case FW_MODEL_AP * 8 + FW_STENCIL_ANISO9:
            run_tile<ModelAP, FW_STENCIL_ANISO9>(stims, bt.tile, n0, ks, in_buf, S);
            break;
        case FW_MODEL_MS * 8 + FW_STENCIL_ISO5:
            run_tile<ModelMS, FW_STENCIL_ISO5>(stims, bt.tile, n0, ks, in_buf, S);
            break;
        case FW_MODEL_MS * 8 + FW_STENCIL_ANISO9:
            run_tile<ModelMS, FW_STENCIL_ANISO9>(stims, bt.tile, n0, ks, in_buf, S);
            break;
        case FW_MODEL_FK * 8 + FW_STENCIL_ISO5:
            run_tile<ModelFK, FW_STENCIL_ISO5>(stims, bt.tile, n0, ks, in_buf, S);
            break;
        case FW_MODEL_FK * 8 + FW_STENCIL_ANISO9:
            run_tile<ModelFK, FW_STENCIL_ANISO9>(stims, bt.tile, n0, ks, in_buf, S);
            break;
        default:
            // rejected by the plan; reached only through a corrupted one
            if (tid == 0 && T.status) atomicOr(T.status, FW_DEV_BATCH_FAULT);
            break;
        }
        __syncthreads();
    }
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&scratch[1], 1u) == gridDim.x - 1) {
            atomicExch(&scratch[0], 0u);
            atomicExch(&scratch[1], 0u);
        }
    }
}

constexpr size_t kSmem = sizeof(BSmem);

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

int check_tissue(const fw_step_args *a, int i)
{
    if (!a) {
        set_error("fw_batch: tissue %d is NULL", i);
        return FW_ERR_ARG;
    }
    if (a->model != FW_MODEL_AP && a->model != FW_MODEL_MS &&
        a->model != FW_MODEL_FK) {
        set_error("fw_batch: tissue %d: model %d has no batched form", i,
                  a->model);
        return FW_ERR_UNSUPPORTED;
    }
    if (a->precision != FW_F32) {
        set_error("fw_batch: tissue %d: float32 only", i);
        return FW_ERR_UNSUPPORTED;
    }
    if (a->stencil != FW_STENCIL_ISO5 && a->stencil != FW_STENCIL_ANISO9) {
        set_error("fw_batch: tissue %d: 2D stencils only", i);
        return FW_ERR_UNSUPPORTED;
    }
    if (a->nk != 1 || a->ni < 3 || a->nj < 3 || a->ni > (1 << 30) ||
        a->nj > (1 << 30)) {
        set_error("fw_batch: tissue %d: bad 2D grid (%lld, %lld, %lld)", i,
                  (long long)a->ni, (long long)a->nj, (long long)a->nk);
        return FW_ERR_ARG;
    }
    if (a->n_at > 1 || a->n_lat > 1 || a->n_probe != 0 || a->n_ecg != 0 ||
        a->n_tip != 0) {
        set_error("fw_batch: tissue %d: at most one activation and one local "
                  "activation tracker, no probes or ECG", i);
        return FW_ERR_UNSUPPORTED;
    }
    if (a->n_stims < 0 || a->n_stims > FW_MAX_STIMS) {
        set_error("fw_batch: tissue %d: n_stims out of range", i);
        return FW_ERR_ARG;
    }
    if (!a->weights || !a->myo || !a->u[0] || !a->u[1]) {
        set_error("fw_batch: tissue %d: null weights, myo or u", i);
        return FW_ERR_ARG;
    }
    int ns = 0, np = 0;
    fw_model_info(a->model, &ns, &np);
    for (int s = 0; s < ns; ++s)
        if (!a->state[s]) {
            set_error("fw_batch: tissue %d: state %d is NULL", i, s);
            return FW_ERR_ARG;
        }
    for (int k = 0; k < a->n_at; ++k)
        if (a->at[k].win.stride <= 0 || !a->at[k].act_step) {
            set_error("fw_batch: tissue %d: bad activation tracker", i);
            return FW_ERR_ARG;
        }
    for (int k = 0; k < a->n_lat; ++k)
        if (a->lat[k].win.stride <= 0 || !a->lat[k].activated ||
            !a->lat[k].cross_steps || !a->lat[k].cross_count) {
            set_error("fw_batch: tissue %d: bad local activation tracker", i);
            return FW_ERR_ARG;
        }
    return FW_OK;
}

int64_t tissue_tiles(const fw_step_args *a)
{
    return ((a->ni + TI - 1) / TI) * ((a->nj + TJ - 1) / TJ);
}

}  // namespace batch

int batch_plan_size(const fw_step_args *const *tissues, int32_t n,
                    int64_t *bytes)
{
    using namespace batch;
    if (!tissues || n <= 0 || !bytes) {
        set_error("fw_batch_plan_size: no tissues or NULL output");
        return FW_ERR_ARG;
    }
    int64_t n_tiles = 0;
    for (int i = 0; i < n; ++i) {
        int rc = check_tissue(tissues[i], i);
        if (rc) return rc;
        n_tiles += tissue_tiles(tissues[i]);
    }
    if (n_tiles > INT32_MAX) {
        set_error("fw_batch_plan_size: too many tiles");
        return FW_ERR_ARG;
    }
    *bytes = (int64_t)(align_up(sizeof(BTissue) * n, 256) +
                       sizeof(BTile) * (size_t)n_tiles);
    return FW_OK;
}

int batch_plan(const fw_step_args *const *tissues, int32_t n,
               const int64_t *n_begin, void *plan, int64_t plan_bytes,
               fw_batch *out, cudaStream_t stream)
{
    using namespace batch;
    int64_t need = 0;
    int rc = batch_plan_size(tissues, n, &need);
    if (rc) return rc;
    if (!n_begin || !plan || !out) {
        set_error("fw_batch_plan: NULL n_begin, plan or out");
        return FW_ERR_ARG;
    }
    if (plan_bytes < need) {
        set_error("fw_batch_plan: plan buffer of %lld bytes, %lld needed",
                  (long long)plan_bytes, (long long)need);
        return FW_ERR_ARG;
    }
    if (((uintptr_t)plan & 15) != 0) {
        set_error("fw_batch_plan: plan must be 16-byte aligned");
        return FW_ERR_ARG;
    }
    std::vector<unsigned char> host((size_t)need, 0);
    BTissue *desc = reinterpret_cast<BTissue *>(host.data());
    BTile *tl = reinterpret_cast<BTile *>(
        host.data() + align_up(sizeof(BTissue) * n, 256));
    int32_t t_count = 0;
    for (int i = 0; i < n; ++i) {
        const fw_step_args *a = tissues[i];
        BHead &T = desc[i].h;
        T.w = (const float *)a->weights;
        T.myo = a->myo;
        T.u[0] = (float *)a->u[0];
        T.u[1] = (float *)a->u[1];
        int ns = 0, np = 0;
        fw_model_info(a->model, &ns, &np);
        for (int s = 0; s < kMaxState; ++s) T.state[s] = s < ns ? a->state[s] : nullptr;
        for (int p = 0; p < kMaxParams; ++p) T.params[p] = p < np ? (float)a->params[p] : 0.f;
        T.dt = (float)a->dt;
        T.model = a->model;
        T.stencil = a->stencil;
        T.ni = (int32_t)a->ni;
        T.nj = (int32_t)a->nj;
        T.tiles_j = (int32_t)((a->nj + TJ - 1) / TJ);
        T.n = a->ni * a->nj;
        T.step_base = n_begin[i];
        T.n_stims = a->n_stims;
        for (int s = 0; s < a->n_stims; ++s) {
            const fw_stim &S = a->stims[s];
            BStim &B = desc[i].stims[s];
            B.first = S.first;
            B.last = S.last;
            B.kind = S.kind;
            B.has_umax = S.has_umax;
            B.value = (float)S.value;
            B.u_max = (float)S.u_max;
            B.lo0 = (int32_t)(S.lo[0] < 0 ? 0 : S.lo[0]);
            B.hi0 = (int32_t)(S.hi[0] > a->ni ? a->ni : S.hi[0]);
            B.lo1 = (int32_t)(S.lo[1] < 0 ? 0 : S.lo[1]);
            B.hi1 = (int32_t)(S.hi[1] > a->nj ? a->nj : S.hi[1]);
            B.mask = S.mask;
        }
        T.has_at = a->n_at;
        if (a->n_at) {
            T.at_win = BWin{a->at[0].win.first, a->at[0].win.last,
                            a->at[0].win.stride};
            T.at_thr = (float)a->at[0].threshold;
            T.at_act = a->at[0].act_step;
        }
        T.has_lat = a->n_lat;
        if (a->n_lat) {
            const fw_lat_tracker &L = a->lat[0];
            T.lat_win = BWin{L.win.first, L.win.last, L.win.stride};
            T.lat_thr = (float)L.threshold;
            T.lat_cap = L.capacity;
            T.lat_activated = L.activated;
            T.lat_steps = L.cross_steps;
            T.lat_count = L.cross_count;
        }
        T.status = a->status;
    }
    // tile list grouped by (model, stencil): CTAs taking consecutive tiles
    // then run the same specialisation of the tile code (one of six inlined
    // copies) instead of switching between them from tile to tile
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        const int kx = tissues[x]->model * 8 + tissues[x]->stencil;
        const int ky = tissues[y]->model * 8 + tissues[y]->stencil;
        return kx < ky;
    });
    for (int i : order) {
        const int32_t nt = (int32_t)tissue_tiles(tissues[i]);
        for (int32_t k = 0; k < nt; ++k) tl[t_count + k] = BTile{i, k};
        t_count += nt;
    }
    FW_CUDA_CHECK(cudaMemcpyAsync(plan, host.data(), (size_t)need,
                                  cudaMemcpyHostToDevice, stream));
    // the host staging buffer is released on return
    FW_CUDA_CHECK(cudaStreamSynchronize(stream));

    int dev = 0, sms = 0, per_sm = 0;
    FW_CUDA_CHECK(cudaGetDevice(&dev));
    FW_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    FW_CUDA_CHECK(cudaFuncSetAttribute(
        k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem));
    FW_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, k_batch, NT, kSmem));
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)sms * per_sm;
    if (grid > t_count) grid = t_count;
    out->plan = plan;
    out->n_tissues = n;
    out->n_tiles = t_count;
    out->ksteps = KMAX;
    out->grid = (int32_t)grid;
    return FW_OK;
}

int batch_run(const fw_batch *b, uint32_t *scratch, int64_t offset,
              int64_t n_steps, cudaStream_t stream)
{
    using namespace batch;
    if (!b || !b->plan || !scratch || b->n_tissues <= 0 || b->grid <= 0) {
        set_error("fw_batch_run: empty plan or NULL scratch");
        return FW_ERR_ARG;
    }
    if (offset < 0 || n_steps < 0) {
        set_error("fw_batch_run: negative offset or step count");
        return FW_ERR_ARG;
    }
    if (n_steps == 0) return FW_OK;
    // the plan set the shared-memory attribute on this device; set it again
    // unless the stream is being captured into a CUDA graph (the launches
    // alone are recorded then)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    FW_CUDA_CHECK(cudaStreamIsCapturing(stream, &cap));
    if (cap == cudaStreamCaptureStatusNone)
        FW_CUDA_CHECK(cudaFuncSetAttribute(
            k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem));
    const BTissue *desc = reinterpret_cast<const BTissue *>(b->plan);
    const BTile *tl = reinterpret_cast<const BTile *>(
        (const unsigned char *)b->plan + align_up(sizeof(BTissue) * b->n_tissues, 256));
    // L launches of <= KMAX steps with L == n_steps (mod 2): the result ends
    // in u[(offset + n_steps) & 1], as after the same steps of the plain form
    int64_t L = (n_steps + KMAX - 1) / KMAX;
    if ((L & 1) != (n_steps & 1)) ++L;
    int64_t done = 0;
    for (int64_t li = 0; li < L; ++li) {
        const int64_t left = n_steps - done, launches_left = L - li;
        int64_t ks = (left + launches_left - 1) / launches_left;
        if (ks > KMAX) ks = KMAX;
        const int in_buf = (int)((offset + li) & 1);
        k_batch<<<b->grid, NT, kSmem, stream>>>(desc, tl, b->n_tiles,
                                               b->n_tissues, offset + done,
                                               (int32_t)ks, in_buf, scratch);
        FW_CHECK_LAUNCH("k_batch");
        done += ks;
    }
    return FW_OK;
}

// ---- fw_batch_run_noalloc ----------------------------------------------------
// The same launches as batch_run with the tile counters in the library's own
// device memory: a file-scope array, one per device, so the call takes no
// scratch buffer from its caller.  Only the counters live here (the plan
// stays in the caller's buffer); they must start at zero, which the set-up
// below ensures, and every launch leaves them at zero.  All calls on a device
// share this one array, so calls whose launches overlap in time (other
// streams, other host threads) race on it and must be ordered by the caller.

namespace {

constexpr int kNoallocScratchBytes = 256;  // the stated maximum
constexpr int kNoallocMaxDevices = 64;

static __device__ __align__(256) uint32_t
    g_noalloc_scratch[kNoallocScratchBytes / sizeof(uint32_t)];

std::mutex g_noalloc_mu;
uint32_t *g_noalloc_ptr[kNoallocMaxDevices];  // device address, per device

}  // namespace

// The batch's scratch (the tile counters) has a fixed size, so the limit is
// checked when the library is compiled: a batch kernel needing more than the
// fixed array holds does not build.
static_assert(kBatchScratchBytes <= kNoallocScratchBytes,
              "fw_batch_run_noalloc: the batch scratch exceeds the fixed array");

int batch_run_noalloc(const fw_batch *b, int64_t offset, int64_t n_steps,
                      cudaStream_t stream)
{
    // the argument checks of batch_run, before the one-time set-up
    if (!b || !b->plan || b->n_tissues <= 0 || b->grid <= 0) {
        set_error("fw_batch_run_noalloc: empty plan");
        return FW_ERR_ARG;
    }
    if (offset < 0 || n_steps < 0) {
        set_error("fw_batch_run_noalloc: negative offset or step count");
        return FW_ERR_ARG;
    }
    int dev = 0;
    FW_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoallocMaxDevices) {
        set_error("fw_batch_run_noalloc: device %d beyond the %d supported",
                  dev, kNoallocMaxDevices);
        return FW_ERR_ARG;
    }
    uint32_t *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        scratch = g_noalloc_ptr[dev];
        if (!scratch) {
            // set-up, once per device, with that device current: the
            // address of this device's copy of the array, then zero it
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess)
                return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
            e = cudaMemsetAsync(p, 0, kNoallocScratchBytes, stream);
            if (e != cudaSuccess)
                return cuda_error(e, "cudaMemsetAsync(g_noalloc_scratch)");
            scratch = static_cast<uint32_t *>(p);
            g_noalloc_ptr[dev] = scratch;
        }
    }
    return batch_run(b, scratch, offset, n_steps, stream);
}

}  // namespace fw
