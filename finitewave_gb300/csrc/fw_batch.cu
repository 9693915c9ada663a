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

#include "fw_fused_tma.cuh"

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
    void *state[2][kMaxState];   // both state buffers (read [in], write [in ^ 1])
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
        st[r] = M::template load<float>(T.state[in_buf], p);
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
            const float uu = fused::fused_update<M>(b1, un, st[r], P, dt);
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
            M::template store<float>(T.state[in_buf ^ 1], p, st[r]);
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
        if (!a->state[s] || !a->state_b[s] || a->state[s] == a->state_b[s]) {
            set_error("fw_batch: tissue %d: state %d or its second buffer "
                      "(state_b) is NULL or aliased", i, s);
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

// ---- the TMA form of the batch (kernel 2) ------------------------------------
//
// The single-tissue TMA pipeline (fw_fused_tma.cuh) over the ragged tile
// list: one persistent 512-thread CTA per SM, two shared-memory stages, the
// tile computed by the fused kernels' tile code (tma_tile), so a tissue
// advanced here is bitwise the same as when run alone by k_fused_tma.
// Everything a tile needs arrives asynchronously: for the tile after the
// current one, one bulk copy of its tissue's launch description (a FusedK
// kept in the plan, whose per-launch fields k_batch_events fills before
// each launch) and the TMA copies of its region through the tissue's own
// tensor maps (also in the plan), all completing on the stage's mbarrier,
// issued right after the wait for the current tile's stage (by one lane
// each of warps 0, 1 and 2 in the strip kernel, batch_issue_split).
// Thread 0 claims runs of consecutive tiles from the counter one run ahead
// and reads each list entry one tile ahead, so none of its loads is waited
// for on the way.  Tissues need rows of a multiple of 16 nodes, which the
// caller provides as a row pitch (fw_step_args.pitch) on copies of the
// TMA-read arrays.

constexpr int kTmaR = 4;                           // rows per thread
constexpr int kRun = 4;                            // tiles per counter claim
constexpr int kTmaNT = fused::kTW * (LH / kTmaR);  // 512 threads

struct alignas(128) BTissueT {
    fused::TmaMaps maps;   // 64-byte aligned tensor maps of this tissue
    fused::FusedK f;       // launch description (static part from the plan)
    BWin stim_win[FW_MAX_STIMS];
    BWin at_win[fused::kMaxFusedAt];
    BWin lat_win[fused::kMaxFusedLat];
    float *u[2];
    void *state[2][FW_MAX_FUSED_STATE];
    int64_t step_base;
};

// One entry of the TMA form's tile list.
struct BTileT {
    int32_t tissue;
    int32_t key;           // model * 8 + stencil, | kTileLat
    int32_t oi, oj;        // region origin
};
// BTileT.key: the tissue has a local activation tracker, whose flags are
// staged with the region
constexpr int32_t kTileLat = 1 << 8;

constexpr int kAcq = 64;   // entries of the table of acquired tissues

template <int NS, int NWO>
struct BatchTmaSmem {
    fused::TmaSmem<LH, NS, NWO> t;
    fused::FusedK f[2];    // launch description of each stage's tile
    int ftissue[2];        // the tissue whose description f[] holds (-1: none)
    int tile[2];           // the stage's tile index (>= the group's end: none)
    int oi[2], oj[2];      // its region origin
    int ok[2];             // 0 for a skipped tile
    // tissues whose tensor maps thread 0 has acquired in this launch: a
    // direct-mapped table (tissue % kAcq -> tissue, -1: none); the maps do
    // not change during a launch, so one acquire per tissue and CTA suffices
    int acq[kAcq];
    // the split issue of the loop (batch_issue_split): the next tile and its
    // list entry, published by thread 0 before the stage wait, and the
    // tables of tissues acquired by each of the three issuing lanes
    int nt;
    BTileT nbt;
    int acq3[3][kAcq];
};

// The batch's (model, stencil) groups, in the order the plan sorts tiles;
// each group is advanced by its own instantiation of k_batch_tma.
constexpr int kGroups = 6;
constexpr int kGroupKey[kGroups] = {
    FW_MODEL_AP * 8 + FW_STENCIL_ISO5, FW_MODEL_AP * 8 + FW_STENCIL_ANISO9,
    FW_MODEL_MS * 8 + FW_STENCIL_ISO5, FW_MODEL_MS * 8 + FW_STENCIL_ANISO9,
    FW_MODEL_FK * 8 + FW_STENCIL_ISO5, FW_MODEL_FK * 8 + FW_STENCIL_ANISO9};

// The per-launch fields of every tissue's launch description: step window
// masks of the stimuli and trackers, first step, step count and the
// potential buffers.  One warp per tissue.
__global__ void k_batch_events(BTissueT *__restrict__ tissues, int32_t n,
                               int64_t koff, int32_t ks, int32_t in_buf)
{
    const int i = blockIdx.x * blockDim.y + threadIdx.y;
    if (i >= n) return;
    BTissueT &T = tissues[i];
    fused::FusedK &F = T.f;
    const int lane = threadIdx.x;
    const int64_t n0 = T.step_base + koff;
    if (lane < F.n_stims)
        F.stims[lane].on =
            window_bits(n0, ks, T.stim_win[lane].first, T.stim_win[lane].last, 1);
    if (lane >= 16 && lane - 16 < F.n_at) {
        const BWin &w = T.at_win[lane - 16];
        F.at[lane - 16].on = window_bits(n0, ks, w.first, w.last, w.stride);
    }
    if (lane >= 24 && lane - 24 < F.n_lat) {
        const BWin &w = T.lat_win[lane - 24];
        F.lat[lane - 24].on = window_bits(n0, ks, w.first, w.last, w.stride);
    }
    __syncwarp();
    if (lane == 0) {
        uint32_t any = 0;
        for (int s = 0; s < F.n_stims; ++s) any |= F.stims[s].on;
        F.stim_on = any;
        F.n0 = n0;
        F.ksteps = ks;
        F.u_in = T.u[in_buf];
        F.u_out = T.u[in_buf ^ 1];
        for (int q = 0; q < FW_MAX_FUSED_STATE; ++q) {
            F.state[q] = T.state[in_buf][q];
            F.state_out[q] = T.state[in_buf ^ 1][q];
        }
    }
}

__device__ __forceinline__ void tensormap_acquire(const void *map)
{
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy(void *dst, const void *src, unsigned bytes,
                                          uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1], %2, [%3];\n" ::"r"(fused::smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(fused::smem_u32(bar))
        : "memory");
}

// Thread 0: stage tile t (list entry bt) into stage sg.  The tensor maps
// of a tissue are acquired the first time the CTA meets the tissue in the
// launch (S.acq; a table collision only repeats an acquire).
// PAIR: the column-pair kernel, whose weight map is the column-pair view.
template <class M, int ST, bool PAIR, class Sm>
__device__ __noinline__ void batch_issue(const BTissueT *__restrict__ tissues,
                                         int32_t t_end, int32_t n_tissues,
                                         int32_t in_buf, Sm &S, int sg, int t,
                                         BTileT bt)
{
    constexpr int NWO = fused::Stencil2D<ST>::NWO;
    S.tile[sg] = t;
    if (t >= t_end) return;
    uint64_t *bar = &S.t.bar[sg];
    fused::fence_proxy_async();
    if (bt.tissue < 0 || bt.tissue >= n_tissues) {
        // a corrupted plan: flag it and complete the stage's phase without
        // data, so that the tile is skipped
        S.ok[sg] = 0;
        if (tissues[0].f.status) atomicOr(tissues[0].f.status, FW_DEV_BATCH_FAULT);
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(
                         fused::smem_u32(bar))
                     : "memory");
        return;
    }
    const BTissueT &T = tissues[bt.tissue];
    S.ok[sg] = 1;
    S.oi[sg] = bt.oi;
    S.oj[sg] = bt.oj;
    const fused::TmaMaps &Mp = T.maps;
    const bool lat = (bt.key & kTileLat) != 0;
    int &acquired = S.acq[bt.tissue & (kAcq - 1)];
    if (bt.tissue != acquired) {
        tensormap_acquire(&Mp.w);
        tensormap_acquire(&Mp.myo);
        tensormap_acquire(&Mp.u[in_buf]);
        tensormap_acquire(&Mp.wc);
#pragma unroll
        for (int q = 0; q < M::NS; ++q) tensormap_acquire(&Mp.s[in_buf][q]);
        if (lat) tensormap_acquire(&Mp.act);
        acquired = bt.tissue;
    }
    // one arrive on the stage's barrier announces the region's bytes and
    // the launch description's, which rides on the same barrier; a stage
    // whose last tile was of the same tissue holds it already (tiles come
    // in runs of one tissue, and a description does not change within a
    // launch)
    constexpr unsigned kF = (unsigned)sizeof(fused::FusedK);
    const bool fresh = S.ftissue[sg] != bt.tissue;
    fused::issue_region<KMAX, M::NS, NWO, PAIR>(Mp, in_buf, S.t.stage[sg], bar,
                                                bt.oi, bt.oj, fresh ? kF : 0u, lat);
    if (fresh) {
        bulk_copy(&S.f[sg], &T.f, kF, bar);
        S.ftissue[sg] = bt.tissue;
    }
}

// The loop's per-tile issue of the strip kernel, spread over one lane of
// each of warps 0, 1 and 2 (tid 0, 32, 64) so that no warp carries all of
// it into the tile's first sub-step: the next tile (S.nt) and its list
// entry (S.nbt) were published by thread 0 before the stage wait; tid 0
// records the tile, announces the stage's bytes (the barrier's one
// arrival) and copies the weights and, when the stage's last tile was of
// another tissue, the launch description; tid 32 copies the potential and
// the state, tid 64 the myocyte flags, the centre weights and the local
// activation flags.  Each lane acquires the tensor maps it uses, once per
// tissue and launch (its own table).  Copies may complete before the
// announcement: the phase cannot end before the arrival.
template <class M, int ST, class Sm>
__device__ __noinline__ void batch_issue_split(const BTissueT *__restrict__ tissues,
                                               int32_t t_end, int32_t n_tissues,
                                               int32_t in_buf, Sm &S, int sg, int tid)
{
    constexpr int NWO = fused::Stencil2D<ST>::NWO;
    constexpr int NS = M::NS;
    const int part = tid >> 5;
    const int t = S.nt;
    const BTileT bt = S.nbt;
    if (part == 0) S.tile[sg] = t;
    if (t >= t_end) return;
    uint64_t *bar = &S.t.bar[sg];
    fused::fence_proxy_async();
    if (bt.tissue < 0 || bt.tissue >= n_tissues) {
        // a corrupted plan: flag it and complete the stage's phase without
        // data, so that the tile is skipped
        if (part == 0) {
            S.ok[sg] = 0;
            if (tissues[0].f.status) atomicOr(tissues[0].f.status, FW_DEV_BATCH_FAULT);
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(
                             fused::smem_u32(bar))
                         : "memory");
        }
        return;
    }
    const BTissueT &T = tissues[bt.tissue];
    const fused::TmaMaps &Mp = T.maps;
    const bool lat = (bt.key & kTileLat) != 0;
    int &acquired = S.acq3[part][bt.tissue & (kAcq - 1)];
    const bool acq = bt.tissue != acquired;
    if (acq) acquired = bt.tissue;
    auto &G = S.t.stage[sg];
    const int x4 = fused::floor_to(bt.oj - 1, 4), x16 = fused::floor_to(bt.oj, 16);
    if (part == 0) {
        S.ok[sg] = 1;
        S.oi[sg] = bt.oi;
        S.oj[sg] = bt.oj;
        if (acq) tensormap_acquire(&Mp.w);
        constexpr unsigned kF = (unsigned)sizeof(fused::FusedK);
        const bool fresh = S.ftissue[sg] != bt.tissue;
        const unsigned bytes =
            (unsigned)(sizeof(G.wa) * (NWO == 8 ? 2 : 1) + sizeof(G.u) +
                       NS * sizeof(G.s[0]) + sizeof(G.myo) + sizeof(G.wc)) +
            (lat ? (unsigned)sizeof(G.act) : 0u) + (fresh ? kF : 0u);
        fused::mbar_expect_tx(bar, bytes);
        fused::tma_3d(&G.wa[0][0], &Mp.w, 0, bt.oj, bt.oi, bar);
        if constexpr (NWO == 8) fused::tma_3d(&G.wb[0][0], &Mp.w, 4, bt.oj, bt.oi, bar);
        if (fresh) {
            bulk_copy(&S.f[sg], &T.f, kF, bar);
            S.ftissue[sg] = bt.tissue;
        }
    } else if (part == 1) {
        if (acq) {
            tensormap_acquire(&Mp.u[in_buf]);
#pragma unroll
            for (int q = 0; q < NS; ++q) tensormap_acquire(&Mp.s[in_buf][q]);
        }
        fused::tma_2d(&G.u[0][0], &Mp.u[in_buf], x4, bt.oi - 1, bar);
#pragma unroll
        for (int q = 0; q < NS; ++q)
            fused::tma_2d(&G.s[q][0][0], &Mp.s[in_buf][q], x4, bt.oi, bar);
    } else {
        if (acq) {
            tensormap_acquire(&Mp.myo);
            tensormap_acquire(&Mp.wc);
            if (lat) tensormap_acquire(&Mp.act);
        }
        fused::tma_2d(&G.myo[0][0], &Mp.myo, x16, bt.oi, bar);
        fused::tma_2d(&G.wc[0][0], &Mp.wc, x4, bt.oi, bar);
        if (lat) fused::tma_2d(&G.act[0][0], &Mp.act, x16, bt.oi, bar);
    }
}

// One (model, stencil) group of the batch: tiles [t_begin, t_end) of the
// list, claimed kRun at a time from counters[0] (counters[1] counts the
// CTAs that are done; the last one zeroes both).  PAIR (kernel 3): the tile
// code of the column-pair kernels in two-wide float32 instructions
// (tma_tile2), 2 x 2 nodes per thread, the same bits as the strip tiles.
template <class M, int ST, bool PAIR>
__global__ void __launch_bounds__(kTmaNT, 1)
    k_batch_tma(const BTissueT *__restrict__ tissues, const BTileT *__restrict__ tiles,
                int32_t t_begin, int32_t t_end, int32_t n_tissues, int32_t in_buf,
                uint32_t *counters)
{
    using Sm = BatchTmaSmem<M::NS, fused::Stencil2D<ST>::NWO>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned mis = fused::smem_u32(smem_raw) & 127u;
    Sm &S = *reinterpret_cast<Sm *>(smem_raw + (mis ? 128u - mis : 0u));
    const int tid = threadIdx.x;
    // the next group's kernel, launched with programmatic serialisation,
    // may place its CTAs on the SMs this grid's CTAs leave (its tissues are
    // not this group's, so nothing it reads is written here)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    uint32_t own_c, ring_c;
    if constexpr (PAIR)
        fused::pair_masks<KMAX, LH>(2 * (tid % (fused::kTW / 2)),
                                    (tid / (fused::kTW / 2)) * 2, own_c, ring_c);
    else
        fused::strip_masks<KMAX, LH, kTmaR>(tid % fused::kTW,
                                            (tid / fused::kTW) * kTmaR, own_c, ring_c);
    const BTileT none{-1, -1, 0, 0};
    // thread 0's tiles: runs of kRun consecutive list entries (mostly of
    // one tissue), each
    // run's start taken from counters[0] one run ahead; the list entry of
    // tile i + 1 is read while tile i is computed
    int run_cur = t_end, run_end = t_end, run_next = t_end;
    auto take_run = [&]() -> int {
        const int64_t s =
            (int64_t)t_begin + (int64_t)atomicAdd(&counters[0], 1u) * kRun;
        return s < t_end ? (int)s : t_end;
    };
    auto next_tile = [&]() -> int {
        if (run_cur >= run_end) {
            if (run_next >= t_end) return t_end;
            run_cur = run_next;
            run_end = run_next + kRun < t_end ? run_next + kRun : t_end;
            run_next = take_run();
        }
        return run_cur++;
    };
    int t_next = t_end;
    BTileT b_next = none;
    if (tid == 0) {
        fused::mbar_init(&S.t.bar[0], 1);
        fused::mbar_init(&S.t.bar[1], 1);
        fused::mbar_fence_init();
        S.ftissue[0] = S.ftissue[1] = -1;
        for (int i = 0; i < kAcq; ++i) S.acq[i] = -1;
        for (int i = 0; i < 3 * kAcq; ++i) S.acq3[i / kAcq][i % kAcq] = -1;
        run_next = take_run();
        const int t0 = next_tile();
        t_next = next_tile();
        batch_issue<M, ST, PAIR>(tissues, t_end, n_tissues, in_buf, S, 0, t0,
                           t0 < t_end ? tiles[t0] : none);
        if (t_next < t_end) b_next = tiles[t_next];
    }
    __syncthreads();
    unsigned parity = 0u;
    for (int it = 0;; ++it) {
        const int sg = it & 1;
        if (S.tile[sg] >= t_end) break;
        if (!PAIR && tid == 0) {
            // the next tile, for the three issuing lanes after the wait
            S.nt = t_next;
            S.nbt = b_next;
        }
        const unsigned ph = (parity >> sg) & 1u;
        const bool arrived = fused::mbar_wait(&S.t.bar[sg], ph);
        parity ^= 1u << sg;
        if (__syncthreads_or(!arrived)) {
            if (tid == 0) {
                // flag it, then wait (bounded) for the copy in flight (the
                // other stage's next tile is issued after this point)
                if (tissues[0].f.status) atomicOr(tissues[0].f.status, FW_DEV_TIMEOUT);
                if (!arrived) fused::mbar_wait(&S.t.bar[sg], ph);
            }
            break;
        }
        // the next tile into the other stage, whose readers finished before
        // the wait above ended; issued here, after the wait, so that the
        // other warps start this tile meanwhile
        if constexpr (PAIR) {
            if (tid == 0)
                batch_issue<M, ST, PAIR>(tissues, t_end, n_tissues, in_buf, S, sg ^ 1,
                                         t_next, b_next);
        } else {
            if (tid == 0 || tid == 32 || tid == 64)
                batch_issue_split<M, ST>(tissues, t_end, n_tissues, in_buf, S, sg ^ 1,
                                         tid);
        }
        if (tid == 0) {
            t_next = next_tile();
            b_next = t_next < t_end ? tiles[t_next] : none;
        }
        if (S.ok[sg]) {
            const fused::FusedK &f = S.f[sg];
            Params<float, M::NP> P;
#pragma unroll
            for (int i = 0; i < M::NP; ++i) P.v[i] = f.params[i];
            if constexpr (PAIR)
                fused::tma_tile2<M, ST, KMAX, LH, true>(f, S.t.stage[sg], S.t, S.oi[sg],
                                                        S.oj[sg], own_c, ring_c, P);
            else
                fused::tma_tile<M, ST, KMAX, LH, kTmaR>(f, S.t.stage[sg], S.t,
                                                       S.oi[sg], S.oj[sg], own_c,
                                                       ring_c, P);
        } else {
            // a skipped tile has no sub-step barrier to publish thread 0's
            // record of the next tile
            __syncthreads();
        }
        // no barrier here otherwise: the tile's sub-step barriers publish
        // that record, and the next iteration's wait ends in one before any
        // thread touches the ping-pong rows or this stage is refilled
    }
    if (tid == 0) {
        // this grid completes only after the group's kernel launched before
        // it (a no-op without programmatic serialisation), so the stream's
        // next ordinary launch finds every group of the launch finished
        asm volatile("griddepcontrol.wait;" ::: "memory");
        __threadfence();
        if (atomicAdd(&counters[1], 1u) == gridDim.x - 1) {
            atomicExch(&counters[0], 0u);
            atomicExch(&counters[1], 0u);
        }
    }
}

template <class M, int ST>
constexpr size_t tma_smem()
{
    return sizeof(BatchTmaSmem<M::NS, fused::Stencil2D<ST>::NWO>) + 128;
}
static_assert(tma_smem<ModelFK, FW_STENCIL_ANISO9>() <= 232448,
              "the batched TMA stages exceed 227 KB");

using BatchTmaKernel = void (*)(const BTissueT *, const BTileT *, int32_t, int32_t,
                                int32_t, int32_t, uint32_t *);

inline int batch_group_launch_k(BatchTmaKernel kern, size_t smem, bool attr_only,
                                cudaLaunchConfig_t &cfg, const BTissueT *desc,
                                const BTileT *tl, int32_t t_begin, int32_t t_end,
                                int32_t n_tissues, int32_t in_buf, uint32_t *counters)
{
    if (attr_only) {
        FW_CUDA_CHECK(cudaFuncSetAttribute(
            kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return FW_OK;
    }
    cfg.dynamicSmemBytes = smem;
    FW_CUDA_CHECK(cudaLaunchKernelEx(&cfg, kern, desc, tl, t_begin, t_end, n_tissues,
                                     in_buf, counters));
    FW_CHECK_LAUNCH("k_batch_tma");
    return FW_OK;
}

// Launch group g's kernel (or set its shared-memory attribute when
// `attr_only`); `pair`: the column-pair form (kernel 3).  `overlap`:
// launched with programmatic stream serialisation, so that its CTAs start
// as the previous group's CTAs finish instead of after the whole previous
// grid (the groups' tissues are disjoint).
inline int batch_group_launch(int g, bool pair, bool attr_only, bool overlap, int grid,
                              const BTissueT *desc, const BTileT *tl, int32_t t_begin,
                              int32_t t_end, int32_t n_tissues, int32_t in_buf,
                              uint32_t *counters, cudaStream_t stream)
{
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = overlap ? 1 : 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kTmaNT);
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
#define FW_BATCH_GROUP(GI, M, ST)                                                 \
    case GI:                                                                      \
        if (pair)                                                                 \
            return batch_group_launch_k(k_batch_tma<M, ST, true>,                 \
                                        tma_smem<M, ST>(), attr_only, cfg, desc,  \
                                        tl, t_begin, t_end, n_tissues, in_buf,    \
                                        counters);                                \
        return batch_group_launch_k(k_batch_tma<M, ST, false>, tma_smem<M, ST>(), \
                                    attr_only, cfg, desc, tl, t_begin, t_end,     \
                                    n_tissues, in_buf, counters);
    switch (g) {
        FW_BATCH_GROUP(0, ModelAP, FW_STENCIL_ISO5)
        FW_BATCH_GROUP(1, ModelAP, FW_STENCIL_ANISO9)
        FW_BATCH_GROUP(2, ModelMS, FW_STENCIL_ISO5)
        FW_BATCH_GROUP(3, ModelMS, FW_STENCIL_ANISO9)
        FW_BATCH_GROUP(4, ModelFK, FW_STENCIL_ISO5)
        FW_BATCH_GROUP(5, ModelFK, FW_STENCIL_ANISO9)
    }
#undef FW_BATCH_GROUP
    set_error("fw_batch: no group %d", g);
    return FW_ERR_ARG;
}

static_assert(sizeof(fused::FusedK) % 16 == 0 && offsetof(BTissueT, f) % 16 == 0,
              "the launch description moves as one bulk copy");

inline bool aligned16(const void *p) { return p && ((uintptr_t)p & 15) == 0; }

// The TMA form can take this tissue: rows (the pitch) a multiple of 16
// nodes, every TMA-read array (the local activation flags included)
// 16-byte aligned, packed weights.
bool tma_tissue_ok(const fw_step_args *a)
{
    const int64_t pitch = a->pitch ? a->pitch : a->nj;
    if (pitch < a->nj || pitch % 16 || pitch >= (1 << 30)) return false;
    if (!aligned16(a->weights_packed) || !aligned16(a->weights) ||
        !aligned16(a->u[0]) || !aligned16(a->u[1]) || !aligned16(a->myo))
        return false;
    int ns = 0, np = 0;
    fw_model_info(a->model, &ns, &np);
    for (int q = 0; q < ns; ++q)
        if (!aligned16(a->state[q]) || !aligned16(a->state_b[q])) return false;
    for (int l = 0; l < a->n_lat; ++l)
        if (!aligned16(a->lat[l].activated)) return false;
    return fused::tensor_map_encoder() != nullptr;
}

// Fill one tissue's descriptor of the TMA form.
int fill_tma_tissue(const fw_step_args *a, int64_t n_begin, BTissueT &T, bool pair)
{
    using namespace fused;
    const int64_t pitch = a->pitch ? a->pitch : a->nj;
    const int nwo = a->stencil == FW_STENCIL_ISO5 ? 4 : 8;
    const int cen = a->stencil == FW_STENCIL_ISO5 ? 2 : 4;
    int ns = 0, np = 0;
    fw_model_info(a->model, &ns, &np);
    bool ok = (pair ? encode_weights_pairs(&T.maps.w, a->weights_packed, nwo, a->nj,
                                           a->ni, LH, pitch)
                    : encode_weights(&T.maps.w, a->weights_packed, nwo, a->nj, a->ni,
                                     LH, pitch)) &&
              encode_2d(&T.maps.myo, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, a->myo, a->nj,
                        a->ni, kBoxB, LH, pitch) &&
              encode_2d(&T.maps.u[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a->u[0],
                        a->nj, a->ni, kBoxF, LH + 2, pitch) &&
              encode_2d(&T.maps.u[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a->u[1],
                        a->nj, a->ni, kBoxF, LH + 2, pitch) &&
              encode_2d(&T.maps.wc, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                        (const float *)a->weights + (int64_t)cen * a->ni * pitch,
                        a->nj, a->ni, kBoxF, LH, pitch);
    // maps of two state arrays in both buffers exist for every tissue (the
    // kernel acquires them); models with one state variable map the first
    // twice
    void *const *sbuf[2] = {a->state, a->state_b};
    for (int b = 0; b < 2; ++b)
        for (int q = 0; q < 2 && ok; ++q)
            ok = encode_2d(&T.maps.s[b][q], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                           sbuf[b][q < ns ? q : 0], a->nj, a->ni, kBoxF, LH, pitch);
    // the local activation flags (rows of `pitch` nodes, like the state)
    if (ok && a->n_lat > 0)
        ok = encode_2d(&T.maps.act, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1,
                       a->lat[0].activated, a->nj, a->ni, kBoxB, LH, pitch);
    if (!ok) {
        set_error("fw_batch_plan: tensor map encoding failed");
        return FW_ERR_UNSUPPORTED;
    }
    FusedK &f = T.f;
    f.w = nullptr;
    f.myo = a->myo;
    for (int b = 0; b < 2; ++b)
        for (int q = 0; q < FW_MAX_FUSED_STATE; ++q)
            T.state[b][q] = q < ns ? sbuf[b][q] : nullptr;
    for (int i = 0; i < FW_MAX_PARAMS; ++i) f.params[i] = (float)a->params[i];
    f.dt = (float)a->dt;
    f.ni = (int32_t)a->ni;
    f.nj = (int32_t)a->nj;
    f.pitch = (int32_t)pitch;
    f.n = a->ni * a->nj;
    f.tiles_j = (int32_t)((a->nj + TJ - 1) / TJ);
    f.status = a->status;
    f.n_stims = a->n_stims;
    for (int i = 0; i < a->n_stims; ++i) {
        const fw_stim &St = a->stims[i];
        FStim &F = f.stims[i];
        F.on = 0;
        F.kind = St.kind;
        F.has_umax = St.has_umax;
        F.value = (float)St.value;
        F.u_max = (float)St.u_max;
        F.lo0 = (int32_t)(St.lo[0] < 0 ? 0 : St.lo[0]);
        F.hi0 = (int32_t)(St.hi[0] > a->ni ? a->ni : St.hi[0]);
        F.lo1 = (int32_t)(St.lo[1] < 0 ? 0 : St.lo[1]);
        F.hi1 = (int32_t)(St.hi[1] > a->nj ? a->nj : St.hi[1]);
        F.mask = St.mask;
        T.stim_win[i] = BWin{St.first, St.last, 1};
    }
    f.n_at = a->n_at;
    for (int i = 0; i < a->n_at; ++i) {
        f.at[i] = FAt{0u, (float)a->at[i].threshold, a->at[i].act_step};
        T.at_win[i] = BWin{a->at[i].win.first, a->at[i].win.last, a->at[i].win.stride};
    }
    f.n_lat = a->n_lat;
    for (int i = 0; i < a->n_lat; ++i) {
        const fw_lat_tracker &L = a->lat[i];
        f.lat[i] = FLat{0u, (float)L.threshold, L.activated, L.cross_steps,
                        L.cross_count, L.capacity};
        T.lat_win[i] = BWin{L.win.first, L.win.last, L.win.stride};
    }
    f.n_probe = 0;
    T.u[0] = (float *)a->u[0];
    T.u[1] = (float *)a->u[1];
    T.step_base = n_begin;
    return FW_OK;
}

// Kernel of a batch: 2 (TMA) when every tissue can take it, unless every
// tissue asks for cp.async staging (fused_variant 1 or 2), or 3 (TMA,
// column pairs in two-wide instructions) when every tissue asks for
// fused_variant 6; else 1.  A row pitch other than nj needs a TMA kernel.
int choose_kernel(const fw_step_args *const *tissues, int32_t n, int *kernel)
{
    bool tma = true, cp = true, pair = true, pitched = false;
    for (int i = 0; i < n; ++i) {
        const fw_step_args *a = tissues[i];
        tma &= tma_tissue_ok(a);
        cp &= a->fused_variant == 1 || a->fused_variant == 2;
        pair &= a->fused_variant == 6;
        pitched |= a->pitch != 0 && a->pitch != a->nj;
    }
    if (pitched && (!tma || cp)) {
        set_error("fw_batch: a row pitch other than nj needs the TMA kernel "
                  "(pitch a multiple of 16 nodes, 16-byte aligned arrays, "
                  "packed weights)");
        return FW_ERR_UNSUPPORTED;
    }
    *kernel = tma && !cp ? (pair ? 3 : 2) : 1;
    return FW_OK;
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
    int kernel = 0;
    {
        int rc = choose_kernel(tissues, n, &kernel);
        if (rc) return rc;
    }
    const size_t desc = kernel >= 2 ? sizeof(BTissueT) : sizeof(BTissue);
    const size_t tile = kernel >= 2 ? sizeof(BTileT) : sizeof(BTile);
    *bytes = (int64_t)(align_up(desc * n, 256) + tile * (size_t)n_tiles);
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
    int kernel = 1;
    rc = choose_kernel(tissues, n, &kernel);
    if (rc) return rc;
    if (((uintptr_t)plan & (kernel >= 2 ? 127 : 15)) != 0) {
        set_error("fw_batch_plan: plan must be %d-byte aligned",
                  kernel >= 2 ? 128 : 16);
        return FW_ERR_ARG;
    }
    // host staging, 128-byte aligned like the device plan (the descriptors
    // of the TMA form hold 64-byte aligned tensor maps)
    std::vector<unsigned char> raw((size_t)need + 128, 0);
    unsigned char *host = raw.data() + ((128 - ((uintptr_t)raw.data() & 127)) & 127);
    const size_t desc_bytes = kernel >= 2 ? sizeof(BTissueT) : sizeof(BTissue);
    unsigned char *tiles_host = host + align_up(desc_bytes * n, 256);
    if (kernel >= 2) {
        BTissueT *desc = reinterpret_cast<BTissueT *>(host);
        for (int i = 0; i < n; ++i) {
            rc = fill_tma_tissue(tissues[i], n_begin[i], desc[i], kernel == 3);
            if (rc) return rc;
        }
    } else {
        BTissue *desc = reinterpret_cast<BTissue *>(host);
        for (int i = 0; i < n; ++i) {
            const fw_step_args *a = tissues[i];
            BHead &T = desc[i].h;
            T.w = (const float *)a->weights;
            T.myo = a->myo;
            T.u[0] = (float *)a->u[0];
            T.u[1] = (float *)a->u[1];
            int ns = 0, np = 0;
            fw_model_info(a->model, &ns, &np);
            for (int s = 0; s < kMaxState; ++s) {
                T.state[0][s] = s < ns ? a->state[s] : nullptr;
                T.state[1][s] = s < ns ? a->state_b[s] : nullptr;
            }
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
    int32_t t_count = 0;
    for (int i : order) {
        const fw_step_args *a = tissues[i];
        const int32_t nt = (int32_t)tissue_tiles(a);
        if (kernel >= 2) {
            BTileT *tl = reinterpret_cast<BTileT *>(tiles_host);
            const int32_t tj = (int32_t)((a->nj + TJ - 1) / TJ);
            for (int32_t k = 0; k < nt; ++k)
                tl[t_count + k] = BTileT{i,
                                         a->model * 8 + a->stencil +
                                             (a->n_lat ? kTileLat : 0),
                                         (k / tj) * TI - KMAX, (k % tj) * TJ - KMAX};
        } else {
            BTile *tl = reinterpret_cast<BTile *>(tiles_host);
            for (int32_t k = 0; k < nt; ++k) tl[t_count + k] = BTile{i, k};
        }
        t_count += nt;
    }
    FW_CUDA_CHECK(cudaMemcpyAsync(plan, host, (size_t)need,
                                  cudaMemcpyHostToDevice, stream));
    // the host staging buffer is released on return
    FW_CUDA_CHECK(cudaStreamSynchronize(stream));

    int dev = 0, sms = 0, per_sm = 0;
    FW_CUDA_CHECK(cudaGetDevice(&dev));
    FW_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (kernel >= 2) {
        // one persistent CTA per SM (the stages fill its shared memory)
        for (int g = 0; g < kGroups; ++g) {
            int rc2 = batch_group_launch(g, kernel == 3, true, false, 0, nullptr,
                                         nullptr, 0, 0, 0, 0, nullptr, stream);
            if (rc2) return rc2;
        }
        per_sm = 1;
    } else {
        FW_CUDA_CHECK(cudaFuncSetAttribute(
            k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem));
        FW_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, k_batch, NT, kSmem));
    }
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)sms * per_sm;
    if (grid > t_count) grid = t_count;
    out->plan = plan;
    out->n_tissues = n;
    out->n_tiles = t_count;
    out->ksteps = KMAX;
    out->grid = (int32_t)grid;
    out->kernel = kernel;
    // cumulative tile counts of the (model, stencil) groups in list order
    for (int g = 0; g < kGroups; ++g) {
        int32_t end = 0;
        for (int i = 0; i < n; ++i)
            if (tissues[i]->model * 8 + tissues[i]->stencil <= kGroupKey[g])
                end += (int32_t)tissue_tiles(tissues[i]);
        out->group_end[g] = end;
    }
    out->reserved = 0;
    return FW_OK;
}

int batch_run(const fw_batch *b, uint32_t *scratch, int64_t offset,
              int64_t n_steps, cudaStream_t stream)
{
    using namespace batch;
    if (!b || !b->plan || !scratch || b->n_tissues <= 0 || b->grid <= 0 ||
        b->kernel < 1 || b->kernel > 3) {
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
    const bool tma = b->kernel >= 2, pair = b->kernel == 3;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    FW_CUDA_CHECK(cudaStreamIsCapturing(stream, &cap));
    if (cap == cudaStreamCaptureStatusNone) {
        if (tma) {
            for (int g = 0; g < kGroups; ++g) {
                int rc = batch_group_launch(g, pair, true, false, 0, nullptr, nullptr, 0,
                                            0, 0, 0, nullptr, stream);
                if (rc) return rc;
            }
        } else {
            FW_CUDA_CHECK(cudaFuncSetAttribute(
                k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem));
        }
    }
    const size_t desc_bytes = tma ? sizeof(BTissueT) : sizeof(BTissue);
    const BTissue *desc = reinterpret_cast<const BTissue *>(b->plan);
    BTissueT *desc_t = reinterpret_cast<BTissueT *>(b->plan);
    const unsigned char *tiles_dev =
        (const unsigned char *)b->plan + align_up(desc_bytes * b->n_tissues, 256);
    const BTile *tl = reinterpret_cast<const BTile *>(tiles_dev);
    const BTileT *tl_t = reinterpret_cast<const BTileT *>(tiles_dev);
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
        if (tma) {
            const dim3 eb(32, 4);
            k_batch_events<<<(unsigned)((b->n_tissues + 3) / 4), eb, 0, stream>>>(
                desc_t, b->n_tissues, offset + done, (int32_t)ks, in_buf);
            FW_CHECK_LAUNCH("k_batch_events");
            // one kernel per (model, stencil) group, each on its own pair
            // of counters
            // of a launch: the first after k_batch_events in stream order,
            // the others overlapping the one before
            int32_t begin = 0;
            bool first = true;
            for (int g = 0; g < kGroups; ++g) {
                const int32_t end = b->group_end[g];
                if (end > begin) {
                    const int grid = end - begin < b->grid ? end - begin : b->grid;
                    int rc = batch_group_launch(g, pair, false, !first, grid, desc_t, tl_t,
                                                begin, end, b->n_tissues, in_buf,
                                                scratch + 2 + 2 * g, stream);
                    if (rc) return rc;
                    first = false;
                }
                begin = end;
            }
        } else {
            k_batch<<<b->grid, NT, kSmem, stream>>>(desc, tl, b->n_tiles,
                                                   b->n_tissues, offset + done,
                                                   (int32_t)ks, in_buf, scratch);
            FW_CHECK_LAUNCH("k_batch");
        }
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
    if (!b || !b->plan || b->n_tissues <= 0 || b->grid <= 0 ||
        b->kernel < 1 || b->kernel > 3) {
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
