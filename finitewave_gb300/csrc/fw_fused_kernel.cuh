// fw_fused_kernel.cuh -- the fused, temporally blocked FP32 form of the 2D
// step.
//
// One CTA owns a tile of TI x TJ grid nodes and advances it up to KMAX time
// steps per launch.  It stages a (TI + 2 KMAX) x (TJ + 2 KMAX) region once:
// the off-centre stencil weights and the potential go to shared memory with
// cp.async (no register staging), the ionic state and the myocyte flags of
// the nodes a thread owns go to registers.  The sub-steps then run on chip:
// after sub-step s every node at distance >= s from the region's edge is
// exact, so after KMAX sub-steps the tile interior is; the halo is computed
// redundantly by the neighbouring CTAs.  Per launch the tile's weights,
// state and potential cross HBM once instead of once per time step.
//
// Each thread owns a strip of R nodes in one column.  Per sub-step it reads
// the (R + 2) x 3 window of the current potential into registers first, then
// updates its R nodes into the other buffer, so no shared load waits behind a
// shared store.
//
// The diffusion sum  w_c u + sum_k w_k u_k  is one FMA chain (stencil_fma)
// over the stored weights: the off-centre ones from shared memory, each
// node's centre weight from its plane into registers with the state.  The
// TMA kernels and the batched kernel form it the same way, so every fused
// kernel gives bitwise the same node values.
//
// Inside each sub-step (global step n), in the reference's order
// (core/model/cardiac_model.py:164-178): stimuli on u (every node of the
// region with mesh == 1), trackers on the tile interior (they read u after
// the stimuli), then diffusion + ionic update into the other buffer.  Which
// stimuli and trackers act on which sub-step of a launch is decided on the
// host (bit s of `on`).
// Requirements (checked by the host): no special boundaries, and u and
// u_new equal at non-myocytes, so that a non-myocyte's value is the same in
// both buffers.
//
// Arithmetic: float32 with FMA contraction and fast division; compared with
// the float64 path by tolerance, not bitwise.
#pragma once

#include <stdio.h>
#include <string.h>

#include <type_traits>

#include "fw_internal.cuh"
#include "fw_models.cuh"

namespace fw {
namespace fused {

constexpr int kMaxFusedStims = FW_MAX_STIMS;
constexpr int kMaxFusedProbeEntries = 128;
// trackers evaluated in the fused kernel (more -> the host uses the plain
// form); kept small so that their state stays in registers
constexpr int kMaxFusedAt = 2;
constexpr int kMaxFusedLat = 1;

struct FStim {
    uint32_t on;  // bit s: applied on sub-step s of this launch
    int32_t kind, has_umax;
    float value, u_max;
    int32_t lo0, hi0, lo1, hi1;
    const int8_t *mask;
};

struct FAt {
    uint32_t on;
    float thr;
    int32_t *act;
};

struct FLat {
    uint32_t on;
    float thr;
    uint8_t *activated;
    int32_t *steps;
    int32_t *count;
    int32_t cap;
};

struct FProbe {
    uint32_t on;
    int64_t sample0;  // sample index of the first active sub-step
    const int64_t *cells;
    double *out;
    int64_t capacity;
    int32_t n_cells, n_vars;
    int32_t var_ids[FW_MAX_PROBE_VARS];
};

// (16-byte aligned and sized: the batched TMA kernel moves it with one
// bulk copy)
struct alignas(16) FusedK {
    const float *w;
    const int8_t *myo;
    const float *u_in;
    float *u_out;
    // the launch reads the state from `state` and writes the tiles' new
    // state to `state_out` (the other buffer, fw_step_args.state_b): a
    // region's halo state is then never one a neighbouring tile of the same
    // launch has already advanced
    void *state[FW_MAX_FUSED_STATE];
    void *state_out[FW_MAX_FUSED_STATE];
    // float32 parameters, rounded on the host: in the kernel they are plain
    // constant-bank operands (no float64 conversion on the device)
    float params[FW_MAX_PARAMS];
    float dt;
    int32_t ni, nj;
    int32_t pitch;   // row pitch (nodes) of u_out, state and myo (TMA forms)
    int64_t n;
    int64_t n0;
    int32_t ksteps;
    int32_t tiles_j;
    int32_t n_stims, n_at, n_lat, n_probe;
    uint32_t stim_on, probe_on;  // OR of the stimuli's / probes' masks
    FStim stims[kMaxFusedStims];
    FAt at[kMaxFusedAt];
    FLat lat[kMaxFusedLat];
    FProbe probe[FW_MAX_PROBE];
    int32_t *status;
    // weights formed on chip (fused_variant 5): D_al, D_ac, the scalar
    // conductivity and D_model * dt / dr**2, rounded to float32
    float fly_dal, fly_dac, fly_cond, fly_scale;
};

struct ProbeEntry {
    int16_t lr, col;
    int16_t tracker;
    int32_t cell;
};

// Off-centre weights held in shared memory, and the index of the centre plane
// in the global weight array.
template <int ST>
struct Stencil2D {
    static constexpr int NWO = ST == FW_STENCIL_ISO5 ? 4 : 8;
    static constexpr int CENTRE = ST == FW_STENCIL_ISO5 ? 2 : 4;
};

// Weights are grouped four per node (float4), so a node's off-centre weights
// are one (ISO5) or two (ANISO9) 16-byte shared loads.
template <int LW, int LH, int NWO>
struct Smem {
    float4 w[NWO / 4][LH][LW];
    // potential, ping-pong, with a one-node pad on every side so that the
    // 3x3 window of any region node needs no index clamping
    float u[2][LH + 2][LW + 2];
    uint32_t probe_bits[(LH * LW + 31) / 32];
    ProbeEntry probe_list[kMaxFusedProbeEntries];
    int probe_count;
};

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem,
                                          bool valid)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s),
                 "l"(gmem), "r"(valid ? 4 : 0));
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::);
}

// The diffusion sum of one node, w_c u + sum_k w_k u_k, as one FMA chain in
// the reference's term order (isotropic_stencil_2d.py:98-132,
// asymmetric_stencil_2d.py:165-201): rows above (ul, uc, ur), the node's own
// row (ml, mr) and below (dl, dc, dr).  Every fused kernel forms it this way
// from the stored weights, so they agree bitwise node by node.
template <int ST>
__device__ __forceinline__ float stencil_fma(float wcen, float c, const float4 &wa,
                                             const float4 &wb, float ul, float uc,
                                             float ur, float ml, float mr, float dl,
                                             float dc, float dr)
{
    float un = f_mul(wcen, c);
    if constexpr (ST == FW_STENCIL_ISO5) {
        un = f_fma(wa.x, uc, un);
        un = f_fma(wa.y, ml, un);
        un = f_fma(wa.z, mr, un);
        un = f_fma(wa.w, dc, un);
    } else {
        un = f_fma(wa.x, ul, un);
        un = f_fma(wa.y, uc, un);
        un = f_fma(wa.z, ur, un);
        un = f_fma(wa.w, ml, un);
        un = f_fma(wb.x, mr, un);
        un = f_fma(wb.y, dl, un);
        un = f_fma(wb.z, dc, un);
        un = f_fma(wb.w, dr, un);
    }
    return un;
}

// stencil_fma for two adjacent nodes of a row in two-wide instructions:
// w[q] = (node 0's, node 1's) off-centre weight q, and each window argument
// the pair of values the two nodes' chains take at that position.  Each
// lane is stencil_fma's chain, bit for bit.
template <int ST>
__device__ __forceinline__ float2 stencil_fma2(float2 wcen, float2 c, const float2 *w,
                                               float2 ul, float2 uc, float2 ur,
                                               float2 ml, float2 mr, float2 dl,
                                               float2 dc, float2 dr)
{
    float2 un = f2_mul(wcen, c);
    if constexpr (ST == FW_STENCIL_ISO5) {
        un = f2_fma(w[0], uc, un);
        un = f2_fma(w[1], ml, un);
        un = f2_fma(w[2], mr, un);
        un = f2_fma(w[3], dc, un);
    } else {
        un = f2_fma(w[0], ul, un);
        un = f2_fma(w[1], uc, un);
        un = f2_fma(w[2], ur, un);
        un = f2_fma(w[3], ml, un);
        un = f2_fma(w[4], mr, un);
        un = f2_fma(w[5], dl, un);
        un = f2_fma(w[6], dc, un);
        un = f2_fma(w[7], dr, un);
    }
    return un;
}

// The ionic update of the fused and batched kernels: a model with a
// two-node form (M::update_pair) uses its explicitly rounded float32
// update (M::update_fused), which the pair form reproduces per node;
// otherwise update<float>, once per node.
template <class M, class = void>
struct has_pair_form : std::false_type {};
template <class M>
struct has_pair_form<M, std::void_t<decltype(&M::update_pair)>> : std::true_type {};

template <class M>
__device__ __forceinline__ float fused_update(float u, float un,
                                              typename M::template St<float> &x,
                                              const Params<float, M::NP> &P, float dt)
{
    if constexpr (has_pair_form<M>::value)
        return M::update_fused(u, un, x, P, dt);
    else
        return M::template update<float>(u, un, x, P, dt);
}

template <class M>
__device__ __forceinline__ float2 fused_update_pair(float2 u, float2 un,
                                                   typename M::template St<float> &x0,
                                                   typename M::template St<float> &x1,
                                                   const Params<float, M::NP> &P,
                                                   float dt)
{
    if constexpr (has_pair_form<M>::value) {
        return M::update_pair(u, un, x0, x1, P, dt);
    } else {
        const float a = M::template update<float>(u.x, un.x, x0, P, dt);
        const float b = M::template update<float>(u.y, un.y, x1, P, dt);
        return make_float2(a, b);
    }
}

// Rows r < R of a strip (potential x[r + 1]) that compare with a threshold,
// as bit masks: the trackers test whole strips without a branch per row and
// branch only on the rare rows that record something.  Each comparison is
// the reference's own, so NaN rows match none of them.
template <int R>
__device__ __forceinline__ uint32_t rows_gt(const float (&x)[R + 2], float thr)
{
    uint32_t m = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) m |= (x[r + 1] > thr ? 1u : 0u) << r;
    return m;
}

template <int R>
__device__ __forceinline__ uint32_t rows_ge(const float (&x)[R + 2], float thr)
{
    uint32_t m = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) m |= (x[r + 1] >= thr ? 1u : 0u) << r;
    return m;
}

template <int R>
__device__ __forceinline__ uint32_t rows_lt(const float (&x)[R + 2], float thr)
{
    uint32_t m = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) m |= (x[r + 1] < thr ? 1u : 0u) << r;
    return m;
}

// Append step n to the crossing list of node p (rare: once per crossing).
static __device__ __noinline__ void lat_record(const FLat &L, int64_t p,
                                               int64_t n_nodes, int64_t n,
                                               int32_t *status)
{
    const int32_t c = L.count[p];
    if (c < L.cap)
        L.steps[(int64_t)c * n_nodes + p] = (int32_t)n;
    else if (status)
        atomicOr(status, FW_DEV_LAT_OVERFLOW);
    L.count[p] = c + 1;
}

// Probe trackers at node (lr, col) on sub-step s: u after stimuli (u_c) and
// the state variables after the update, or, at a non-myocyte, the unchanging
// stored state (action_potential_2d_tracker.py:46-53, multi_variable_2d_
// tracker.py:58-69).  Rare path, kept out of line.
template <class M>
__device__ __noinline__ void write_probes(
    const FusedK &k, const ProbeEntry *list, int count, int lr, int col, int s,
    float u_c, const typename M::template St<float> st, bool myo, int64_t p)
{
    for (int e = 0; e < count && e < kMaxFusedProbeEntries; ++e) {
        const ProbeEntry pe = list[e];
        if (pe.lr != lr || pe.col != col) continue;
        const FProbe &PR = k.probe[pe.tracker];
        if (!((PR.on >> s) & 1u)) continue;
        const int64_t smp = PR.sample0 + __popc(PR.on & ((1u << s) - 1u));
        if (smp >= PR.capacity) {
            if (k.status) atomicOr(k.status, FW_DEV_PROBE_OVERFLOW);
            continue;
        }
        for (int v = 0; v < PR.n_vars; ++v) {
            const int id = PR.var_ids[v];
            double x;
            if (id == 0)
                x = (double)u_c;
            else if (myo)
                x = M::probe(st, id - 1);
            else
                x = (double)((const float *)k.state[id - 1])[p];
            PR.out[(smp * PR.n_vars + v) * (int64_t)PR.n_cells + pe.cell] = x;
        }
    }
}

template <class M, int ST, int KMAX, int LW, int LH, int R, int MINB>
__global__ void __launch_bounds__(LW *(LH / R), MINB)
    k_fused(const __grid_constant__ FusedK k)
{
    constexpr int NT = LW * (LH / R);
    constexpr int TI = LH - 2 * KMAX, TJ = LW - 2 * KMAX;
    constexpr int NWO = Stencil2D<ST>::NWO;
    constexpr int CEN = Stencil2D<ST>::CENTRE;
    static_assert(LH % R == 0 && NT % LW == 0, "strip layout");
    static_assert(TI > 0 && TJ > 0, "halo larger than the region");
    static_assert(R <= 8 && KMAX <= 32, "bit masks");

    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem<LW, LH, NWO> &S = *reinterpret_cast<Smem<LW, LH, NWO> *>(smem_raw);

    const int tid = threadIdx.x;
    const int col = tid % LW;
    const int strip = tid / LW;
    const int r0 = strip * R;
    const int tile = blockIdx.x;
    const int bi = tile / k.tiles_j, bj = tile % k.tiles_j;
    const int oi = bi * TI - KMAX;   // global row of region row 0
    const int oj = bj * TJ - KMAX;   // global column of region column 0
    const int gj = oj + col;
    const bool col_in = gj >= 0 && gj < k.nj;
    const bool col_interior = col >= KMAX && col < KMAX + TJ;

    // ---- stage the region ------------------------------------------------------
    // Thread tid stages column `col` at rows tid / LW + i * (NT / LW):
    // the potential and the off-centre weight planes, cp.async straight into
    // shared memory; nodes outside the grid are zero-filled.
    {
        constexpr int ROWS = NT / LW, PER = LH / ROWS;
        const int lr0 = tid / LW;
        const float *wbase[NWO];
#pragma unroll
        for (int q = 0; q < NWO; ++q)
            wbase[q] = k.w + (int64_t)(q < CEN ? q : q + 1) * k.n;
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const int lr = lr0 + i * ROWS;
            const int gi = oi + lr;
            const bool in = col_in && gi >= 0 && gi < k.ni;
            const int64_t p = in ? (int64_t)gi * k.nj + gj : 0;
            cp_async4(&S.u[0][lr + 1][col + 1], k.u_in + p, in);
#pragma unroll
            for (int q = 0; q < NWO; ++q)
                cp_async4(reinterpret_cast<float *>(&S.w[q >> 2][lr][col]) + (q & 3),
                          wbase[q] + p, in);
        }
    }
    // state, centre weights and myocyte flags of the nodes this thread owns
    typename M::template St<float> st[R];
    float wcen[R];
    uint32_t myo_bits = 0, own = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int lr = r0 + r, gi = oi + lr;
        const bool in = col_in && gi >= 0 && gi < k.ni;
        const int64_t p = in ? (int64_t)gi * k.nj + gj : 0;
        const int8_t m = k.myo[p];
        st[r] = M::template load<float>(k.state, p);
        wcen[r] = k.w[(int64_t)CEN * k.n + p];
        if (in && m) myo_bits |= 1u << r;
        if (in && col_interior && lr >= KMAX && lr < KMAX + TI) own |= 1u << r;
    }
    if (k.n_probe) {
        for (int i = tid; i < (LH * LW + 31) / 32; i += NT) S.probe_bits[i] = 0;
        if (tid == 0) S.probe_count = 0;
    }
    // zero the pad ring of both potential buffers (read, never used)
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
    // local activation state of owned nodes: bit (l * 8 + r)
    uint32_t lat_act = 0, at_done = 0;
#pragma unroll
    for (int l = 0; l < kMaxFusedLat; ++l)
        if (l < k.n_lat) {
#pragma unroll
            for (int r = 0; r < R; ++r)
                if ((own >> r) & 1u) {
                    const int64_t p = (int64_t)(oi + r0 + r) * k.nj + gj;
                    if (k.lat[l].activated[p]) lat_act |= 1u << (l * 8 + r);
                }
        }
    cp_async_wait_all();
    __syncthreads();
    // (buffer 1 needs no copy: every sub-step writes every node of the other
    // buffer, non-myocytes with their unchanged value)

    // ---- probe cells inside this tile's interior ------------------------------------
    uint32_t probe_mine = 0;
    if (k.n_probe) {
        for (int t = 0; t < k.n_probe; ++t) {
            const FProbe &pr = k.probe[t];
            for (int c = tid; c < pr.n_cells; c += NT) {
                const int64_t p = pr.cells[c];
                const int gi = (int)(p / k.nj), gjj = (int)(p % k.nj);
                const int lr = gi - oi, lc = gjj - oj;
                if (lr >= KMAX && lr < KMAX + TI && lc >= KMAX &&
                    lc < KMAX + TJ) {
                    const int e = atomicAdd(&S.probe_count, 1);
                    if (e < kMaxFusedProbeEntries) {
                        S.probe_list[e] = ProbeEntry{(int16_t)lr, (int16_t)lc,
                                                     (int16_t)t, c};
                        const int bit = lr * LW + lc;
                        atomicOr(&S.probe_bits[bit >> 5], 1u << (bit & 31));
                    } else if (k.status) {
                        atomicOr(k.status, FW_DEV_PROBE_OVERFLOW);
                    }
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int bit = (r0 + r) * LW + col;
            if ((S.probe_bits[bit >> 5] >> (bit & 31)) & 1u)
                probe_mine |= 1u << r;
        }
    }

    Params<float, M::NP> P;
#pragma unroll
    for (int i = 0; i < M::NP; ++i) P.v[i] = k.params[i];
    const float dt = k.dt;
    // rows whose update is defined (the region's outer ring is never read)
    uint32_t upd = 0;
    if (col > 0 && col < LW - 1) {
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (r0 + r > 0 && r0 + r < LH - 1) upd |= 1u << r;
    }
    upd &= myo_bits;

    // ---- sub-steps ----------------------------------------------------------------
    for (int s = 0; s < k.ksteps; ++s) {
        const int64_t n = k.n0 + s;
        const int cb = s & 1;
        // padded buffers: region node (lr, c) lives at [lr + 1][c + 1]
        float(*cur)[LW + 2] = S.u[cb];
        float(*nxt)[LW + 2] = S.u[cb ^ 1];

        // stimuli (stim_sequence.py:65-77) on every node of the region
        if ((k.stim_on >> s) & 1u) {
            for (int i = 0; i < k.n_stims; ++i) {
                const FStim &F = k.stims[i];
                if (!((F.on >> s) & 1u)) continue;
                if (gj < F.lo1 || gj >= F.hi1) continue;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (!((myo_bits >> r) & 1u)) continue;
                    const int lr = r0 + r, gi = oi + lr;
                    if (gi < F.lo0 || gi >= F.hi0) continue;
                    if (F.mask && !F.mask[(int64_t)gi * k.nj + gj]) continue;
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

        // the (R + 2) x 3 window of u: region rows r0 - 1 .. r0 + R
        float wl[R + 2], wc[R + 2], wr[R + 2];
#pragma unroll
        for (int i = 0; i < R + 2; ++i) {
            wl[i] = cur[r0 + i][col];
            wc[i] = cur[r0 + i][col + 1];
            wr[i] = cur[r0 + i][col + 2];
        }

        // trackers on the owned interior nodes (tracker.py:70-83)
        if (own) {
#pragma unroll
            for (int a = 0; a < kMaxFusedAt; ++a) {
                if (a >= k.n_at || !((k.at[a].on >> s) & 1u)) continue;
                // (act_t < 0) & (u > threshold)
                // (activation_time_2d_tracker.py:61-63): the first crossing
                // has the smallest step and "never" (-1) is the largest
                // unsigned value, so an unsigned atomic minimum keeps the
                // first step without reading it
                // the strip's maximum first: most sub-steps cross nowhere
                // (fmaxf skips NaN rows, which never cross)
                float mx = wc[1];
#pragma unroll
                for (int r = 1; r < R; ++r) mx = fmaxf(mx, wc[r + 1]);
                if (!(mx > k.at[a].thr)) continue;
                const uint32_t hit =
                    rows_gt<R>(wc, k.at[a].thr) & own & ~(at_done >> (a * 8));
                if (hit) {
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        if (!((hit >> r) & 1u)) continue;
                        const int64_t p = (int64_t)(oi + r0 + r) * k.nj + gj;
                        atomicMin(reinterpret_cast<unsigned *>(k.at[a].act) + p,
                                  (unsigned)n);
                    }
                    at_done |= hit << (a * 8);
                }
            }
#pragma unroll
            for (int l = 0; l < kMaxFusedLat; ++l) {
                if (l >= k.n_lat || !((k.lat[l].on >> s) & 1u)) continue;
                // cross_threshold (local_activation_time_2d_tracker.py:71-89):
                // rows rising to >= threshold record the step, rows below it
                // re-arm
                const uint32_t was = (lat_act >> (l * 8)) & 0xffu;
                const uint32_t rise = rows_ge<R>(wc, k.lat[l].thr) & own & ~was;
                const uint32_t fall = rows_lt<R>(wc, k.lat[l].thr) & own & was;
                lat_act ^= (rise | fall) << (l * 8);
                if (rise) {
#pragma unroll
                    for (int r = 0; r < R; ++r)
                        if ((rise >> r) & 1u)
                            lat_record(k.lat[l], (int64_t)(oi + r0 + r) * k.nj + gj,
                                       k.n, n, k.status);
                }
            }
        }

        // diffusion + ionic update of the strip into the other buffer.  The
        // update is computed for every node and kept only where it is defined
        // (myocytes off the region's ring); the state of the other nodes is
        // never written back.
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float b1 = wc[r + 1];
            const int lr = r0 + r;
            const float4 wa = S.w[0][lr][col];
            const float4 wb = NWO == 8 ? S.w[NWO / 4 - 1][lr][col] : wa;
            const float un = stencil_fma<ST>(wcen[r], b1, wa, wb, wl[r], wc[r], wr[r],
                                             wl[r + 1], wr[r + 1], wl[r + 2],
                                             wc[r + 2], wr[r + 2]);
            const float uu = fused_update<M>(b1, un, st[r], P, dt);
            nxt[lr + 1][col + 1] = ((upd >> r) & 1u) ? uu : b1;
        }
        // probes: u after the stimuli, the state after the update
        if (probe_mine && ((k.probe_on >> s) & 1u)) {
#pragma unroll
            for (int r = 0; r < R; ++r)
                if ((probe_mine >> r) & 1u)
                    write_probes<M>(k, S.probe_list, S.probe_count, r0 + r, col, s,
                                    wc[r + 1], st[r], ((myo_bits >> r) & 1u) != 0,
                                    (int64_t)(oi + r0 + r) * k.nj + gj);
        }
        __syncthreads();
    }

    // ---- write the interior back --------------------------------------------------
    const int fb = k.ksteps & 1;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (!((own >> r) & 1u)) continue;
        const int lr = r0 + r;
        const int64_t p = (int64_t)(oi + lr) * k.nj + gj;
        if ((myo_bits >> r) & 1u) {
            const float uo = S.u[fb][lr + 1][col + 1];
            k.u_out[p] = uo;
            if (!isfinite(uo) && k.status) atomicOr(k.status, FW_DEV_NONFINITE);
            M::template store<float>(k.state_out, p, st[r]);
        }
#pragma unroll
        for (int l = 0; l < kMaxFusedLat; ++l)
            if (l < k.n_lat)
                k.lat[l].activated[p] = (lat_act >> (l * 8 + r)) & 1u;
    }
}

// ---------------------------------------------------------------- host side

// Bit s set when step n0 + s (s < ks) is in [first, last] and a multiple of
// stride.
inline uint32_t sub_step_mask(int64_t n0, int64_t ks, int64_t first,
                              int64_t last, int64_t stride)
{
    uint32_t m = 0;
    for (int64_t s = 0; s < ks; ++s) {
        const int64_t n = n0 + s;
        if (n >= first && n <= last && n % stride == 0) m |= 1u << s;
    }
    return m;
}

// Stimuli and trackers acting during the launch of steps n0..n1 (ks steps):
// per sub-step activity masks, computed on the host.
inline int fill_events(const fw_step_args *a, FusedK &k, int64_t n0, int64_t n1,
                       int64_t ks, int64_t *probe_samples)
{
    k.n_stims = 0;
    k.stim_on = 0;
    for (int i = 0; i < a->n_stims; ++i) {
        const fw_stim &St = a->stims[i];
        if (St.last < n0 || St.first > n1) continue;
        if (k.n_stims >= kMaxFusedStims) {
            set_error("fw_step (fused): more than %d stimuli active in one "
                      "launch", kMaxFusedStims);
            return FW_ERR_UNSUPPORTED;
        }
        FStim &f = k.stims[k.n_stims++];
        f.on = sub_step_mask(n0, ks, St.first, St.last, 1);
        f.kind = St.kind;
        f.has_umax = St.has_umax;
        f.value = (float)St.value;
        f.u_max = (float)St.u_max;
        f.lo0 = (int32_t)(St.lo[0] < 0 ? 0 : St.lo[0]);
        f.hi0 = (int32_t)(St.hi[0] > a->ni ? a->ni : St.hi[0]);
        f.lo1 = (int32_t)(St.lo[1] < 0 ? 0 : St.lo[1]);
        f.hi1 = (int32_t)(St.hi[1] > a->nj ? a->nj : St.hi[1]);
        f.mask = St.mask;
        k.stim_on |= f.on;
    }
    k.n_at = 0;
    for (int i = 0; i < a->n_at; ++i) {
        const fw_at_tracker &A = a->at[i];
        const uint32_t on = sub_step_mask(n0, ks, A.win.first, A.win.last,
                                          A.win.stride);
        if (!on) continue;
        if (k.n_at >= kMaxFusedAt) {
            set_error("fw_step (fused): more than %d activation trackers "
                      "active in one launch", kMaxFusedAt);
            return FW_ERR_UNSUPPORTED;
        }
        k.at[k.n_at++] = FAt{on, (float)A.threshold, A.act_step};
    }
    k.n_lat = 0;
    for (int i = 0; i < a->n_lat; ++i) {
        const fw_lat_tracker &Lt = a->lat[i];
        k.lat[k.n_lat++] = FLat{sub_step_mask(n0, ks, Lt.win.first,
                                              Lt.win.last, Lt.win.stride),
                                (float)Lt.threshold, Lt.activated,
                                Lt.cross_steps, Lt.cross_count,
                                Lt.capacity};
    }
    k.n_probe = 0;
    k.probe_on = 0;
    for (int i = 0; i < a->n_probe; ++i) {
        const fw_probe_tracker &Pp = a->probe[i];
        const uint32_t on = sub_step_mask(n0, ks, Pp.win.first, Pp.win.last,
                                          Pp.win.stride);
        if (!on) continue;
        FProbe &f = k.probe[k.n_probe++];
        f.on = on;
        f.sample0 = probe_samples[i];
        probe_samples[i] += __builtin_popcount(on);
        f.cells = Pp.cells;
        f.out = Pp.out;
        f.capacity = Pp.capacity;
        f.n_cells = Pp.n_cells;
        f.n_vars = Pp.n_vars;
        for (int v = 0; v < FW_MAX_PROBE_VARS; ++v)
            f.var_ids[v] = Pp.var_ids[v];
        k.probe_on |= on;
    }
    return FW_OK;
}

template <class M, int ST, int KMAX, int LW, int LH, int R, int MINB>
int launch_fused(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                 cudaStream_t stream)
{
    constexpr int TI = LH - 2 * KMAX, TJ = LW - 2 * KMAX;
    constexpr int NT = LW * (LH / R);
    constexpr size_t SMEM = sizeof(Smem<LW, LH, Stencil2D<ST>::NWO>);
    auto kern = k_fused<M, ST, KMAX, LW, LH, R, MINB>;
    // per call (cheap), so that it holds on whichever device is current
    FW_CUDA_CHECK(cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM));
    if (a->n_lat > kMaxFusedLat) {
        set_error("fw_step (fused): at most %d local activation tracker",
                  kMaxFusedLat);
        return FW_ERR_UNSUPPORTED;
    }
    FusedK k;
    memset(&k, 0, sizeof k);
    k.w = (const float *)a->weights;
    k.myo = a->myo;
    void *const *sbuf[2] = {a->state, a->state_b};
    for (int i = 0; i < FW_MAX_PARAMS; ++i) k.params[i] = (float)a->params[i];
    k.dt = (float)a->dt;
    k.ni = (int32_t)a->ni;
    k.nj = (int32_t)a->nj;
    k.n = a->ni * a->nj;
    k.status = a->status;
    const int tiles_i = (int)((a->ni + TI - 1) / TI);
    k.tiles_j = (int)((a->nj + TJ - 1) / TJ);
    const int64_t blocks = (int64_t)tiles_i * k.tiles_j;
    int64_t probe_samples[FW_MAX_PROBE];
    for (int i = 0; i < a->n_probe; ++i) probe_samples[i] = a->probe[i].sample_offset;

    // launch sizes: L launches of <= KMAX steps with L == n_steps (mod 2), so
    // that the result ends in u[n_steps & 1] as in the plain form.
    int64_t L = (n_steps + KMAX - 1) / KMAX;
    if ((L & 1) != (n_steps & 1)) ++L;
    int64_t done = 0;
    for (int64_t li = 0; li < L; ++li) {
        const int64_t left = n_steps - done, launches_left = L - li;
        int64_t ks = (left + launches_left - 1) / launches_left;
        if (ks > KMAX) ks = KMAX;
        const int64_t n0 = n_begin + done;
        const int64_t n1 = n0 + ks - 1;
        k.n0 = n0;
        k.ksteps = (int32_t)ks;
        k.u_in = (const float *)a->u[li & 1];
        k.u_out = (float *)a->u[(li + 1) & 1];
        for (int q = 0; q < FW_MAX_FUSED_STATE; ++q) {
            k.state[q] = sbuf[li & 1][q];
            k.state_out[q] = sbuf[(li + 1) & 1][q];
        }
        int rc = fill_events(a, k, n0, n1, ks, probe_samples);
        if (rc) return rc;
        kern<<<(unsigned)blocks, NT, SMEM, stream>>>(k);
        FW_CHECK_LAUNCH("k_fused");
        done += ks;
    }
    return FW_OK;
}

}  // namespace fused
}  // namespace fw
