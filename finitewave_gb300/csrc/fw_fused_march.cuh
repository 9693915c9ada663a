// fw_fused_march.cuh -- the fused float32 2D step as a row-marching wavefront
// (fused variant 7).
//
// The tile kernels (fw_fused_tma.cuh) advance a 64 x 32 region K steps and
// keep only its 56 x 24 interior: at K = 4 they compute 1.52 node-updates
// per node kept.  This kernel removes the halo along rows.  A CTA owns a
// 64-column strip (56 interior columns, K halo columns each side, as the
// tiles) and a segment of rows, and marches down the segment in blocks of
// 8 rows with all K time levels in flight at once:
//
//   * phase p: level 1 (the first time step) advances row block p from
//     the input rows, level 2 advances block p - 1 from level 1's rows,
//     ..., level K block p - K + 1 from level K - 1's rows, which is
//     written out.  Level s's blocks are shifted up by s - 1 rows, so that
//     level s's block b depends only on level s - 1's blocks b - 1 and b,
//     both finished in earlier phases: one barrier per phase;
//   * the input rows (potential, state, packed weights, centre weights,
//     myocyte and local activation flags) arrive by TMA in blocks of 8
//     rows into a ring of K + 3 blocks, two blocks ahead of their first
//     use, each block on its own mbarrier; a level's output rows go to a
//     ring of three blocks in shared memory;
//   * thread (r, c) -- column c, row r of a block -- handles at every level
//     the one row i == r (mod 8) of that level's block, so a node meets the
//     same thread at all K levels: its state variables and tracker flags
//     pass from level to level in registers (one phase later, or two where
//     (r + s) is a multiple of 8, which is fixed per thread and level).
//
// Only the K - 1 + K extra rows at each end of a segment are computed twice
// (segments are hundreds of rows), so the work per node kept is 64 / 56 =
// 1.14 node-updates.  Each node-update is the tile kernels' own arithmetic:
// the same FMA chain over the same stored weights (stencil_fma) and the
// same ionic update (fused_update), stimuli applied to the potential a
// level reads and trackers tested on it in the reference's order
// (core/model/cardiac_model.py:164-178), so every node gets the bits of
// the other fused variants.  Probe trackers are not handled here (the host
// picks another variant when a model has them).
#pragma once

#include "fw_fused_tma.cuh"

namespace fw {
namespace fused {

constexpr int kMBR = 8;               // rows per block
constexpr int kMNT = kTW * kMBR;      // 512 threads
constexpr int kMarchSeg = 512;        // rows per segment (a multiple of kMBR)

template <int NS, int NWO, int KMAX>
struct MarchSmem {
    static constexpr int NBI = KMAX + 3;      // input blocks in the ring
    static constexpr int RI = NBI * kMBR;     // input ring rows
    static constexpr int RL = 3 * kMBR;       // rows of a level's ring
    alignas(128) float4 wa[RI][kTW];                 // packed weights 0..3
    alignas(128) float4 wb[NWO == 8 ? RI : 1][kTW];  // packed weights 4..7
    alignas(128) float wc[RI][kBoxF];                // centre weights
    alignas(128) float u0[RI][kBoxF];                // input potential
    alignas(128) float s0[NS][RI][kBoxF];            // input state
    alignas(128) int8_t myo[RI][kBoxB];
    alignas(128) uint8_t act[RI][kBoxB];             // local activation flags
    alignas(128) float ul[KMAX > 1 ? KMAX - 1 : 1][RL][kBoxF];  // levels 1..K-1
    alignas(8) uint64_t bar[NBI];
};

struct MarchK {
    TmaK t;              // maps (8-row boxes), launch description, items
    int32_t strips;      // 64-column strips
    int32_t segs;        // row segments per strip
};

// Issue input block q (rows 8q + 1 .. 8q + 8) into ring slot `slot`.
template <int NS, int NWO, class Sm>
__device__ __forceinline__ void march_issue(const TmaMaps &maps, int in_buf, Sm &S,
                                            int slot, int q, int oj, bool lat)
{
    constexpr int BR = kMBR;
    const int y0 = q * BR + 1, r0 = slot * BR;
    const int x4 = floor_to(oj - 1, 4), x16 = floor_to(oj, 16);
    uint64_t *bar = &S.bar[slot];
    const unsigned bytes =
        (unsigned)(BR * (sizeof(S.wa[0]) * (NWO == 8 ? 2 : 1) + sizeof(S.wc[0]) +
                         sizeof(S.u0[0]) + NS * sizeof(S.s0[0][0]) + sizeof(S.myo[0]) +
                         (lat ? sizeof(S.act[0]) : 0)));
    mbar_expect_tx(bar, bytes);
    tma_3d(&S.wa[r0][0], &maps.w, 0, oj, y0, bar);
    if constexpr (NWO == 8) tma_3d(&S.wb[r0][0], &maps.w, 4, oj, y0, bar);
    tma_2d(&S.wc[r0][0], &maps.wc, x4, y0, bar);
    tma_2d(&S.u0[r0][0], &maps.u[in_buf], x4, y0, bar);
#pragma unroll
    for (int q2 = 0; q2 < NS; ++q2)
        tma_2d(&S.s0[q2][r0][0], &maps.s[in_buf][q2], x4, y0, bar);
    tma_2d(&S.myo[r0][0], &maps.myo, x16, y0, bar);
    if (lat) tma_2d(&S.act[r0][0], &maps.act, x16, y0, bar);
}

template <class M, int ST, int KMAX>
__global__ void __launch_bounds__(kMNT, 1) k_fused_march(const __grid_constant__ MarchK mk)
{
    constexpr int BR = kMBR;
    constexpr int NS = M::NS;
    constexpr int NWO = Stencil2D<ST>::NWO;
    using Sm = MarchSmem<NS, NWO, KMAX>;
    constexpr int NBI = Sm::NBI, RI = Sm::RI, RL = Sm::RL;
    static_assert(KMAX >= 1 && KMAX <= 4, "levels in flight");
    static_assert(NS <= kMaxTmaState, "state arrays");
    static_assert(kMarchSeg % BR == 0, "segments of whole blocks");

    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned mis = smem_u32(smem_raw) & 127u;
    Sm &S = *reinterpret_cast<Sm *>(smem_raw + (mis ? 128u - mis : 0u));
    const TmaK &k = mk.t;
    const FusedK &f = k.f;

    const int tid = threadIdx.x;
    const int c = tid % kTW;        // column of the strip
    const int r = tid / kTW;        // row of a block (0..7)
    const bool lat = f.n_lat > 0;

    if (tid == 0) {
        for (int j = 0; j < NBI; ++j) mbar_init(&S.bar[j], 1);
        mbar_fence_init();
    }
    __syncthreads();

    Params<float, M::NP> P;
#pragma unroll
    for (int i = 0; i < M::NP; ++i) P.v[i] = f.params[i];
    const float dt = f.dt;
    const int ksteps = f.ksteps;
    const int64_t n0 = f.n0;
    const uint32_t stim_on = f.stim_on;
    uint32_t at_on[kMaxFusedAt], lat_on[kMaxFusedLat];
    float at_thr[kMaxFusedAt], lat_thr[kMaxFusedLat];
#pragma unroll
    for (int a = 0; a < kMaxFusedAt; ++a) {
        at_on[a] = a < f.n_at ? f.at[a].on : 0u;
        at_thr[a] = f.at[a].thr;
    }
#pragma unroll
    for (int l = 0; l < kMaxFusedLat; ++l) {
        lat_on[l] = l < f.n_lat ? f.lat[l].on : 0u;
        lat_thr[l] = f.lat[l].thr;
    }
    // transition s -> s + 1 of this thread's nodes waits two phases where
    // (r + s) is a multiple of 8 (bit s)
    uint32_t gap2 = 0;
#pragma unroll
    for (int s = 1; s < KMAX; ++s)
        if (((r + s) & 7) == 0) gap2 |= 1u << s;

    int64_t g0 = 0;   // blocks this CTA has issued before the current segment
    for (int item = blockIdx.x; item < k.tiles; item += gridDim.x) {
        const int sj = item % mk.strips, sg = item / mk.strips;
        const int oj = sj * (kTW - 2 * KMAX) - KMAX;
        const int R0 = sg * kMarchSeg;
        const int R1 = R0 + kMarchSeg < f.ni ? R0 + kMarchSeg : f.ni;
        const int xo = oj - floor_to(oj - 1, 4);    // 1..4
        const int xo8 = oj - floor_to(oj, 16);      // 0..15
        const int gj = oj + c;
        const bool col_in = (unsigned)gj < (unsigned)f.nj;
        const bool col_own = col_in && c >= KMAX && c < kTW - KMAX;
        const bool col_upd = c > 0 && c < kTW - 1;
        // level 1's blocks p0 .. bend cover rows R0 - K + 1 .. R1 + K - 2;
        // input blocks p0 - 1 .. bend
        const int p0 = floor_to(R0 - KMAX + 1, BR) / BR;
        const int bend = (R1 + KMAX - 2) / BR;
        const int qf = p0 - 1, ql = bend;
        // input ring row of global row i: block q = floor((i - 1) / 8) sits in
        // slot (g0 + q - qf) % NBI
        const int base = (int)((g0 % NBI) * BR) - BR * qf - 1 + RI * 64;
        auto irow = [&](int i) -> int { return (i + base) % RI; };
        auto slot_of = [&](int q) -> int { return (int)((g0 + (q - qf)) % NBI); };
        auto parity_of = [&](int q) -> unsigned { return (unsigned)(((g0 + (q - qf)) / NBI) & 1); };

        if (tid == 0) {
            fence_proxy_async();
            for (int q = qf; q <= qf + 2 && q <= ql; ++q)
                march_issue<NS, NWO>(k.maps, k.in_buf, S, slot_of(q), q, oj, lat);
        }

        // per-node values carried from level to level (this thread's
        // nodes): the state entering level s, and 4 flag bits per level at
        // bit 4 s -- the local activation flag (bit 0) and whether each
        // activation tracker has recorded the node in this launch (bits 1, 2)
        typename M::template St<float> st_in[KMAX + 1], st_out[KMAX + 1],
            st_hold[KMAX + 1];
        uint32_t bits_in = 0, bits_out = 0, bits_hold = 0;
        bool nonfinite = false;
        // this thread's row at level s in the current phase (it advances by
        // one block per phase), its input ring row and its level ring row
        int i_s[KMAX + 1], ir_s[KMAX + 1], lr_s[KMAX + 1];
#pragma unroll
        for (int s = 1; s <= KMAX; ++s) {
            i_s[s] = BR * (p0 - s + 1) - s + 1 + ((r + s - 1) & 7);
            ir_s[s] = irow(i_s[s]);
            lr_s[s] = (i_s[s] + s - 1 + RL * 64) % RL;
        }

        const int p_last = bend + ksteps - 1;
        for (int p = p0; p <= p_last; ++p) {
            // the next block but one, into the slot of a block no longer read
            if (tid == 0 && p + 2 > qf + 2 && p + 2 <= ql) {
                fence_proxy_async();
                march_issue<NS, NWO>(k.maps, k.in_buf, S, slot_of(p + 2), p + 2, oj, lat);
            }
            bool arrived = true;
            if (p <= ql) arrived = mbar_wait(&S.bar[slot_of(p)], parity_of(p));
            if (p == p0) arrived = mbar_wait(&S.bar[slot_of(qf)], parity_of(qf)) && arrived;
            if (__syncthreads_or(!arrived || k.force_timeout)) {
                if (tid == 0) {
                    if (f.status) atomicOr(f.status, FW_DEV_TIMEOUT);
                    // wait (bounded) for every block issued and not yet
                    // seen complete, so none lands after the CTA has exited
                    const int q_hi = (p + 2 <= ql) ? p + 2 : ql;
                    for (int q = (p == p0 ? qf : p); q <= q_hi; ++q)
                        mbar_wait(&S.bar[slot_of(q)], parity_of(q));
                }
                return;
            }
            // stimuli of the first sub-step on the input rows (block p, and
            // at the first phase block p0 - 1), before level 1 reads them
            if (stim_on & 1u) {
                for (int q = (p == p0 ? qf : p); q <= p && q <= ql; ++q) {
                    const int i = q * BR + 1 + r;
                    if ((unsigned)i < (unsigned)f.ni && col_in) {
                        const int ir = irow(i);
                        if (S.myo[ir][c + xo8]) {
                            for (int si = 0; si < f.n_stims; ++si) {
                                const FStim &F = f.stims[si];
                                if (!(F.on & 1u)) continue;
                                if (gj < F.lo1 || gj >= F.hi1 || i < F.lo0 || i >= F.hi0)
                                    continue;
                                if (F.mask && !F.mask[(int64_t)i * f.nj + gj]) continue;
                                float x = S.u0[ir][c + xo];
                                if (F.kind == FW_STIM_VOLTAGE) {
                                    x = F.value;
                                } else {
                                    x = x + F.value;
                                    if (F.has_umax && x > F.u_max) x = F.u_max;
                                }
                                S.u0[ir][c + xo] = x;
                            }
                        }
                    }
                }
                __syncthreads();
            }

            // every level advances its node in every phase: levels outside
            // their blocks p0 .. bend (the march's first and last phases)
            // compute rows no written node depends on, and write only their
            // own rings, so the levels need no branches and interleave
#pragma unroll
            for (int s = 1; s <= KMAX; ++s) {
                const int i = i_s[s], ir = ir_s[s], lr = lr_s[s];
                const bool row_in = (unsigned)i < (unsigned)f.ni;
                const bool myo = row_in && col_in && S.myo[ir][c + xo8] != 0;
                const bool upd = myo && col_upd;
                const bool own = col_own && (unsigned)(i - R0) < (unsigned)(R1 - R0);
                // window of level s - 1 (input rows for s = 1)
                const float *row0, *row1, *row2;
                if (s == 1) {
                    row0 = &S.u0[ir == 0 ? RI - 1 : ir - 1][0];
                    row1 = &S.u0[ir][0];
                    row2 = &S.u0[ir == RI - 1 ? 0 : ir + 1][0];
                } else {
                    float(*ring)[kBoxF] = S.ul[s - 2 < 0 ? 0 : s - 2];
                    row0 = &ring[lr >= 2 ? lr - 2 : lr + RL - 2][0];
                    row1 = &ring[lr >= 1 ? lr - 1 : lr + RL - 1][0];
                    row2 = &ring[lr][0];
                }
                const int cx = c + xo;
                const float ul = row0[cx - 1], uc = row0[cx], ur = row0[cx + 1];
                const float ml = row1[cx - 1], b1 = row1[cx], mr = row1[cx + 1];
                const float dl = row2[cx - 1], dc = row2[cx], dr = row2[cx + 1];
                // the node's state entering level s
                typename M::template St<float> st;
                uint32_t bits;
                if (s == 1) {
                    float sv[kMaxTmaState];
#pragma unroll
                    for (int q2 = 0; q2 < NS; ++q2) sv[q2] = S.s0[q2][ir][cx];
                    st = M::template from_array<float>(sv);
                    bits = (lat && own && S.act[ir][c + xo8]) ? 1u : 0u;
                } else {
                    st = st_in[s];
                    bits = (bits_in >> (4 * s)) & 15u;
                }
                const int64_t n = n0 + s - 1;
                if (own) {
#pragma unroll
                    for (int a = 0; a < kMaxFusedAt; ++a) {
                        if (!((at_on[a] >> (s - 1)) & 1u)) continue;
                        // first crossing: unsigned minimum, "never" = -1
                        // (activation_time_2d_tracker.py:61-63)
                        if (b1 > at_thr[a] && !((bits >> (1 + a)) & 1u)) {
                            atomicMin(reinterpret_cast<unsigned *>(f.at[a].act) +
                                          (int64_t)i * f.nj + gj,
                                      (unsigned)n);
                            bits |= 1u << (1 + a);
                        }
                    }
                    if ((lat_on[0] >> (s - 1)) & 1u) {
                        // (local_activation_time_2d_tracker.py:71-89)
                        const bool was = bits & 1u;
                        if (!was && b1 >= lat_thr[0]) {
                            bits |= 1u;
                            lat_record(f.lat[0], (int64_t)i * f.nj + gj, f.n, n, f.status);
                        } else if (was && b1 < lat_thr[0]) {
                            bits &= ~1u;
                        }
                    }
                }
                const float4 wa = S.wa[ir][c];
                float4 wb = wa;
                if constexpr (NWO == 8) wb = S.wb[ir][c];
                const float un = stencil_fma<ST>(S.wc[ir][cx], b1, wa, wb, ul, uc, ur, ml,
                                                 mr, dl, dc, dr);
                const float uu = fused_update<M>(b1, un, st, P, dt);
                float out = upd ? uu : b1;
                if (s < KMAX) {
                    // stimuli of sub-step s + 1 on the value level s + 1 reads
                    if (((stim_on >> s) & 1u) && myo) {
                        for (int si = 0; si < f.n_stims; ++si) {
                            const FStim &F = f.stims[si];
                            if (!((F.on >> s) & 1u)) continue;
                            if (gj < F.lo1 || gj >= F.hi1 || i < F.lo0 || i >= F.hi0)
                                continue;
                            if (F.mask && !F.mask[(int64_t)i * f.nj + gj]) continue;
                            if (F.kind == FW_STIM_VOLTAGE) {
                                out = F.value;
                            } else {
                                out = out + F.value;
                                if (F.has_umax && out > F.u_max) out = F.u_max;
                            }
                        }
                    }
                    S.ul[s - 1 < KMAX - 1 ? s - 1 : 0][lr][cx] = out;
                    st_out[s] = st;
                    bits_out = (bits_out & ~(15u << (4 * s))) | ((bits & 15u) << (4 * s));
                }
                if (s == ksteps && own) {
                    // the launch's last sub-step: write the node back
                    const int64_t pp = (int64_t)i * f.pitch + gj;
                    if (myo) {
                        const float uo = upd ? uu : b1;
                        f.u_out[pp] = uo;
                        nonfinite |= !isfinite(uo);
                        M::template store<float>(f.state_out, pp, st);
                    }
                    if (lat && ((bits & 1u) != (S.act[ir][c + xo8] != 0 ? 1u : 0u)))
                        f.lat[0].activated[pp] = bits & 1u;
                }
            }
            __syncthreads();
            // hand each node's state and flags to the next level: one phase
            // later, or two where this thread's transition waits (gap2); every
            // level moves one block down
#pragma unroll
            for (int s = 1; s < KMAX; ++s) {
                const bool g2 = (gap2 >> s) & 1u;
                st_in[s + 1] = g2 ? st_hold[s] : st_out[s];
                st_hold[s] = st_out[s];
                const uint32_t m = 15u << (4 * s);
                const uint32_t from = g2 ? bits_hold : bits_out;
                bits_in = (bits_in & ~(m << 4)) | ((from & m) << 4);
            }
            bits_hold = bits_out;
#pragma unroll
            for (int s = 1; s <= KMAX; ++s) {
                i_s[s] += BR;
                ir_s[s] = ir_s[s] + BR >= RI ? ir_s[s] + BR - RI : ir_s[s] + BR;
                lr_s[s] = lr_s[s] + BR >= RL ? lr_s[s] + BR - RL : lr_s[s] + BR;
            }
        }
        if (nonfinite && f.status) atomicOr(f.status, FW_DEV_NONFINITE);
        g0 += ql - qf + 1;
        __syncthreads();
    }
}


// ---- host side -------------------------------------------------------------------

template <class M, int ST, int KMAX>
int launch_fused_march(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                       cudaStream_t stream)
{
    constexpr int NWO = Stencil2D<ST>::NWO;
    constexpr int BR = kMBR;
    constexpr size_t SMEM = sizeof(MarchSmem<M::NS, NWO, KMAX>) + 1024;
    static_assert(SMEM <= 232448, "the march kernel's rings exceed 227 KB");
    auto kern = k_fused_march<M, ST, KMAX>;
    FW_CUDA_CHECK(cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM));
    if (a->n_probe > 0) {
        set_error("fw_step (fused variant 7): probe trackers need another "
                  "fused variant");
        return FW_ERR_UNSUPPORTED;
    }
    if (a->n_lat > kMaxFusedLat) {
        set_error("fw_step (fused): at most %d local activation tracker",
                  kMaxFusedLat);
        return FW_ERR_UNSUPPORTED;
    }
    MarchK mk;  // kernel argument, copied at each launch
    memset(&mk, 0, sizeof mk);
    TmaK &k = mk.t;
    k.force_timeout = (a->debug_flags & FW_DEBUG_FORCE_TIMEOUT) ? 1 : 0;
    bool ok = encode_weights(&k.maps.w, a->weights_packed, NWO, a->nj, a->ni, BR) &&
              encode_2d(&k.maps.myo, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, a->myo, a->nj,
                        a->ni, kBoxB, BR) &&
              encode_2d(&k.maps.u[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a->u[0],
                        a->nj, a->ni, kBoxF, BR) &&
              encode_2d(&k.maps.u[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a->u[1],
                        a->nj, a->ni, kBoxF, BR);
    for (int q = 0; q < M::NS && ok; ++q)
        ok = encode_2d(&k.maps.s[0][q], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                       a->state[q], a->nj, a->ni, kBoxF, BR) &&
             encode_2d(&k.maps.s[1][q], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                       a->state_b[q], a->nj, a->ni, kBoxF, BR);
    if (ok) {
        const float *wcen_plane = (const float *)a->weights +
                                  (int64_t)Stencil2D<ST>::CENTRE * a->ni * a->nj;
        ok = encode_2d(&k.maps.wc, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, wcen_plane,
                       a->nj, a->ni, kBoxF, BR);
    }
    if (ok && a->n_lat > 0)
        ok = encode_2d(&k.maps.act, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1,
                       a->lat[0].activated, a->nj, a->ni, kBoxB, BR);
    if (!ok) {
        set_error("fw_step (fused march): tensor map encoding failed");
        return FW_ERR_UNSUPPORTED;
    }
    FusedK &f = k.f;
    f.w = nullptr;
    f.myo = a->myo;
    void *const *sbuf[2] = {a->state, a->state_b};
    for (int i = 0; i < FW_MAX_PARAMS; ++i) f.params[i] = (float)a->params[i];
    f.dt = (float)a->dt;
    f.ni = (int32_t)a->ni;
    f.nj = (int32_t)a->nj;
    f.n = a->ni * a->nj;
    f.pitch = (int32_t)a->nj;
    f.status = a->status;
    mk.strips = (int32_t)((a->nj + (kTW - 2 * KMAX) - 1) / (kTW - 2 * KMAX));
    mk.segs = (int32_t)((a->ni + kMarchSeg - 1) / kMarchSeg);
    f.tiles_j = mk.strips;
    const int64_t items = (int64_t)mk.strips * mk.segs;
    if (items > INT32_MAX) {
        set_error("fw_step (fused march): grid too large");
        return FW_ERR_ARG;
    }
    k.tiles = (int32_t)items;
    int sms = sm_count();
    if (sms <= 0) sms = 152;
    const int grid = k.tiles < sms ? k.tiles : sms;
    int64_t probe_samples[FW_MAX_PROBE] = {0};

    int64_t L = (n_steps + KMAX - 1) / KMAX;
    if ((L & 1) != (n_steps & 1)) ++L;
    int64_t done = 0;
    for (int64_t li = 0; li < L; ++li) {
        const int64_t left = n_steps - done, launches_left = L - li;
        int64_t ks = (left + launches_left - 1) / launches_left;
        if (ks > KMAX) ks = KMAX;
        const int64_t n0 = n_begin + done;
        const int64_t n1 = n0 + ks - 1;
        f.n0 = n0;
        f.ksteps = (int32_t)ks;
        k.in_buf = (int32_t)(li & 1);
        f.u_in = (const float *)a->u[li & 1];
        f.u_out = (float *)a->u[(li + 1) & 1];
        for (int q = 0; q < FW_MAX_FUSED_STATE; ++q) {
            f.state[q] = sbuf[li & 1][q];
            f.state_out[q] = sbuf[(li + 1) & 1][q];
        }
        int rc = fill_events(a, f, n0, n1, ks, probe_samples);
        if (rc) return rc;
        kern<<<grid, kMNT, SMEM, stream>>>(mk);
        FW_CHECK_LAUNCH("k_fused_march");
        done += ks;
    }
    return FW_OK;
}

}  // namespace fused
}  // namespace fw
