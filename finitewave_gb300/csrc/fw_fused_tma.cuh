// fw_fused_tma.cuh -- the fused FP32 2D step with a TMA pipeline.
//
// Same per-tile algorithm as fw_fused_kernel.cuh (temporal blocking of up to
// KMAX steps on a 64 x LH region, halo recomputed), organised for Blackwell:
//   * one persistent CTA per SM walks the tiles (tile, tile + gridDim.x, ...);
//   * its region is staged by the Tensor Memory Accelerator:
//     cp.async.bulk.tensor copies (packed weights, potential, state,
//     myocyte flags) that complete on an mbarrier;
//   * two stages: while the CTA computes tile i from one stage, the TMA
//     fills the other with tile i + 1, so HBM traffic overlaps compute; the
//     copies of tile i + 1 are issued right after the wait for tile i's,
//     by one lane each of warps 0, 1 and 2 (k_fused_tma), so that the other
//     warps start on tile i meanwhile.
// Every wait on an mbarrier is bounded; a timeout sets FW_DEV_TIMEOUT in the
// status word and the CTA returns once its copies in flight have landed
// (again a bounded wait).  The sub-steps form the diffusion sum as
// w_c u + sum_k w_k u_k  in one FMA chain (stencil_fma, shared with the
// cp.async and batched kernels), with the centre weight w_c staged from the
// weights' own centre plane beside the packed off-centre weights (9 FMA per
// node and sub-step instead of 17 operations for  u + sum_k w_k (u_k - u)).
//
// Layout requirements (checked by the host): nj % 16 == 0 (TMA row strides
// and the int8 myocyte rows) and the packed weight array of fw_pack_weights.
// Boxes start at 16-byte aligned x coordinates (x rounded down, the data is
// addressed at an offset inside the box), negative and past-the-end
// coordinates read zeros.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include "fw_fused_kernel.cuh"

namespace fw {
namespace fused {

constexpr int kTW = 64;    // region width (nodes)
constexpr int kBoxF = 72;  // f32 box width: columns oj - 1 .. oj + 64 from a 4-aligned start
constexpr int kBoxB = 80;  // int8 box width: columns oj .. oj + 63 from a 16-aligned start
constexpr int kMaxTmaState = 2;
// f32 box width of the float32 fiber pairs (weights formed on chip): the
// region's 64 columns, two floats each, from a 16-byte aligned start
constexpr int kBoxFib = 132;

template <int LH, int NS, int NWO>
struct TmaStage {
    alignas(128) float4 wa[LH][kTW];                   // weights 0..3
    alignas(128) float4 wb[NWO == 8 ? LH : 1][kTW];    // weights 4..7
    alignas(128) float u[LH + 2][kBoxF];               // rows oi - 1 .. oi + LH
    alignas(128) float s[NS][LH][kBoxF];               // rows oi .. oi + LH - 1
    alignas(128) int8_t myo[LH][kBoxB];
    alignas(128) float wc[LH][kBoxF];                  // centre weights, rows oi ..
    alignas(128) uint8_t act[LH][kBoxB];               // local activation flags
};

template <int LH, int NS, int NWO>
struct TmaSmem {
    TmaStage<LH, NS, NWO> stage[2];
    alignas(128) float u1[LH + 2][kBoxF];              // ping-pong partner
    uint32_t probe_bits[(LH * kTW + 31) / 32];
    ProbeEntry probe_list[kMaxFusedProbeEntries];
    int probe_count;
    alignas(8) uint64_t bar[2];
};

struct TmaMaps {
    CUtensorMap w;      // packed weights: dims (NWO, nj, ni)
    CUtensorMap myo;    // int8 (nj, ni)
    CUtensorMap u[2];   // f32 (nj, ni), the two potential buffers
    CUtensorMap s[2][kMaxTmaState];  // the state arrays, both buffers
    CUtensorMap wc;     // the centre weight plane, f32 (nj, ni)
    CUtensorMap act;    // the local activation tracker's flags, u8 (nj, ni)
    CUtensorMap fib;    // float32 fiber pairs, f32 (2 nj, ni) (weights on chip)
};
static_assert(kMaxFusedLat == 1, "one tensor map of local activation flags");

struct TmaK {
    TmaMaps maps;
    FusedK f;
    int32_t in_buf;     // potential buffer holding step n0
    int32_t tiles;
    int32_t force_timeout;  // testing: report every wait as timed out after
                            // its copy has arrived (FW_DEBUG_FORCE_TIMEOUT)
};

// ---- PTX wrappers ------------------------------------------------------------

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)),
                 "r"(count));
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile(
        "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;\n" ::"r"(
            smem_u32(bar)),
        "r"(bytes)
        : "memory");
}

// Bounded wait for phase `parity` of the barrier; false on timeout.  Each
// try_wait suspends for at most ~1 us (the hint), so the bound is ~2 s.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    const unsigned a = smem_u32(bar);
    for (int i = 0; i < (1 << 21); ++i) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n"
            " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity), "r"(1000)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_2d(void *dst, const CUtensorMap *map, int x,
                                       int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::"
        "bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_3d(void *dst, const CUtensorMap *map, int x,
                                       int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::"
        "bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_4d(void *dst, const CUtensorMap *map, int x,
                                       int y, int z, int w, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::"
        "bytes [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
        : "memory");
}

// A CTA giving up on its pipeline: set FW_DEV_TIMEOUT, then wait (bounded)
// for the bulk copies it still has in flight -- the one into stage sg when
// its wait did not see it arrive, and the prefetch into the other stage when
// one was issued -- so that no copy lands in shared memory after the CTA
// has exited.  Called by thread 0 only.
template <class TK>
__device__ __noinline__ void tma_abandon(const TK &k, uint64_t *bar, int sg,
                                         unsigned ph, unsigned parity,
                                         bool arrived, int next)
{
    if (k.f.status) atomicOr(k.f.status, FW_DEV_TIMEOUT);
    if (!arrived) mbar_wait(&bar[sg], ph);
    if (next < k.tiles) mbar_wait(&bar[sg ^ 1], (parity >> (sg ^ 1)) & 1u);
}

__device__ __forceinline__ int floor_to(int x, int m)
{
    return x >= 0 ? x - x % m : -((-x + m - 1) / m) * m;
}

// ---- kernel ----------------------------------------------------------------------

// Copy one tile's region into a stage: packed weights, potential, the
// model's NS state arrays, myocyte flags and centre weights, all completing
// on `bar`.  NS and NWO are the model's and the stencil's; the stage may be
// laid out for more (the batched kernel's stages hold the largest model).
// PAIRS: the weight map is the column-pair view of encode_weights_pairs, and
// the weights land as [row][column parity][column pair] (k_fused_tma2).
// `lat`: also the local activation tracker's flags (maps.act).
// The barrier has an arrival count of one: this is the stage's only
// arrive, and it announces the region's bytes plus `extra` bytes of other
// copies the caller issues on the same barrier.
// FLY: instead of the weights, the region's float32 fiber pairs (into the
// stage's wb area, from which the tile forms its weights on chip).
template <int KMAX, int NS, int NWO, bool PAIRS = false, bool FLY = false, class Stage>
__device__ __forceinline__ void issue_region(const TmaMaps &maps, int in_buf,
                                             Stage &G, uint64_t *bar, int oi,
                                             int oj, unsigned extra = 0,
                                             bool lat = false)
{
    const int x4 = floor_to(oj - 1, 4), x16 = floor_to(oj, 16);
    if constexpr (FLY) {
        constexpr int kRows = (int)(sizeof(G.myo) / sizeof(G.myo[0]));
        constexpr unsigned kFib = (unsigned)(kRows * kBoxFib * sizeof(float));
        static_assert(NWO == 8 && sizeof(G.wb) >= kFib, "fiber box in the wb area");
        const unsigned bytes = (unsigned)(sizeof(G.u) + NS * sizeof(G.s[0]) +
                                          sizeof(G.myo)) +
                               kFib + (lat ? (unsigned)sizeof(G.act) : 0u);
        mbar_expect_tx(bar, bytes + extra);
        if (lat) tma_2d(&G.act[0][0], &maps.act, x16, oi, bar);
        tma_2d(&G.wb[0][0], &maps.fib, floor_to(2 * oj, 4), oi, bar);
        tma_2d(&G.u[0][0], &maps.u[in_buf], x4, oi - 1, bar);
#pragma unroll
        for (int q = 0; q < NS; ++q)
            tma_2d(&G.s[q][0][0], &maps.s[in_buf][q], x4, oi, bar);
        tma_2d(&G.myo[0][0], &maps.myo, x16, oi, bar);
        return;
    }
    const unsigned bytes = (unsigned)(sizeof(G.wa) * (NWO == 8 ? 2 : 1) +
                                      sizeof(G.u) + NS * sizeof(G.s[0]) +
                                      sizeof(G.myo) + sizeof(G.wc)) +
                           (lat ? (unsigned)sizeof(G.act) : 0u);
    mbar_expect_tx(bar, bytes + extra);
    if (lat) tma_2d(&G.act[0][0], &maps.act, x16, oi, bar);
    if constexpr (PAIRS) {
        tma_4d(&G.wa[0][0], &maps.w, 0, oj / 2, 0, oi, bar);
        if constexpr (NWO == 8) tma_4d(&G.wb[0][0], &maps.w, 4, oj / 2, 0, oi, bar);
    } else {
        tma_3d(&G.wa[0][0], &maps.w, 0, oj, oi, bar);
        if constexpr (NWO == 8) tma_3d(&G.wb[0][0], &maps.w, 4, oj, oi, bar);
    }
    tma_2d(&G.u[0][0], &maps.u[in_buf], x4, oi - 1, bar);
#pragma unroll
    for (int q = 0; q < NS; ++q)
        tma_2d(&G.s[q][0][0], &maps.s[in_buf][q], x4, oi, bar);
    tma_2d(&G.myo[0][0], &maps.myo, x16, oi, bar);
    tma_2d(&G.wc[0][0], &maps.wc, x4, oi, bar);
}

template <int KMAX, int LH, int NS, int NWO, bool PAIRS = false, bool FLY = false>
__device__ __forceinline__ void issue_tile(const TmaK &k, TmaStage<LH, NS, NWO> &G,
                                           uint64_t *bar, int bi, int bj)
{
    constexpr int TI = LH - 2 * KMAX, TJ = kTW - 2 * KMAX;
    issue_region<KMAX, NS, NWO, PAIRS, FLY>(k.maps, k.in_buf, G, bar,
                                            bi * TI - KMAX, bj * TJ - KMAX, 0u,
                                            k.f.n_lat > 0);
}

// issue_tile's copies (stored weights, strip layout) spread over the first
// lanes of warps 0, 1 and 2 (tid 0, 32, 64), so that no single warp carries
// the whole issue into the tile's first sub-step: tid 0 announces the
// stage's bytes (the barrier's one arrival) and copies the weights, tid 32
// the potential and the state, tid 64 the flags and the centre weights.
// Copies may complete before the announcement: the phase cannot end before
// the arrival, which carries the full byte count.
template <int KMAX, int LH, int NS, int NWO>
__device__ __forceinline__ void issue_tile_split(const TmaK &k,
                                                 TmaStage<LH, NS, NWO> &G,
                                                 uint64_t *bar, int bi, int bj,
                                                 int tid)
{
    constexpr int TI = LH - 2 * KMAX, TJ = kTW - 2 * KMAX;
    if (tid != 0 && tid != 32 && tid != 64) return;
    fence_proxy_async();
    const int oi = bi * TI - KMAX, oj = bj * TJ - KMAX;
    const int x4 = floor_to(oj - 1, 4), x16 = floor_to(oj, 16);
    const bool lat = k.f.n_lat > 0;
    if (tid == 0) {
        const unsigned bytes = (unsigned)(sizeof(G.wa) * (NWO == 8 ? 2 : 1) +
                                          sizeof(G.u) + NS * sizeof(G.s[0]) +
                                          sizeof(G.myo) + sizeof(G.wc)) +
                               (lat ? (unsigned)sizeof(G.act) : 0u);
        mbar_expect_tx(bar, bytes);
        tma_3d(&G.wa[0][0], &k.maps.w, 0, oj, oi, bar);
        if constexpr (NWO == 8) tma_3d(&G.wb[0][0], &k.maps.w, 4, oj, oi, bar);
    } else if (tid == 32) {
        tma_2d(&G.u[0][0], &k.maps.u[k.in_buf], x4, oi - 1, bar);
#pragma unroll
        for (int q = 0; q < NS; ++q)
            tma_2d(&G.s[q][0][0], &k.maps.s[k.in_buf][q], x4, oi, bar);
    } else {
        tma_2d(&G.myo[0][0], &k.maps.myo, x16, oi, bar);
        tma_2d(&G.wc[0][0], &k.maps.wc, x4, oi, bar);
        if (lat) tma_2d(&G.act[0][0], &k.maps.act, x16, oi, bar);
    }
}

// minor_component (asymmetric_stencil_2d.py:204-259) in float32.
__device__ __forceinline__ void minor_f32(float d, int m0, int m1, int m2, int m3,
                                          int m4, int m5, float r[6])
{
    const int mh = m2 + m3 + m4 + m5, ml = m0 + m1 + m2 + m3;
    if (m2 == 0 || m3 == 0 || mh < 3 || ml < 3) {
        r[0] = r[1] = r[2] = r[3] = r[4] = r[5] = 0.f;
        return;
    }
    const float dh = (float)mh, dl = (float)ml;
    r[0] = (-d) * (float)m0 / dl;
    r[1] = (-d) * (float)m1 / dl;
    r[2] = d * ((float)m2 / dh - (float)m2 / dl);
    r[3] = d * ((float)m3 / dh - (float)m3 / dl);
    r[4] = d * (float)m4 / dh;
    r[5] = d * (float)m5 / dh;
}

// The region's AsymmetricStencil2D weights formed on chip (fused_variant 5)
// from the staged float32 fiber pairs (in the stage's wb area) and myocyte
// flags: the reference's four face fluxes, each a major and a six-point
// minor component, accumulated in its order (asymmetric_stencil_2d.py:
// 291-433), the half-step diffusion components 0.5 (D c + D' c) over a node
// and its +1 neighbour (:104-136), then scaled by D_model dt / dr**2 with 1
// added to the centre (:46-84) -- all in float32, so within float32
// rounding of the stored weights (built in float64).  Weights are formed
// for the myocytes off the region's outer ring (no other node's weights are
// read) and written where the TMA form stages them: w0..w3 into wa, w5..w8
// into wb once every thread has read its fibers, the centre into wc.
template <int LH, int R, class Stage>
__device__ __forceinline__ void fly_weights(const FusedK &f, Stage &G, int r0,
                                            int col, int oj, int xo, int xo8)
{
    const float *fb = reinterpret_cast<const float *>(&G.wb[0][0]);
    const int xf = 2 * oj - floor_to(2 * oj, 4);
    const float dal = f.fly_dal, dac = f.fly_dac, cnd = f.fly_cond;
    const float sc = f.fly_scale;
    auto M = [&](int lr, int c) -> int { return G.myo[lr][c + xo8] != 0; };
    // D_ac (a0 == a1) + (D_al - D_ac) f_a0 f_a1 at region node (lr, c)
    auto D = [&](int lr, int c, int a0, int a1) -> float {
        const float *fp = fb + lr * kBoxFib + 2 * c + xf;
        return (a0 == a1 ? dac : 0.f) + (dal - dac) * fp[a0] * fp[a1];
    };
    auto H = [&](int lr, int c, int ax, int comp) -> float {
        return 0.5f * (D(lr, c, ax, comp) * cnd +
                       D(lr + (ax == 0), c + (ax == 1), ax, comp) * cnd);
    };
    float4 wb_out[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int lr = r0 + r, c = col;
        float o[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (lr >= 1 && lr <= LH - 2 && c >= 1 && c <= kTW - 2 && M(lr, c)) {
            float m[6], q;
            // q (i-1/2, j)
            q = H(lr - 1, c, 0, 0) * (float)M(lr - 1, c);
            o[1] += q; o[4] -= q;
            minor_f32(H(lr - 1, c, 0, 1), M(lr - 1, c - 1), M(lr, c - 1), M(lr - 1, c),
                      M(lr, c), M(lr - 1, c + 1), M(lr, c + 1), m);
            o[0] -= m[0]; o[3] -= m[1]; o[1] -= m[2];
            o[4] -= m[3]; o[2] -= m[4]; o[5] -= m[5];
            // q (i, j-1/2)
            q = H(lr, c - 1, 1, 1) * (float)M(lr, c - 1);
            o[3] += q; o[4] -= q;
            minor_f32(H(lr, c - 1, 1, 0), M(lr - 1, c - 1), M(lr - 1, c), M(lr, c - 1),
                      M(lr, c), M(lr + 1, c - 1), M(lr + 1, c), m);
            o[0] -= m[0]; o[1] -= m[1]; o[3] -= m[2];
            o[4] -= m[3]; o[6] -= m[4]; o[7] -= m[5];
            // q (i, j+1/2)
            q = H(lr, c, 1, 1) * (float)M(lr, c + 1);
            o[5] += q; o[4] -= q;
            minor_f32(H(lr, c, 1, 0), M(lr - 1, c + 1), M(lr - 1, c), M(lr, c + 1),
                      M(lr, c), M(lr + 1, c + 1), M(lr + 1, c), m);
            o[2] += m[0]; o[1] += m[1]; o[5] += m[2];
            o[4] += m[3]; o[8] += m[4]; o[7] += m[5];
            // q (i+1/2, j)
            q = H(lr, c, 0, 0) * (float)M(lr + 1, c);
            o[7] += q; o[4] -= q;
            minor_f32(H(lr, c, 0, 1), M(lr + 1, c - 1), M(lr, c - 1), M(lr + 1, c),
                      M(lr, c), M(lr + 1, c + 1), M(lr, c + 1), m);
            o[6] += m[0]; o[3] += m[1]; o[7] += m[2];
            o[4] += m[3]; o[8] += m[4]; o[5] += m[5];
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) o[k] *= sc;
        o[4] += 1.f;
        G.wa[lr][col] = make_float4(o[0], o[1], o[2], o[3]);
        G.wc[lr][col + xo] = o[4];
        wb_out[r] = make_float4(o[5], o[6], o[7], o[8]);
    }
    __syncthreads();  // the fibers in the wb area have been read
#pragma unroll
    for (int r = 0; r < R; ++r) G.wb[r0 + r][col] = wb_out[r];
    __syncthreads();
}

// Rows r < R of the strip of thread (col, r0) inside the region's interior
// (own) and off its outer ring (ring): the same for every tile.
template <int KMAX, int LH, int R>
__device__ __forceinline__ void strip_masks(int col, int r0, uint32_t &own_c,
                                            uint32_t &ring_c)
{
    constexpr int TI = LH - 2 * KMAX, TJ = kTW - 2 * KMAX;
    own_c = ring_c = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int lr = r0 + r;
        if (col >= KMAX && col < KMAX + TJ && lr >= KMAX && lr < KMAX + TI)
            own_c |= 1u << r;
        if (col > 0 && col < kTW - 1 && lr > 0 && lr < LH - 1) ring_c |= 1u << r;
    }
}

// One staged tile: K sub-steps of the region with origin (oi, oj) from
// stage G, then the interior written back.  f describes the tissue and the
// launch (its u_out, state and myocyte arrays have row pitch f.pitch; the
// tracker arrays and stimulus masks row length f.nj).  u1 is the ping-pong
// partner of the stage's potential.  Thread (col, r0) owns the strip of R
// rows of column col.  Shared by the single-tissue and the batched kernels.
template <class M, int ST, int KMAX, int LH, int R, bool FLY = false, class Stage,
          class Sm>
__device__ __forceinline__ void tma_tile(const FusedK &f, Stage &G, Sm &S, int oi,
                                         int oj, uint32_t own_c, uint32_t ring_c,
                                         const Params<float, M::NP> &P)
{
    constexpr int LW = kTW;
    constexpr int NT = LW * (LH / R);
    constexpr int TI = LH - 2 * KMAX, TJ = LW - 2 * KMAX;
    constexpr int NS = M::NS;
    constexpr int NWO = Stencil2D<ST>::NWO;
    const int tid = threadIdx.x;
    const int col = tid % LW;
    const int r0 = (tid / LW) * R;
    const float dt = f.dt;

    const int xo = oj - floor_to(oj - 1, 4);   // 1..4
    const int xo8 = oj - floor_to(oj, 16);     // 0..15
    const int gj = oj + col;
    const bool col_in = (unsigned)gj < (unsigned)f.nj;
    if constexpr (FLY) fly_weights<LH, R>(f, G, r0, col, oj, xo, xo8);

    // per-thread flags and state of the strip
    typename M::template St<float> st[R];
    uint32_t myo_bits = 0, inb = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int lr = r0 + r;
        if (col_in && (unsigned)(oi + lr) < (unsigned)f.ni) inb |= 1u << r;
        if (G.myo[lr][col + xo8]) myo_bits |= 1u << r;
        float sv[kMaxTmaState];
#pragma unroll
        for (int q = 0; q < NS; ++q) sv[q] = G.s[q][lr][col + xo];
        st[r] = M::template from_array<float>(sv);
    }
    myo_bits &= inb;
    const uint32_t own = own_c & inb;
    const uint32_t upd = ring_c & myo_bits;
    // centre weights of the strip (the stored plane); the sub-steps form
    // the reference's sum  w_c u + sum_k w_k u_k  as one FMA chain
    float wcen[R];
    float4 wreg[R];   // the first four off-centre weights, kept for the tile
#pragma unroll
    for (int r = 0; r < R; ++r) {
        wcen[r] = G.wc[r0 + r][col + xo];
        wreg[r] = G.wa[r0 + r][col];
    }

    // probe cells of this tile
    uint32_t probe_mine = 0;
    if (f.n_probe) {
        for (int i = tid; i < (LH * LW + 31) / 32; i += NT) S.probe_bits[i] = 0;
        if (tid == 0) S.probe_count = 0;
        __syncthreads();
        for (int t = 0; t < f.n_probe; ++t) {
            const FProbe &pr = f.probe[t];
            for (int c = tid; c < pr.n_cells; c += NT) {
                const int64_t p = pr.cells[c];
                const int gi = (int)(p / f.nj), gjj = (int)(p % f.nj);
                const int lr = gi - oi, lc = gjj - oj;
                if (lr >= KMAX && lr < KMAX + TI && lc >= KMAX &&
                    lc < KMAX + TJ) {
                    const int e = atomicAdd(&S.probe_count, 1);
                    if (e < kMaxFusedProbeEntries) {
                        S.probe_list[e] = ProbeEntry{(int16_t)lr, (int16_t)lc,
                                                     (int16_t)t, c};
                        const int bit = lr * LW + lc;
                        atomicOr(&S.probe_bits[bit >> 5], 1u << (bit & 31));
                    } else if (f.status) {
                        atomicOr(f.status, FW_DEV_PROBE_OVERFLOW);
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
    // the local activation flags of the strip, staged with the region
    uint32_t lat_act = 0, at_done = 0;
    if (f.n_lat) {
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (((own >> r) & 1u) && G.act[r0 + r][col + xo8]) lat_act |= 1u << r;
    }
    const uint32_t lat_act0 = lat_act;

    // the launch's per-sub-step controls, read once per tile (the batched
    // kernel keeps its launch description in shared memory)
    const int ksteps = f.ksteps;
    const int64_t n0 = f.n0;
    const uint32_t stim_on = f.stim_on, probe_on = f.probe_on;
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

    // ---- sub-steps ----
    for (int s = 0; s < ksteps; ++s) {
        const int64_t n = n0 + s;
        float(*cur)[kBoxF] = (s & 1) ? S.u1 : G.u;
        float(*nxt)[kBoxF] = (s & 1) ? G.u : S.u1;

        if ((stim_on >> s) & 1u) {
            for (int i = 0; i < f.n_stims; ++i) {
                const FStim &F = f.stims[i];
                if (!((F.on >> s) & 1u)) continue;
                if (gj < F.lo1 || gj >= F.hi1) continue;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (!((myo_bits >> r) & 1u)) continue;
                    const int lr = r0 + r, gi = oi + lr;
                    if (gi < F.lo0 || gi >= F.hi0) continue;
                    if (F.mask && !F.mask[(int64_t)gi * f.nj + gj]) continue;
                    float x = cur[lr + 1][col + xo];
                    if (F.kind == FW_STIM_VOLTAGE) {
                        x = F.value;
                    } else {
                        x = x + F.value;
                        if (F.has_umax && x > F.u_max) x = F.u_max;
                    }
                    cur[lr + 1][col + xo] = x;
                }
            }
            __syncthreads();
        }

        float wl[R + 2], wc[R + 2], wr[R + 2];
#pragma unroll
        for (int i = 0; i < R + 2; ++i) {
            wl[i] = cur[r0 + i][col + xo - 1];
            wc[i] = cur[r0 + i][col + xo];
            wr[i] = cur[r0 + i][col + xo + 1];
        }

        if (own) {
#pragma unroll
            for (int a = 0; a < kMaxFusedAt; ++a) {
                if (!((at_on[a] >> s) & 1u)) continue;
                // the strip's maximum first: most sub-steps cross nowhere
                // (fmaxf skips NaN rows, which never cross)
                float mx = wc[1];
#pragma unroll
                for (int r = 1; r < R; ++r) mx = fmaxf(mx, wc[r + 1]);
                if (!(mx > at_thr[a])) continue;
                const uint32_t hit =
                    rows_gt<R>(wc, at_thr[a]) & own & ~(at_done >> (a * 8));
                if (hit) {
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        if (!((hit >> r) & 1u)) continue;
                        // first crossing: unsigned minimum, "never" = -1
                        // (activation_time_2d_tracker.py:61-63)
                        const int64_t p = (int64_t)(oi + r0 + r) * f.nj + gj;
                        atomicMin(reinterpret_cast<unsigned *>(f.at[a].act) + p,
                                  (unsigned)n);
                    }
                    at_done |= hit << (a * 8);
                }
            }
#pragma unroll
            for (int l = 0; l < kMaxFusedLat; ++l) {
                if (!((lat_on[l] >> s) & 1u)) continue;
                // (local_activation_time_2d_tracker.py:71-89)
                const uint32_t was = (lat_act >> (l * 8)) & 0xffu;
                const uint32_t rise = rows_ge<R>(wc, lat_thr[l]) & own & ~was;
                const uint32_t fall = rows_lt<R>(wc, lat_thr[l]) & own & was;
                lat_act ^= (rise | fall) << (l * 8);
                if (rise) {
#pragma unroll
                    for (int r = 0; r < R; ++r)
                        if ((rise >> r) & 1u)
                            lat_record(f.lat[l],
                                       (int64_t)(oi + r0 + r) * f.nj + gj, f.n, n,
                                       f.status);
                }
            }
        }

#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float b1 = wc[r + 1];
            const int lr = r0 + r;
            const float4 wa = wreg[r];
            float4 wb = wa;
            if constexpr (NWO == 8) wb = G.wb[lr][col];
            const float un = stencil_fma<ST>(wcen[r], b1, wa, wb, wl[r], wc[r],
                                             wr[r], wl[r + 1], wr[r + 1],
                                             wl[r + 2], wc[r + 2], wr[r + 2]);
            const float uu = fused_update<M>(b1, un, st[r], P, dt);
            nxt[lr + 1][col + xo] = ((upd >> r) & 1u) ? uu : b1;
        }
        // probes: u after the stimuli, the state after the update
        if (probe_mine && ((probe_on >> s) & 1u)) {
#pragma unroll
            for (int r = 0; r < R; ++r)
                if ((probe_mine >> r) & 1u)
                    write_probes<M>(f, S.probe_list, S.probe_count, r0 + r, col,
                                    s, wc[r + 1], st[r],
                                    ((myo_bits >> r) & 1u) != 0,
                                    (int64_t)(oi + r0 + r) * f.pitch + gj);
        }
        __syncthreads();
    }

    // ---- write the interior back ----
    float(*fin)[kBoxF] = (ksteps & 1) ? S.u1 : G.u;
    bool nonfinite = false;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (!((own >> r) & 1u)) continue;
        const int lr = r0 + r;
        if ((myo_bits >> r) & 1u) {
            const int64_t pp = (int64_t)(oi + lr) * f.pitch + gj;
            const float uo = fin[lr + 1][col + xo];
            f.u_out[pp] = uo;
            nonfinite |= !isfinite(uo);
            M::template store<float>(f.state_out, pp, st[r]);
        }
        // the flags that changed in this launch (rows of f.pitch nodes)
        if (((lat_act ^ lat_act0) >> r) & 1u)
            f.lat[0].activated[(int64_t)(oi + lr) * f.pitch + gj] = (lat_act >> r) & 1u;
    }
    if (nonfinite && f.status) atomicOr(f.status, FW_DEV_NONFINITE);
}

template <class M, int ST, int KMAX, int LH, int R, bool FLY = false>
__global__ void __launch_bounds__(kTW *(LH / R), 1)
    k_fused_tma(const __grid_constant__ TmaK k)
{
    constexpr int LW = kTW;
    constexpr int TI = LH - 2 * KMAX, TJ = LW - 2 * KMAX;
    constexpr int NS = M::NS;
    constexpr int NWO = Stencil2D<ST>::NWO;
    static_assert(LH % R == 0 && R <= 8 && TI > 0 && TJ > 0, "tile shape");
    static_assert(NS <= kMaxTmaState, "state arrays");

    // TMA destinations are 128-byte aligned: round the dynamic shared window
    // up (the launch reserves 1 KB of slack for this)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned mis = smem_u32(smem_raw) & 127u;
    TmaSmem<LH, NS, NWO> &S = *reinterpret_cast<TmaSmem<LH, NS, NWO> *>(
        smem_raw + (mis ? 128u - mis : 0u));
    const FusedK &f = k.f;

    const int tid = threadIdx.x;
    uint32_t own_c, ring_c;
    strip_masks<KMAX, LH, R>(tid % LW, (tid / LW) * R, own_c, ring_c);

    if (tid == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    int tile = blockIdx.x;
    // tile = bi * tiles_j + bj, advanced by gridDim.x tiles per iteration
    // without an integer division in the loop
    const int tj = f.tiles_j;
    const int di = (int)gridDim.x / tj, dj = (int)gridDim.x % tj;
    int bi = tile / tj, bj = tile % tj;
    if (tid == 0 && tile < k.tiles)
        issue_tile<KMAX, LH, NS, NWO, false, FLY>(k, S.stage[0], &S.bar[0], bi, bj);

    Params<float, M::NP> P;
#pragma unroll
    for (int i = 0; i < M::NP; ++i) P.v[i] = f.params[i];
    unsigned parity = 0u;  // bit sg: phase parity expected next on bar[sg]

    for (int it = 0; tile < k.tiles; ++it, tile += gridDim.x) {
        const int sg = it & 1;
        TmaStage<LH, NS, NWO> &G = S.stage[sg];
        int ni_ = bi + di, nj_ = bj + dj;
        if (nj_ >= tj) {
            nj_ -= tj;
            ++ni_;
        }
        const unsigned ph = (parity >> sg) & 1u;
        const bool arrived = mbar_wait(&S.bar[sg], ph);
        parity ^= 1u << sg;
        if (__syncthreads_or(!arrived || k.force_timeout)) {
            // the next tile is issued after this point: only this stage's
            // copy can be in flight
            if (tid == 0) tma_abandon(k, S.bar, sg, ph, parity, arrived, k.tiles);
            return;
        }
        // prefetch the next tile into the other stage (its readers finished
        // at the barrier that closed the previous iteration); issued after
        // the wait, so the other warps start this tile meanwhile
        const int next = tile + gridDim.x;
        if (next < k.tiles) {
            if constexpr (FLY) {
                if (tid == 0) {
                    fence_proxy_async();
                    issue_tile<KMAX, LH, NS, NWO, false, FLY>(k, S.stage[sg ^ 1],
                                                              &S.bar[sg ^ 1], ni_, nj_);
                }
            } else {
                issue_tile_split<KMAX, LH, NS, NWO>(k, S.stage[sg ^ 1], &S.bar[sg ^ 1],
                                                    ni_, nj_, tid);
            }
        }
        const int oi = bi * TI - KMAX, oj = bj * TJ - KMAX;
        bi = ni_;
        bj = nj_;
        // no barrier here: the next iteration's wait ends in one, before any
        // thread touches the ping-pong rows or thread 0 refills this stage
        tma_tile<M, ST, KMAX, LH, R, FLY>(f, G, S, oi, oj, own_c, ring_c, P);
    }
}

// ---- column-pair kernel ----------------------------------------------------------
//
// The same tile pipeline as k_fused_tma with each thread on two adjacent
// columns and two rows (a 2 x 2 block of nodes) instead of one column and
// four rows: a row of the potential window is then one float2 load plus its
// two outer neighbours (3 loads for 2 nodes instead of 6), and the state,
// centre weights and updated potential move as float2.  The weights arrive
// from the column-pair view of the packed array (encode_weights_pairs) as
// [row][column parity][column pair], so the lanes of a warp read contiguous
// float4s.  Each node's arithmetic is k_fused_tma's, in the same order.
// Needs an even region origin (even KMAX), which makes the float2 offsets
// 8-byte aligned.
//
// PACK (fused variant 6): the two columns of a row advance together in
// Blackwell's two-wide float32 instructions (f2_fma, f2_mul, f2_add: one
// issue for both lanes, each lane rounded as the scalar instruction).  The
// block's weights are read from the stage once per tile into registers as
// (column c0, column c0 + 1) pairs; a sub-step forms a row's two diffusion
// sums as one chain of pair FMAs over the window pairs left = (c0 - 1, c0),
// centre = (c0, c0 + 1) and right = (c0 + 1, c0 + 2), and the ionic update
// in pair form where the model has one (M::update_pair).  The arithmetic
// instructions per node about halve; every node keeps k_fused_tma's bits.

// Nodes j = 2 r + h (row r0 + r, column c0 + h) of the block of thread
// (c0, r0) inside the region's interior (own) and off its outer ring (ring).
template <int KMAX, int LH>
__device__ __forceinline__ void pair_masks(int c0, int r0, uint32_t &own_c,
                                           uint32_t &ring_c)
{
    constexpr int TI = LH - 2 * KMAX, TJ = kTW - 2 * KMAX;
    own_c = ring_c = 0;
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int lr = r0 + r, lc = c0 + h, j = 2 * r + h;
            if (lc >= KMAX && lc < KMAX + TJ && lr >= KMAX && lr < KMAX + TI)
                own_c |= 1u << j;
            if (lc > 0 && lc < kTW - 1 && lr > 0 && lr < LH - 1) ring_c |= 1u << j;
        }
}

// One staged tile of the column-pair kernels (k_fused_tma2 and the batched
// pair kernel): K sub-steps of the region with origin (oi, oj) from stage G,
// then the interior written back.  As tma_tile: u_out, state and the local
// activation flags have row pitch f.pitch, the tracker arrays and stimulus
// masks row length f.nj; u1 is the ping-pong partner of the stage's
// potential.
template <class M, int ST, int KMAX, int LH, bool PACK, class Stage, class Sm>
__device__ __forceinline__ void tma_tile2(const FusedK &f, Stage &G, Sm &S, int oi,
                                          int oj, uint32_t own_c, uint32_t ring_c,
                                          const Params<float, M::NP> &P)
{
    constexpr int LW = kTW, HW = kTW / 2;   // columns, column pairs
    constexpr int R = 2;                     // rows per thread
    constexpr int NT = HW * (LH / R);
    constexpr int TI = LH - 2 * KMAX, TJ = LW - 2 * KMAX;
    constexpr int NS = M::NS;
    constexpr int NWO = Stencil2D<ST>::NWO;
    const int tid = threadIdx.x;
    const int cp = tid % HW;        // column pair
    const int c0 = 2 * cp;          // first of the thread's two columns
    const int r0 = (tid / HW) * R;
    const float dt = f.dt;

    const int xo = oj - floor_to(oj - 1, 4);   // 2 or 4 (oj is even)
    const int xo8 = oj - floor_to(oj, 16);     // 0..14, even
    const int gj0 = oj + c0;
    const int cx = c0 + xo;                    // float2-aligned window column

    typename M::template St<float> st[2 * R];
    uint32_t myo_bits = 0, inb = 0;
    float wcen[2 * R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int lr = r0 + r, gi = oi + lr;
        const bool row_in = (unsigned)gi < (unsigned)f.ni;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int j = 2 * r + h;
            if (row_in && (unsigned)(gj0 + h) < (unsigned)f.nj) inb |= 1u << j;
            if (G.myo[lr][c0 + h + xo8]) myo_bits |= 1u << j;
        }
        float sv0[kMaxTmaState], sv1[kMaxTmaState];
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            const float2 v2 = *reinterpret_cast<const float2 *>(&G.s[q][lr][cx]);
            sv0[q] = v2.x;
            sv1[q] = v2.y;
        }
        st[2 * r] = M::template from_array<float>(sv0);
        st[2 * r + 1] = M::template from_array<float>(sv1);
        const float2 w2 = *reinterpret_cast<const float2 *>(&G.wc[lr][cx]);
        wcen[2 * r] = w2.x;
        wcen[2 * r + 1] = w2.y;
    }
    myo_bits &= inb;
    const uint32_t own = own_c & inb;
    const uint32_t upd = ring_c & myo_bits;

    // PACK: the block's weights as (column c0, column c0 + 1) pairs, read
    // once for the tile
    float2 wp[PACK ? R : 1][PACK ? NWO : 1];
    float2 wcp[PACK ? R : 1];
    if constexpr (PACK) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int lr = r0 + r;
            const float4 a0 = G.wa[lr][cp], a1 = G.wa[lr][HW + cp];
            wp[r][0] = make_float2(a0.x, a1.x);
            wp[r][1] = make_float2(a0.y, a1.y);
            wp[r][2] = make_float2(a0.z, a1.z);
            wp[r][3] = make_float2(a0.w, a1.w);
            if constexpr (NWO == 8) {
                const float4 b0 = G.wb[lr][cp], b1 = G.wb[lr][HW + cp];
                wp[r][4] = make_float2(b0.x, b1.x);
                wp[r][5] = make_float2(b0.y, b1.y);
                wp[r][6] = make_float2(b0.z, b1.z);
                wp[r][7] = make_float2(b0.w, b1.w);
            }
            wcp[r] = make_float2(wcen[2 * r], wcen[2 * r + 1]);
        }
    }

    // probe cells of this tile
    uint32_t probe_mine = 0;
    if (f.n_probe) {
        for (int i = tid; i < (LH * LW + 31) / 32; i += NT) S.probe_bits[i] = 0;
        if (tid == 0) S.probe_count = 0;
        __syncthreads();
        for (int t = 0; t < f.n_probe; ++t) {
            const FProbe &pr = f.probe[t];
            for (int c = tid; c < pr.n_cells; c += NT) {
                const int64_t p = pr.cells[c];
                const int gi = (int)(p / f.nj), gjj = (int)(p % f.nj);
                const int lr = gi - oi, lc = gjj - oj;
                if (lr >= KMAX && lr < KMAX + TI && lc >= KMAX && lc < KMAX + TJ) {
                    const int e = atomicAdd(&S.probe_count, 1);
                    if (e < kMaxFusedProbeEntries) {
                        S.probe_list[e] = ProbeEntry{(int16_t)lr, (int16_t)lc,
                                                     (int16_t)t, c};
                        const int bit = lr * LW + lc;
                        atomicOr(&S.probe_bits[bit >> 5], 1u << (bit & 31));
                    } else if (f.status) {
                        atomicOr(f.status, FW_DEV_PROBE_OVERFLOW);
                    }
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 2 * R; ++j) {
            const int bit = (r0 + j / 2) * LW + c0 + (j & 1);
            if ((S.probe_bits[bit >> 5] >> (bit & 31)) & 1u) probe_mine |= 1u << j;
        }
    }
    // the local activation flags of the block, staged with the region
    uint32_t lat_act = 0, at_done = 0;
    if (f.n_lat) {
#pragma unroll
        for (int j = 0; j < 2 * R; ++j)
            if (((own >> j) & 1u) && G.act[r0 + j / 2][c0 + (j & 1) + xo8])
                lat_act |= 1u << j;
    }
    const uint32_t lat_act0 = lat_act;

    // the launch's per-sub-step controls, read once per tile
    const int ksteps = f.ksteps;
    const int64_t n0 = f.n0;
    const uint32_t stim_on = f.stim_on, probe_on = f.probe_on;
    uint32_t at_on[kMaxFusedAt], lat_on[kMaxFusedLat];
    float at_thr[kMaxFusedAt], lat_thr[kMaxFusedLat];
#pragma unroll
    for (int aa = 0; aa < kMaxFusedAt; ++aa) {
        at_on[aa] = aa < f.n_at ? f.at[aa].on : 0u;
        at_thr[aa] = f.at[aa].thr;
    }
#pragma unroll
    for (int l = 0; l < kMaxFusedLat; ++l) {
        lat_on[l] = l < f.n_lat ? f.lat[l].on : 0u;
        lat_thr[l] = f.lat[l].thr;
    }

    // ---- sub-steps ----
    for (int s = 0; s < ksteps; ++s) {
        const int64_t n = n0 + s;
        float(*cur)[kBoxF] = (s & 1) ? S.u1 : G.u;
        float(*nxt)[kBoxF] = (s & 1) ? G.u : S.u1;

        if ((stim_on >> s) & 1u) {
            for (int i = 0; i < f.n_stims; ++i) {
                const FStim &F = f.stims[i];
                if (!((F.on >> s) & 1u)) continue;
#pragma unroll
                for (int j = 0; j < 2 * R; ++j) {
                    if (!((myo_bits >> j) & 1u)) continue;
                    const int lr = r0 + j / 2, gi = oi + lr, gj = gj0 + (j & 1);
                    if (gj < F.lo1 || gj >= F.hi1) continue;
                    if (gi < F.lo0 || gi >= F.hi0) continue;
                    if (F.mask && !F.mask[(int64_t)gi * f.nj + gj]) continue;
                    float x = cur[lr + 1][cx + (j & 1)];
                    if (F.kind == FW_STIM_VOLTAGE) {
                        x = F.value;
                    } else {
                        x = x + F.value;
                        if (F.has_umax && x > F.u_max) x = F.u_max;
                    }
                    cur[lr + 1][cx + (j & 1)] = x;
                }
            }
            __syncthreads();
        }

        // window rows r0 - 1 .. r0 + R: a = column c0 - 1, (m0, m1) =
        // columns c0, c0 + 1, b = column c0 + 2
        float a[R + 2], m0[R + 2], m1[R + 2], b[R + 2];
#pragma unroll
        for (int i = 0; i < R + 2; ++i) {
            a[i] = cur[r0 + i][cx - 1];
            const float2 mm = *reinterpret_cast<const float2 *>(&cur[r0 + i][cx]);
            m0[i] = mm.x;
            m1[i] = mm.y;
            b[i] = cur[r0 + i][cx + 2];
        }

        if (own) {
            const float mx = fmaxf(fmaxf(m0[1], m1[1]), fmaxf(m0[2], m1[2]));
#pragma unroll
            for (int aa = 0; aa < kMaxFusedAt; ++aa) {
                if (!((at_on[aa] >> s) & 1u)) continue;
                // (fmaxf skips NaN nodes, which never cross)
                const float thr = at_thr[aa];
                if (!(mx > thr)) continue;
                uint32_t hit = (m0[1] > thr ? 1u : 0u) | (m1[1] > thr ? 2u : 0u) |
                               (m0[2] > thr ? 4u : 0u) | (m1[2] > thr ? 8u : 0u);
                hit &= own & ~(at_done >> (aa * 8));
                if (hit) {
#pragma unroll
                    for (int j = 0; j < 2 * R; ++j) {
                        if (!((hit >> j) & 1u)) continue;
                        // first crossing: unsigned minimum, "never" = -1
                        // (activation_time_2d_tracker.py:61-63)
                        const int64_t p =
                            (int64_t)(oi + r0 + j / 2) * f.nj + gj0 + (j & 1);
                        atomicMin(reinterpret_cast<unsigned *>(f.at[aa].act) + p,
                                  (unsigned)n);
                    }
                    at_done |= hit << (aa * 8);
                }
            }
#pragma unroll
            for (int l = 0; l < kMaxFusedLat; ++l) {
                if (!((lat_on[l] >> s) & 1u)) continue;
                // (local_activation_time_2d_tracker.py:71-89)
                const float thr = lat_thr[l];
                const uint32_t ge = (m0[1] >= thr ? 1u : 0u) | (m1[1] >= thr ? 2u : 0u) |
                                    (m0[2] >= thr ? 4u : 0u) | (m1[2] >= thr ? 8u : 0u);
                const uint32_t lt = (m0[1] < thr ? 1u : 0u) | (m1[1] < thr ? 2u : 0u) |
                                    (m0[2] < thr ? 4u : 0u) | (m1[2] < thr ? 8u : 0u);
                const uint32_t was = (lat_act >> (l * 8)) & 0xffu;
                const uint32_t rise = ge & own & ~was;
                const uint32_t fall = lt & own & was;
                lat_act ^= (rise | fall) << (l * 8);
                if (rise) {
#pragma unroll
                    for (int j = 0; j < 2 * R; ++j)
                        if ((rise >> j) & 1u)
                            lat_record(f.lat[l],
                                       (int64_t)(oi + r0 + j / 2) * f.nj + gj0 + (j & 1),
                                       f.n, n, f.status);
                }
            }
        }

#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int lr = r0 + r;
            float2 uu;
            if constexpr (PACK) {
                const float2 c1 = make_float2(m0[r + 1], m1[r + 1]);
                const float2 un = stencil_fma2<ST>(
                    wcp[r], c1, wp[r], make_float2(a[r], m0[r]),
                    make_float2(m0[r], m1[r]), make_float2(m1[r], b[r]),
                    make_float2(a[r + 1], m0[r + 1]), make_float2(m1[r + 1], b[r + 1]),
                    make_float2(a[r + 2], m0[r + 2]), make_float2(m0[r + 2], m1[r + 2]),
                    make_float2(m1[r + 2], b[r + 2]));
                uu = fused_update_pair<M>(c1, un, st[2 * r], st[2 * r + 1], P, dt);
            } else {
                const float4 wa0 = G.wa[lr][cp], wa1 = G.wa[lr][HW + cp];
                float4 wb0 = wa0, wb1 = wa1;
                if constexpr (NWO == 8) {
                    wb0 = G.wb[lr][cp];
                    wb1 = G.wb[lr][HW + cp];
                }
                const float un0 = stencil_fma<ST>(wcen[2 * r], m0[r + 1], wa0, wb0, a[r],
                                                  m0[r], m1[r], a[r + 1], m1[r + 1],
                                                  a[r + 2], m0[r + 2], m1[r + 2]);
                const float un1 = stencil_fma<ST>(wcen[2 * r + 1], m1[r + 1], wa1, wb1,
                                                  m0[r], m1[r], b[r], m0[r + 1],
                                                  b[r + 1], m0[r + 2], m1[r + 2],
                                                  b[r + 2]);
                uu.x = fused_update<M>(m0[r + 1], un0, st[2 * r], P, dt);
                uu.y = fused_update<M>(m1[r + 1], un1, st[2 * r + 1], P, dt);
            }
            float2 o;
            o.x = ((upd >> (2 * r)) & 1u) ? uu.x : m0[r + 1];
            o.y = ((upd >> (2 * r + 1)) & 1u) ? uu.y : m1[r + 1];
            *reinterpret_cast<float2 *>(&nxt[lr + 1][cx]) = o;
        }
        // probes: u after the stimuli, the state after the update
        if (probe_mine && ((probe_on >> s) & 1u)) {
#pragma unroll
            for (int j = 0; j < 2 * R; ++j)
                if ((probe_mine >> j) & 1u)
                    write_probes<M>(f, S.probe_list, S.probe_count, r0 + j / 2,
                                    c0 + (j & 1), s,
                                    (j & 1) ? m1[j / 2 + 1] : m0[j / 2 + 1], st[j],
                                    ((myo_bits >> j) & 1u) != 0,
                                    (int64_t)(oi + r0 + j / 2) * f.pitch + gj0 +
                                        (j & 1));
        }
        __syncthreads();
    }

    // ---- write the interior back ----
    float(*fin)[kBoxF] = (ksteps & 1) ? S.u1 : G.u;
    bool nonfinite = false;
#pragma unroll
    for (int j = 0; j < 2 * R; ++j) {
        if (!((own >> j) & 1u)) continue;
        const int lr = r0 + j / 2;
        const int64_t pp = (int64_t)(oi + lr) * f.pitch + gj0 + (j & 1);
        if ((myo_bits >> j) & 1u) {
            const float uo = fin[lr + 1][cx + (j & 1)];
            f.u_out[pp] = uo;
            nonfinite |= !isfinite(uo);
            M::template store<float>(f.state_out, pp, st[j]);
        }
        // the flags that changed in this launch (rows of f.pitch nodes)
        if (((lat_act ^ lat_act0) >> j) & 1u)
            f.lat[0].activated[pp] = (lat_act >> j) & 1u;
    }
    if (nonfinite && f.status) atomicOr(f.status, FW_DEV_NONFINITE);
}

template <class M, int ST, int KMAX, int LH, bool PACK>
__global__ void __launch_bounds__((kTW / 2) * (LH / 2), 1)
    k_fused_tma2(const __grid_constant__ TmaK k)
{
    constexpr int LW = kTW, HW = kTW / 2;   // columns, column pairs
    constexpr int R = 2;                     // rows per thread
    constexpr int TI = LH - 2 * KMAX, TJ = LW - 2 * KMAX;
    constexpr int NS = M::NS;
    constexpr int NWO = Stencil2D<ST>::NWO;
    static_assert(KMAX % 2 == 0, "column pairs need an even region origin");
    static_assert(LH % R == 0 && TI > 0 && TJ > 0, "tile shape");
    static_assert(NS <= kMaxTmaState, "state arrays");

    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned mis = smem_u32(smem_raw) & 127u;
    TmaSmem<LH, NS, NWO> &S = *reinterpret_cast<TmaSmem<LH, NS, NWO> *>(
        smem_raw + (mis ? 128u - mis : 0u));
    const FusedK &f = k.f;

    const int tid = threadIdx.x;
    uint32_t own_c, ring_c;
    pair_masks<KMAX, LH>(2 * (tid % HW), (tid / HW) * R, own_c, ring_c);

    if (tid == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    int tile = blockIdx.x;
    const int tj = f.tiles_j;
    const int di = (int)gridDim.x / tj, dj = (int)gridDim.x % tj;
    int bi = tile / tj, bj = tile % tj;
    if (tid == 0 && tile < k.tiles)
        issue_tile<KMAX, LH, NS, NWO, true>(k, S.stage[0], &S.bar[0], bi, bj);

    Params<float, M::NP> P;
#pragma unroll
    for (int i = 0; i < M::NP; ++i) P.v[i] = f.params[i];
    unsigned parity = 0u;

    for (int it = 0; tile < k.tiles; ++it, tile += gridDim.x) {
        const int sg = it & 1;
        TmaStage<LH, NS, NWO> &G = S.stage[sg];
        int ni_ = bi + di, nj_ = bj + dj;
        if (nj_ >= tj) {
            nj_ -= tj;
            ++ni_;
        }
        const int next = tile + gridDim.x;
        if (tid == 0 && next < k.tiles) {
            fence_proxy_async();
            issue_tile<KMAX, LH, NS, NWO, true>(k, S.stage[sg ^ 1], &S.bar[sg ^ 1],
                                                ni_, nj_);
        }
        const unsigned ph = (parity >> sg) & 1u;
        const bool arrived = mbar_wait(&S.bar[sg], ph);
        parity ^= 1u << sg;
        if (__syncthreads_or(!arrived || k.force_timeout)) {
            if (tid == 0) tma_abandon(k, S.bar, sg, ph, parity, arrived, next);
            return;
        }
        const int oi = bi * TI - KMAX, oj = bj * TJ - KMAX;
        bi = ni_;
        bj = nj_;
        tma_tile2<M, ST, KMAX, LH, PACK>(f, G, S, oi, oj, own_c, ring_c, P);
        __syncthreads();
    }
}

// ---- host side -------------------------------------------------------------------

inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// A 2D map of (ni, nj) nodes whose rows start `pitch` nodes apart (0: nj).
inline bool encode_2d(CUtensorMap *m, CUtensorMapDataType t, size_t esize,
                      const void *base, int64_t nj, int64_t ni, int bw, int bh,
                      int64_t pitch = 0)
{
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)nj, (cuuint64_t)ni};
    cuuint64_t strides[1] = {(cuuint64_t)((pitch ? pitch : nj) * esize)};
    cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh};
    cuuint32_t es[2] = {1, 1};
    return enc(m, t, 2, const_cast<void *>(base), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

inline bool encode_weights(CUtensorMap *m, const void *base, int nwo, int64_t nj,
                           int64_t ni, int bh, int64_t pitch = 0)
{
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    cuuint64_t dims[3] = {(cuuint64_t)nwo, (cuuint64_t)nj, (cuuint64_t)ni};
    cuuint64_t strides[2] = {(cuuint64_t)(nwo * 4),
                             (cuuint64_t)((pitch ? pitch : nj) * nwo * 4)};
    cuuint32_t box[3] = {4, (cuuint32_t)kTW, (cuuint32_t)bh};
    cuuint32_t es[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(base), dims,
               strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The same packed weights viewed as (q, column pair, column parity, row):
// a box of 32 pairs x 2 parities lands as [row][parity][pair] float4s.
// With a row pitch (a multiple of 16 nodes, rows padded with zero weights)
// the view spans the pitch: columns nj .. pitch - 1 read the padding.
inline bool encode_weights_pairs(CUtensorMap *m, const void *base, int nwo,
                                 int64_t nj, int64_t ni, int bh, int64_t pitch = 0)
{
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const int64_t w = pitch ? pitch : nj;
    cuuint64_t dims[4] = {(cuuint64_t)nwo, (cuuint64_t)(w / 2), 2, (cuuint64_t)ni};
    cuuint64_t strides[3] = {(cuuint64_t)(2 * nwo * 4), (cuuint64_t)(nwo * 4),
                             (cuuint64_t)(w * nwo * 4)};
    cuuint32_t box[4] = {4, (cuuint32_t)(kTW / 2), 2, (cuuint32_t)bh};
    cuuint32_t es[4] = {1, 1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void *>(base), dims,
               strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

inline int sm_count()
{
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    return n;
}

inline bool aligned16(const void *p) { return p && ((uintptr_t)p & 15) == 0; }

// True when the TMA form can run this configuration: every array it reads
// through a tensor map (packed weights, the weights' centre plane, both
// potential buffers, the myocyte flags, the model's `ns` state arrays and
// the local activation tracker's flags) starts on a 16-byte boundary, and
// rows are a multiple of 16 nodes.
inline bool tma_usable(const fw_step_args *a, int ns)
{
    bool ok = aligned16(a->weights_packed) && aligned16(a->weights) &&
              aligned16(a->u[0]) && aligned16(a->u[1]) && aligned16(a->myo) &&
              a->nj % 16 == 0 && a->ni < (1 << 30) && a->nj < (1 << 30);
    for (int q = 0; q < ns && ok; ++q)
        ok = aligned16(a->state[q]) && aligned16(a->state_b[q]);
    for (int l = 0; l < a->n_lat && ok; ++l) ok = aligned16(a->lat[l].activated);
    return ok && tensor_map_encoder() != nullptr;
}

// The same for the weights formed on chip (fused_variant 5): the float32
// fiber pairs take the place of the weights.
inline bool tma_fly_usable(const fw_step_args *a, int ns)
{
    bool ok = aligned16(a->fibers_f32) && aligned16(a->u[0]) &&
              aligned16(a->u[1]) && aligned16(a->myo) && a->nj % 16 == 0 &&
              a->ni < (1 << 30) && a->nj < (1 << 29);
    for (int q = 0; q < ns && ok; ++q)
        ok = aligned16(a->state[q]) && aligned16(a->state_b[q]);
    for (int l = 0; l < a->n_lat && ok; ++l) ok = aligned16(a->lat[l].activated);
    return ok && tensor_map_encoder() != nullptr;
}

// PAIRS: the column-pair kernel k_fused_tma2 (R is then 2, fixed by it),
// PACK: its two-wide float32 form (fused_variant 6).
// FLY: the weights formed on chip from the float32 fibers (fused_variant 5).
template <class M, int ST, int KMAX, int LH, int R, bool PAIRS = false, bool FLY = false,
          bool PACK = false>
int launch_fused_tma(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                     cudaStream_t stream)
{
    constexpr int TI = LH - 2 * KMAX, TJ = kTW - 2 * KMAX;
    constexpr int NT = PAIRS ? (kTW / 2) * (LH / 2) : kTW * (LH / R);
    constexpr int NWO = Stencil2D<ST>::NWO;
    constexpr size_t SMEM = sizeof(TmaSmem<LH, M::NS, NWO>) + 1024;
    static_assert(!(PAIRS && FLY), "weights on chip: strip kernel only");
    void (*kern)(const TmaK);
    if constexpr (PAIRS)
        kern = k_fused_tma2<M, ST, KMAX, LH, PACK>;
    else
        kern = k_fused_tma<M, ST, KMAX, LH, R, FLY>;
    FW_CUDA_CHECK(cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM));
    if (a->n_lat > kMaxFusedLat) {
        set_error("fw_step (fused): at most %d local activation tracker",
                  kMaxFusedLat);
        return FW_ERR_UNSUPPORTED;
    }
    TmaK k;  // kernel argument, copied at each launch
    memset(&k, 0, sizeof k);
    k.force_timeout = (a->debug_flags & FW_DEBUG_FORCE_TIMEOUT) ? 1 : 0;
    bool ok = (FLY ? encode_2d(&k.maps.fib, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                               a->fibers_f32, 2 * a->nj, a->ni, kBoxFib, LH)
                   : PAIRS ? encode_weights_pairs(&k.maps.w, a->weights_packed, NWO,
                                                  a->nj, a->ni, LH)
                           : encode_weights(&k.maps.w, a->weights_packed, NWO, a->nj,
                                            a->ni, LH)) &&
              encode_2d(&k.maps.myo, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, a->myo,
                        a->nj, a->ni, kBoxB, LH) &&
              encode_2d(&k.maps.u[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a->u[0],
                        a->nj, a->ni, kBoxF, LH + 2) &&
              encode_2d(&k.maps.u[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a->u[1],
                        a->nj, a->ni, kBoxF, LH + 2);
    for (int q = 0; q < M::NS && ok; ++q)
        ok = encode_2d(&k.maps.s[0][q], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                       a->state[q], a->nj, a->ni, kBoxF, LH) &&
             encode_2d(&k.maps.s[1][q], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                       a->state_b[q], a->nj, a->ni, kBoxF, LH);
    // the centre plane of the (nw, ni * nj) float32 weights
    if (ok && !FLY) {
        const float *wcen_plane = (const float *)a->weights +
                                  (int64_t)Stencil2D<ST>::CENTRE * a->ni * a->nj;
        ok = encode_2d(&k.maps.wc, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, wcen_plane,
                       a->nj, a->ni, kBoxF, LH);
    }
    if (ok && a->n_lat > 0)
        ok = encode_2d(&k.maps.act, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1,
                       a->lat[0].activated, a->nj, a->ni, kBoxB, LH);
    if (!ok) {
        set_error("fw_step (fused TMA): tensor map encoding failed");
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
    f.fly_dal = (float)a->fly_D_al;
    f.fly_dac = (float)a->fly_D_ac;
    f.fly_cond = (float)a->fly_cond;
    f.fly_scale = (float)a->fly_scale;
    const int tiles_i = (int)((a->ni + TI - 1) / TI);
    f.tiles_j = (int)((a->nj + TJ - 1) / TJ);
    k.tiles = tiles_i * f.tiles_j;
    int sms = sm_count();
    if (sms <= 0) sms = 152;
    const int grid = k.tiles < sms ? k.tiles : sms;
    int64_t probe_samples[FW_MAX_PROBE];
    for (int i = 0; i < a->n_probe; ++i) probe_samples[i] = a->probe[i].sample_offset;

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
        kern<<<grid, NT, SMEM, stream>>>(k);
        FW_CHECK_LAUNCH("k_fused_tma");
        done += ks;
    }
    return FW_OK;
}

// the row-marching wavefront (fw_fused_march.cuh, fused variant 7)
template <class M, int ST, int KMAX>
int launch_fused_march(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                       cudaStream_t stream);

// Kernel choice (fw_step_args.fused_variant):
//   0: automatic -- the TMA pipeline when it can run, else 1;
//   1: cp.async staging, 64 x 32 regions, 256 threads, two CTAs per SM;
//   2: cp.async staging, 64 x 64 regions, 512 threads, one CTA per SM;
//   3: TMA pipeline: persistent CTAs, 64 x 32 regions, 512 threads with
//      4-node strips, two stages in shared memory;
//   4: the TMA pipeline with 2 x 2 node blocks per thread (even K only);
//   5: variant 3 with the AsymmetricStencil2D weights formed on chip from
//      float32 fibers (fw_step_args.fibers_f32) instead of read from HBM;
//   6: variant 4 in two-wide float32 instructions (each node's bits those
//      of variants 3 and 4; even K only);
//   7: the row-marching wavefront: 64-column strips marched down in 8-row
//      blocks with the K time levels in flight (K <= 4, no probes).
// KMAX (fused_k) in {2, 4, 8} time steps per launch (3 also for 3 and 5).
template <class M, int ST>
int fused_dispatch(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                   cudaStream_t stream)
{
    const int k = a->fused_k ? a->fused_k : 4;
    int v = a->fused_variant;
    static_assert(M::NS <= FW_MAX_FUSED_STATE, "fused state buffers");
    for (int q = 0; q < M::NS; ++q)
        if (!a->state_b[q] || a->state_b[q] == a->state[q]) {
            set_error("fw_step (fused): state_b[%d] missing or equal to "
                      "state[%d] (the fused form needs a second buffer per "
                      "state variable)", q, q);
            return FW_ERR_ARG;
        }
    if (v == 0) v = tma_usable(a, M::NS) ? 3 : 1;
    if (v == 5) {
        if constexpr (ST == FW_STENCIL_ANISO9) {
            if (!tma_fly_usable(a, M::NS)) {
                set_error("fw_step (fused variant 5): needs fibers_f32 and "
                          "16-byte aligned potential, state and myocyte "
                          "arrays with nj %% 16 == 0");
                return FW_ERR_UNSUPPORTED;
            }
#define FW_FLY_CASE(KK)                                                        \
    return launch_fused_tma<M, ST, KK, 32, 4, false, true>(a, n_begin, n_steps, stream)
            if (k == 2) FW_FLY_CASE(2);
            if (k == 3) FW_FLY_CASE(3);
            if (k == 4) FW_FLY_CASE(4);
            if (k == 8) FW_FLY_CASE(8);
#undef FW_FLY_CASE
        } else {
            set_error("fw_step (fused variant 5): the weights are formed on "
                      "chip for AsymmetricStencil2D only");
            return FW_ERR_UNSUPPORTED;
        }
    }
    if ((v == 3 || v == 4 || v == 6 || v == 7) && !tma_usable(a, M::NS)) {
        set_error("fw_step (fused): the TMA kernels need packed weights, "
                  "16-byte aligned weights, potential, state and myocyte "
                  "arrays and nj %% 16 == 0");
        return FW_ERR_UNSUPPORTED;
    }
#define FW_CP_CASE(KK, LH, MINB)                                               \
    return launch_fused<M, ST, KK, 64, LH, 8, MINB>(a, n_begin, n_steps, stream)
#define FW_TMA_CASE(KK)                                                        \
    return launch_fused_tma<M, ST, KK, 32, 4>(a, n_begin, n_steps, stream)
#define FW_TMA2_CASE(KK)                                                       \
    return launch_fused_tma<M, ST, KK, 32, 2, true>(a, n_begin, n_steps, stream)
#define FW_PACK_CASE(KK)                                                       \
    return launch_fused_tma<M, ST, KK, 32, 2, true, false, true>(a, n_begin,   \
                                                                n_steps, stream)
    if (v == 1) {
        if (k == 2) FW_CP_CASE(2, 32, 2);
        if (k == 4) FW_CP_CASE(4, 32, 2);
        if (k == 8) FW_CP_CASE(8, 32, 2);
    } else if (v == 2) {
        if (k == 2) FW_CP_CASE(2, 64, 1);
        if (k == 4) FW_CP_CASE(4, 64, 1);
        if (k == 8) FW_CP_CASE(8, 64, 1);
    } else if (v == 3) {
        if (k == 2) FW_TMA_CASE(2);
        if (k == 3) FW_TMA_CASE(3);
        if (k == 4) FW_TMA_CASE(4);
        if (k == 8) FW_TMA_CASE(8);
    } else if (v == 4) {
        if (k == 2) FW_TMA2_CASE(2);
        if (k == 4) FW_TMA2_CASE(4);
        if (k == 8) FW_TMA2_CASE(8);
    } else if (v == 6) {
        if (k == 2) FW_PACK_CASE(2);
        if (k == 4) FW_PACK_CASE(4);
        if (k == 8) FW_PACK_CASE(8);
    } else if (v == 7) {
        if (k == 2) return launch_fused_march<M, ST, 2>(a, n_begin, n_steps, stream);
        if (k == 3) return launch_fused_march<M, ST, 3>(a, n_begin, n_steps, stream);
        if (k == 4) return launch_fused_march<M, ST, 4>(a, n_begin, n_steps, stream);
    }
#undef FW_CP_CASE
#undef FW_TMA_CASE
#undef FW_TMA2_CASE
#undef FW_PACK_CASE
    set_error("fw_step (fused): no kernel for fused_k=%d fused_variant=%d "
              "(k in 2, 3, 4, 8; variant in 0..7, variants 4 and 6 with even "
              "k, variant 5 for AsymmetricStencil2D, variant 7 with k <= 4)",
              k, a->fused_variant);
    return FW_ERR_UNSUPPORTED;
}

template <class M>
int fused_model(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
                cudaStream_t stream)
{
    switch (a->stencil) {
    case FW_STENCIL_ISO5:
        return fused_dispatch<M, FW_STENCIL_ISO5>(a, n_begin, n_steps, stream);
    case FW_STENCIL_ANISO9:
        return fused_dispatch<M, FW_STENCIL_ANISO9>(a, n_begin, n_steps, stream);
    }
    set_error("fw_step (fused): 2D stencils only");
    return FW_ERR_UNSUPPORTED;
}

}  // namespace fused
}  // namespace fw
