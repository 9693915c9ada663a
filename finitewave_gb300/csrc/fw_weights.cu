// fw_weights.cu -- stencil-weight construction on the GPU.
//
// Built with --fmad=false: every weight is computed in float64 with the
// reference's operation order, so the float64 result is bitwise the
// reference's (and the oracle's).  One thread per node; the half-step
// conductivity / diffusion-tensor means the reference precomputes with
// np.roll are recomputed on the fly from the node and its +1 neighbour along
// the axis, wrapping around at the far edge exactly as np.roll does.
#include "fw_internal.cuh"

namespace fw {
namespace {

struct WArgs {
    const int8_t *mesh;
    const double *cond;
    double cond_scalar;
    const double *fibers;
    double D_al, D_ac, D_model, dt, dr2;
    int64_t ni, nj, nk, n;
    int64_t shape[3];
    int64_t stride[3];
    int dim;
};

__device__ __forceinline__ int m01(const WArgs &a, int64_t p)
{
    return a.mesh[p] == 1;
}

__device__ __forceinline__ double cond_at(const WArgs &a, int64_t p)
{
    // conductivity * np.ones_like(mesh) (isotropic_stencil_2d.py:60-61)
    return a.cond ? a.cond[p] * 1.0 : a.cond_scalar * 1.0;
}

// True for nodes on the outer ring of the grid.  The tissue classes zero the
// ring (cardiac_tissue_2d.py:35-45), so a myocyte there is invalid input; it
// is skipped here (no neighbour access outside the grid) and rejected by the
// host layer before any step runs.
__device__ __forceinline__ bool on_ring(const WArgs &a, int64_t p)
{
    for (int ax = 0; ax < a.dim; ++ax) {
        int64_t c = (p / a.stride[ax]) % a.shape[ax];
        if (c == 0 || c == a.shape[ax] - 1) return true;
    }
    return false;
}

// +1 neighbour of p along `ax` with np.roll(-1) wrap-around.
__device__ __forceinline__ int64_t roll_next(const WArgs &a, int64_t p, int ax)
{
    int64_t s = a.stride[ax], len = a.shape[ax];
    int64_t c = (p / s) % len;
    return (c + 1 == len) ? p - c * s : p + s;
}

// 0.5 * (c + roll(c, -1, axis)) (isotropic_stencil_2d.py:89-94)
__device__ __forceinline__ double half_iso(const WArgs &a, int64_t p, int ax)
{
    int64_t q = roll_next(a, p, ax);
    return 0.5 * (cond_at(a, p) + cond_at(a, q));
}

// D_ac*(a0==a1) + (D_al-D_ac)*f[a0]*f[a1] (asymmetric_stencil_2d.py:160-161)
__device__ __forceinline__ double dcomp(const WArgs &a, int64_t p, int a0,
                                        int a1)
{
    double diag = a.D_ac * (double)(a0 == a1);
    const double *f = a.fibers + p * a.dim;
    return diag + (a.D_al - a.D_ac) * f[a0] * f[a1];
}

// 0.5*(D*c + roll(D)*roll(c)) (asymmetric_stencil_2d.py:128-136)
__device__ __forceinline__ double half_aniso(const WArgs &a, int64_t p,
                                             int ax, int comp)
{
    int64_t q = roll_next(a, p, ax);
    double dp = dcomp(a, p, ax, comp), dq = dcomp(a, q, ax, comp);
    return 0.5 * (dp * cond_at(a, p) + dq * cond_at(a, q));
}

// compute_component (isotropic_stencil_2d.py:135-158)
__device__ __forceinline__ double icomp(double d, int m0, int m1)
{
    return d * (double)m0 * (double)(m0 + (m1 == 0));
}

// minor_component (asymmetric_stencil_2d.py:204-259)
__device__ __forceinline__ void minor(double d, int m0, int m1, int m2,
                                      int m3, int m4, int m5, double r[6])
{
    int mh = m2 + m3 + m4 + m5;
    int ml = m0 + m1 + m2 + m3;
    if (m2 == 0 || m3 == 0 || mh < 3 || ml < 3) {
        r[0] = r[1] = r[2] = r[3] = r[4] = r[5] = 0.0;
        return;
    }
    double dh = (double)mh, dl = (double)ml;
    r[0] = (-d) * (double)m0 / dl;
    r[1] = (-d) * (double)m1 / dl;
    r[2] = d * ((double)m2 / dh - (double)m2 / dl);
    r[3] = d * ((double)m3 / dh - (double)m3 / dl);
    r[4] = d * (double)m4 / dh;
    r[5] = d * (double)m5 / dh;
}

// weights * D_model * dt / dr**2, then +1 on the centre, then store.
template <int NW, class T>
__device__ __forceinline__ void finish(const WArgs &a, int64_t p, double *o,
                                       int centre, T *w)
{
#pragma unroll
    for (int k = 0; k < NW; ++k) {
        double x = o[k] * a.D_model * a.dt / a.dr2;
        if (k == centre) x += 1.0;
        w[k * a.n + p] = (T)x;
    }
}

// IsotropicStencil2D.compute_weights + njit compute_weights
// (isotropic_stencil_2d.py:41-69, 161-204)
template <class T>
__global__ void k_iso5(WArgs a, T *w)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.n;
         p += (int64_t)gridDim.x * blockDim.x) {
        double o[5] = {0, 0, 0, 0, 0};
        if (m01(a, p) && !on_ring(a, p)) {
            int64_t si = a.nj;
            int64_t im = p - si, ip = p + si, jm = p - 1, jp = p + 1;
            o[0] = icomp(half_iso(a, im, 0), m01(a, im), m01(a, ip));
            o[1] = icomp(half_iso(a, jm, 1), m01(a, jm), m01(a, jp));
            o[3] = icomp(half_iso(a, p, 1), m01(a, jp), m01(a, jm));
            o[4] = icomp(half_iso(a, p, 0), m01(a, ip), m01(a, im));
            o[2] = -(o[0] + o[1] + o[3] + o[4]);
        }
        finish<5>(a, p, o, 2, w);
    }
}

// IsotropicStencil3D (isotropic_stencil_3d.py:45-74, 113-149)
template <class T>
__global__ void k_iso7(WArgs a, T *w)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.n;
         p += (int64_t)gridDim.x * blockDim.x) {
        double o[7] = {0, 0, 0, 0, 0, 0, 0};
        if (m01(a, p) && !on_ring(a, p)) {
            int64_t si = a.stride[0], sj = a.stride[1];
            o[0] = icomp(half_iso(a, p - si, 0), m01(a, p - si), m01(a, p + si));
            o[1] = icomp(half_iso(a, p - sj, 1), m01(a, p - sj), m01(a, p + sj));
            o[2] = icomp(half_iso(a, p - 1, 2), m01(a, p - 1), m01(a, p + 1));
            o[4] = icomp(half_iso(a, p, 2), m01(a, p + 1), m01(a, p - 1));
            o[5] = icomp(half_iso(a, p, 1), m01(a, p + sj), m01(a, p - sj));
            o[6] = icomp(half_iso(a, p, 0), m01(a, p + si), m01(a, p - si));
            o[3] = -(o[0] + o[1] + o[2] + o[4] + o[5] + o[6]);
        }
        finish<7>(a, p, o, 3, w);
    }
}

// AsymmetricStencil2D.compute_weights + njit compute_weights
// (asymmetric_stencil_2d.py:46-84, 291-433): four faces, each a major flux
// and a six-point minor flux, accumulated in the reference's order.
template <class T>
__global__ void k_aniso9(WArgs a, T *w)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.n;
         p += (int64_t)gridDim.x * blockDim.x) {
        double o[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (m01(a, p) && !on_ring(a, p)) {
            const int64_t si = a.nj;
#define M(di, dj) m01(a, p + (di) * si + (dj))
#define Q(di, dj) (p + (di) * si + (dj))
            double r[6], q;
            // q (i-1/2, j)
            q = half_aniso(a, Q(-1, 0), 0, 0) * (double)M(-1, 0);
            o[1] += q; o[4] -= q;
            minor(half_aniso(a, Q(-1, 0), 0, 1), M(-1, -1), M(0, -1),
                  M(-1, 0), M(0, 0), M(-1, 1), M(0, 1), r);
            o[0] -= r[0]; o[3] -= r[1]; o[1] -= r[2];
            o[4] -= r[3]; o[2] -= r[4]; o[5] -= r[5];
            // q (i, j-1/2)
            q = half_aniso(a, Q(0, -1), 1, 1) * (double)M(0, -1);
            o[3] += q; o[4] -= q;
            minor(half_aniso(a, Q(0, -1), 1, 0), M(-1, -1), M(-1, 0),
                  M(0, -1), M(0, 0), M(1, -1), M(1, 0), r);
            o[0] -= r[0]; o[1] -= r[1]; o[3] -= r[2];
            o[4] -= r[3]; o[6] -= r[4]; o[7] -= r[5];
            // q (i, j+1/2)
            q = half_aniso(a, p, 1, 1) * (double)M(0, 1);
            o[5] += q; o[4] -= q;
            minor(half_aniso(a, p, 1, 0), M(-1, 1), M(-1, 0), M(0, 1),
                  M(0, 0), M(1, 1), M(1, 0), r);
            o[2] += r[0]; o[1] += r[1]; o[5] += r[2];
            o[4] += r[3]; o[8] += r[4]; o[7] += r[5];
            // q (i+1/2, j)
            q = half_aniso(a, p, 0, 0) * (double)M(1, 0);
            o[7] += q; o[4] -= q;
            minor(half_aniso(a, p, 0, 1), M(1, -1), M(0, -1), M(1, 0),
                  M(0, 0), M(1, 1), M(0, 1), r);
            o[6] += r[0]; o[3] += r[1]; o[7] += r[2];
            o[4] += r[3]; o[8] += r[4]; o[5] += r[5];
#undef M
#undef Q
        }
        finish<9>(a, p, o, 4, w);
    }
}

// SymmetricStencil2D (symmetric_stencil_2d.py:31-250): the diffusion tensor
// D * conductivity averaged to the cell corners,
//   0.25 * (D[i,j] + D[i+1,j] + D[i,j+1] + D[i+1,j+1])  (np.roll wrap),
// and the flux through each of the node's four corner cells distributed to
// the cell's four nodes (compute_components), accumulated in the
// reference's corner order.
__device__ __forceinline__ double dcorner(const WArgs &a, int64_t q, int c0,
                                          int c1)
{
    const int64_t qi = roll_next(a, q, 0), qj = roll_next(a, q, 1);
    const int64_t qij = roll_next(a, qi, 1);
    return 0.25 * (dcomp(a, q, c0, c1) * cond_at(a, q) +
                   dcomp(a, qi, c0, c1) * cond_at(a, qi) +
                   dcomp(a, qj, c0, c1) * cond_at(a, qj) +
                   dcomp(a, qij, c0, c1) * cond_at(a, qij));
}

// compute_components (symmetric_stencil_2d.py:96-140)
__device__ __forceinline__ void sym_corner(const WArgs &a, int64_t q, int m0,
                                           int m1, int m2, int m3, int qx,
                                           int qy, double r[4])
{
    if (m0 + m1 + m2 + m3 < 3) {
        r[0] = r[1] = r[2] = r[3] = 0.0;
        return;
    }
    const double dxx = dcorner(a, q, 0, 0), dxy = dcorner(a, q, 0, 1),
                 dyx = dcorner(a, q, 1, 0), dyy = dcorner(a, q, 1, 1);
    const double qdx = (double)qx * dxx + (double)qy * dyx;
    const double qdy = (double)qx * dxy + (double)qy * dyy;
    const double d0 = m0, d1 = m1, d2 = m2, d3 = m3;
    const double w0 = (-d0) / (d0 + d1) * qdx - d0 / (d0 + d2) * qdy;
    const double w1 = (-d1) / (d0 + d1) * qdx + d1 / (d1 + d3) * qdy;
    const double w2 = d2 / (d2 + d3) * qdx - d2 / (d0 + d2) * qdy;
    const double w3 = d3 / (d2 + d3) * qdx + d3 / (d1 + d3) * qdy;
    r[0] = 0.5 * w0;
    r[1] = 0.5 * w1;
    r[2] = 0.5 * w2;
    r[3] = 0.5 * w3;
}

template <class T>
__global__ void k_sym9(WArgs a, T *w)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.n;
         p += (int64_t)gridDim.x * blockDim.x) {
        double o[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (m01(a, p) && !on_ring(a, p)) {
            const int64_t si = a.nj;
#define M(di, dj) m01(a, p + (di) * si + (dj))
#define Q(di, dj) (p + (di) * si + (dj))
            double r[4];
            // corner (i-1, j-1): nodes (i-1,j-1), (i-1,j), (i,j-1), (i,j)
            sym_corner(a, Q(-1, -1), M(-1, -1), M(-1, 0), M(0, -1), M(0, 0),
                       -1, -1, r);
            o[0] += r[0]; o[1] += r[1]; o[3] += r[2]; o[4] += r[3];
            // corner (i-1, j)
            sym_corner(a, Q(-1, 0), M(-1, 0), M(-1, 1), M(0, 0), M(0, 1), -1,
                       1, r);
            o[1] += r[0]; o[2] += r[1]; o[4] += r[2]; o[5] += r[3];
            // corner (i, j-1)
            sym_corner(a, Q(0, -1), M(0, -1), M(0, 0), M(1, -1), M(1, 0), 1,
                       -1, r);
            o[3] += r[0]; o[4] += r[1]; o[6] += r[2]; o[7] += r[3];
            // corner (i, j)
            sym_corner(a, Q(0, 0), M(0, 0), M(0, 1), M(1, 0), M(1, 1), 1, 1,
                       r);
            o[4] += r[0]; o[5] += r[1]; o[7] += r[2]; o[8] += r[3];
#undef M
#undef Q
        }
        // weights *= D_model * dt / dr**2: the factor first
        // (symmetric_stencil_2d.py:64), unlike the other stencils
        const double scale = a.D_model * a.dt / a.dr2;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            double x = o[k] * scale;
            if (k == 4) x += 1.0;
            w[k * a.n + p] = (T)x;
        }
    }
}

// AsymmetricStencil3D.compute_weights + its serial njit accumulation
// (asymmetric_stencil_3d.py:61-105, 164-458): six faces, each a major flux
// and two six-point minor fluxes.
template <class T>
__global__ void k_aniso19(WArgs a, T *w)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.n;
         p += (int64_t)gridDim.x * blockDim.x) {
        double o[19];
#pragma unroll
        for (int k = 0; k < 19; ++k) o[k] = 0.0;
        if (m01(a, p) && !on_ring(a, p)) {
            const int64_t si = a.stride[0], sj = a.stride[1];
#define M(di, dj, dk) m01(a, p + (di) * si + (dj) * sj + (dk))
#define Q(di, dj, dk) (p + (di) * si + (dj) * sj + (dk))
            double r[6], q;
            // q (i-1/2, j, k)
            q = half_aniso(a, Q(-1, 0, 0), 0, 0) * (double)M(-1, 0, 0);
            o[1] += q; o[4] -= q;
            minor(half_aniso(a, Q(-1, 0, 0), 0, 1), M(-1, -1, 0), M(0, -1, 0),
                  M(-1, 0, 0), M(0, 0, 0), M(-1, 1, 0), M(0, 1, 0), r);
            o[0] -= r[0]; o[3] -= r[1]; o[1] -= r[2];
            o[4] -= r[3]; o[2] -= r[4]; o[5] -= r[5];
            minor(half_aniso(a, Q(-1, 0, 0), 0, 2), M(-1, 0, -1), M(0, 0, -1),
                  M(-1, 0, 0), M(0, 0, 0), M(-1, 0, 1), M(0, 0, 1), r);
            o[15] -= r[0]; o[11] -= r[1]; o[1] -= r[2];
            o[4] -= r[3]; o[17] -= r[4]; o[12] -= r[5];
            // q (i+1/2, j, k)
            q = half_aniso(a, p, 0, 0) * (double)M(1, 0, 0);
            o[7] += q; o[4] -= q;
            minor(half_aniso(a, p, 0, 1), M(1, -1, 0), M(0, -1, 0),
                  M(1, 0, 0), M(0, 0, 0), M(1, 1, 0), M(0, 1, 0), r);
            o[6] += r[0]; o[3] += r[1]; o[7] += r[2];
            o[4] += r[3]; o[8] += r[4]; o[5] += r[5];
            minor(half_aniso(a, p, 0, 2), M(1, 0, -1), M(0, 0, -1),
                  M(1, 0, 0), M(0, 0, 0), M(1, 0, 1), M(0, 0, 1), r);
            o[16] += r[0]; o[11] += r[1]; o[7] += r[2];
            o[4] += r[3]; o[18] += r[4]; o[12] += r[5];
            // q (i, j-1/2, k)
            q = half_aniso(a, Q(0, -1, 0), 1, 1) * (double)M(0, -1, 0);
            o[3] += q; o[4] -= q;
            minor(half_aniso(a, Q(0, -1, 0), 1, 0), M(-1, -1, 0), M(-1, 0, 0),
                  M(0, -1, 0), M(0, 0, 0), M(1, -1, 0), M(1, 0, 0), r);
            o[0] -= r[0]; o[1] -= r[1]; o[3] -= r[2];
            o[4] -= r[3]; o[6] -= r[4]; o[7] -= r[5];
            minor(half_aniso(a, Q(0, -1, 0), 1, 2), M(0, -1, -1), M(0, 0, -1),
                  M(0, -1, 0), M(0, 0, 0), M(0, -1, 1), M(0, 0, 1), r);
            o[9] -= r[0]; o[11] -= r[1]; o[3] -= r[2];
            o[4] -= r[3]; o[10] -= r[4]; o[12] -= r[5];
            // q (i, j+1/2, k)
            q = half_aniso(a, p, 1, 1) * (double)M(0, 1, 0);
            o[5] += q; o[4] -= q;
            minor(half_aniso(a, p, 1, 0), M(-1, 1, 0), M(-1, 0, 0),
                  M(0, 1, 0), M(0, 0, 0), M(1, 1, 0), M(1, 0, 0), r);
            o[2] += r[0]; o[1] += r[1]; o[5] += r[2];
            o[4] += r[3]; o[8] += r[4]; o[7] += r[5];
            minor(half_aniso(a, p, 1, 2), M(0, 1, -1), M(0, 0, -1),
                  M(0, 1, 0), M(0, 0, 0), M(0, 1, 1), M(0, 0, 1), r);
            o[13] += r[0]; o[11] += r[1]; o[5] += r[2];
            o[4] += r[3]; o[14] += r[4]; o[12] += r[5];
            // q (i, j, k-1/2)
            q = half_aniso(a, Q(0, 0, -1), 2, 2) * (double)M(0, 0, -1);
            o[11] += q; o[4] -= q;
            minor(half_aniso(a, Q(0, 0, -1), 2, 0), M(-1, 0, -1), M(-1, 0, 0),
                  M(0, 0, -1), M(0, 0, 0), M(1, 0, -1), M(1, 0, 0), r);
            o[15] -= r[0]; o[1] -= r[1]; o[11] -= r[2];
            o[4] -= r[3]; o[16] -= r[4]; o[7] -= r[5];
            minor(half_aniso(a, Q(0, 0, -1), 2, 1), M(0, -1, -1), M(0, -1, 0),
                  M(0, 0, -1), M(0, 0, 0), M(0, 1, -1), M(0, 1, 0), r);
            o[9] -= r[0]; o[3] -= r[1]; o[11] -= r[2];
            o[4] -= r[3]; o[13] -= r[4]; o[5] -= r[5];
            // q (i, j, k+1/2)
            q = half_aniso(a, p, 2, 2) * (double)M(0, 0, 1);
            o[12] += q; o[4] -= q;
            minor(half_aniso(a, p, 2, 0), M(-1, 0, 1), M(-1, 0, 0),
                  M(0, 0, 1), M(0, 0, 0), M(1, 0, 1), M(1, 0, 0), r);
            o[17] += r[0]; o[1] += r[1]; o[12] += r[2];
            o[4] += r[3]; o[18] += r[4]; o[7] += r[5];
            minor(half_aniso(a, p, 2, 1), M(0, -1, 1), M(0, -1, 0),
                  M(0, 0, 1), M(0, 0, 0), M(0, 1, 1), M(0, 1, 0), r);
            o[10] += r[0]; o[3] += r[1]; o[12] += r[2];
            o[4] += r[3]; o[14] += r[4]; o[5] += r[5];
#undef M
#undef Q
        }
        finish<19>(a, p, o, 4, w);
    }
}

template <class T>
void launch(int32_t stencil, const WArgs &a, void *w, cudaStream_t s)
{
    const int threads = 256;
    int blocks = grid_for(a.n, threads);
    T *wt = (T *)w;
    switch (stencil) {
    case FW_STENCIL_ISO5: k_iso5<T><<<blocks, threads, 0, s>>>(a, wt); break;
    case FW_STENCIL_ANISO9: k_aniso9<T><<<blocks, threads, 0, s>>>(a, wt); break;
    case FW_STENCIL_ISO7: k_iso7<T><<<blocks, threads, 0, s>>>(a, wt); break;
    case FW_STENCIL_ANISO19: k_aniso19<T><<<blocks, threads, 0, s>>>(a, wt); break;
    case FW_STENCIL_SYM9: k_sym9<T><<<blocks, threads, 0, s>>>(a, wt); break;
    }
}

}  // namespace

int build_weights(int32_t stencil, int32_t precision, const int8_t *mesh,
                  const double *cond, double cond_scalar, const double *fibers,
                  double D_al, double D_ac, double D_model, double dt,
                  double dr2, int64_t ni, int64_t nj, int64_t nk, void *w_out,
                  cudaStream_t stream)
{
    // the in-plane-fiber form of the 3D stencil is built as the full one
    if (stencil == FW_STENCIL_ANISO19_XY) stencil = FW_STENCIL_ANISO19;
    int nw = stencil_nw(stencil);
    if (!nw) {
        set_error("fw_build_weights: unknown stencil %d", stencil);
        return FW_ERR_ARG;
    }
    int dim = stencil_dim(stencil);
    bool aniso = stencil == FW_STENCIL_ANISO9 || stencil == FW_STENCIL_ANISO19 ||
                 stencil == FW_STENCIL_SYM9;
    if (!mesh || !w_out || (aniso && !fibers) || ni < 1 || nj < 1 ||
        (dim == 3 && nk < 1)) {
        set_error("fw_build_weights: null pointer or empty grid");
        return FW_ERR_ARG;
    }
    if (precision != FW_F64 && precision != FW_F32) {
        set_error("fw_build_weights: unknown precision %d", precision);
        return FW_ERR_ARG;
    }
    WArgs a;
    a.mesh = mesh;
    a.cond = cond;
    a.cond_scalar = cond_scalar;
    a.fibers = fibers;
    a.D_al = D_al;
    a.D_ac = D_ac;
    a.D_model = D_model;
    a.dt = dt;
    a.dr2 = dr2;
    a.ni = ni;
    a.nj = nj;
    a.nk = dim == 2 ? 1 : nk;
    a.n = ni * nj * a.nk;
    a.dim = dim;
    a.shape[0] = ni;
    a.shape[1] = nj;
    a.shape[2] = a.nk;
    if (dim == 2) {
        a.stride[0] = nj;
        a.stride[1] = 1;
        a.stride[2] = 1;
    } else {
        a.stride[0] = nj * nk;
        a.stride[1] = nk;
        a.stride[2] = 1;
    }
    if (precision == FW_F64)
        launch<double>(stencil, a, w_out, stream);
    else
        launch<float>(stencil, a, w_out, stream);
    FW_CHECK_LAUNCH("fw_build_weights launch");
    return FW_OK;
}

}  // namespace fw
