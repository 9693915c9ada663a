/*
 * fw_oracle.c -- CPU restatement of Finitewave's explicit monodomain step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU library is
 * checked against, and the CPU baseline that the benchmark times beside it.
 * Nothing in the product links or calls it.
 *
 * Every routine below restates one numba kernel of the reference (file:line
 * cited per function) in plain C99 with the reference's operation order kept
 * term by term, so that with `-O2 -fno-fast-math -ffp-contract=off` the
 * float64 results are bitwise those of the reference's float64 arithmetic
 * for the parts that use only + - * / (weights, diffusion, Aliev-Panfilov).
 * Models with exp/log/tanh call the C library, as the reference's numba JIT
 * does; they agree with the pure-Python reference run to a few ulp per call.
 * The `prange` loops of the reference become OpenMP `parallel for` loops.
 *
 * All arrays are C-order.  2D arrays are (ni, nj); 3D arrays are
 * (ni, nj, nk); per-node weights are (..., nw) with the stencil's own point
 * order.  `idx` is the flat myocyte index list (`myo_indexes`).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EXPORT __attribute__((visibility("default")))

EXPORT int fwo_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* half-step coefficients                                              */
/* ------------------------------------------------------------------ */

/* IsotropicStencil2D.compute_half_step_diffusion
 * (cpuwave2D/stencil/isotropic_stencil_2d.py:71-94):
 * D[ax] = 0.5 * (c + roll(c, -1, axis=ax)), roll wraps around. */
static void half_iso(const double *c, const int64_t *shape, int ndim, int ax,
                     double *out)
{
    int64_t n = 1;
    for (int d = 0; d < ndim; ++d) n *= shape[d];
    int64_t stride = 1;
    for (int d = ndim - 1; d > ax; --d) stride *= shape[d];
    int64_t len = shape[ax];
    #pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
        int64_t coord = (p / stride) % len;
        int64_t q = (coord + 1 == len) ? p - coord * stride : p + stride;
        out[p] = 0.5 * (c[p] + c[q]);
    }
}

/* AsymmetricStencil2D.compute_half_step_diffusion + compute_diffusion_
 * components (cpuwave2D/stencil/asymmetric_stencil_2d.py:97-161), shared by
 * the 3D stencil (cpuwave3D/stencil/asymmetric_stencil_3d.py:83-91):
 * comp = D_ac*(a0==a1) + (D_al-D_ac)*f[...,a0]*f[...,a1];
 * out  = 0.5*(comp*c + roll(comp,-1,axis=ax)*roll(c,-1,axis=ax)). */
static double dcomp(const double *f, int64_t p, int ncomp, int a0, int a1,
                    double D_al, double D_ac)
{
    double diag = D_ac * (double)(a0 == a1);
    return diag + (D_al - D_ac) * f[p * ncomp + a0] * f[p * ncomp + a1];
}

static void half_aniso(const double *c, const double *f, const int64_t *shape,
                       int ndim, int ax, int comp, double D_al, double D_ac,
                       double *out)
{
    int64_t n = 1;
    for (int d = 0; d < ndim; ++d) n *= shape[d];
    int64_t stride = 1;
    for (int d = ndim - 1; d > ax; --d) stride *= shape[d];
    int64_t len = shape[ax];
    #pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
        int64_t coord = (p / stride) % len;
        int64_t q = (coord + 1 == len) ? p - coord * stride : p + stride;
        double dp = dcomp(f, p, ndim, ax, comp, D_al, D_ac);
        double dq = dcomp(f, q, ndim, ax, comp, D_al, D_ac);
        out[p] = 0.5 * (dp * c[p] + dq * c[q]);
    }
}

/* weights * D_model * dt / dr**2, then +1 on the centre.  dr2 is the
 * caller's `dr**2` as Python computes it (libm pow, which differs from dr*dr
 * in the last ulp for some dr)
 * (isotropic_stencil_2d.py:66-67, asymmetric_stencil_2d.py:81-82, and the
 * 3D equivalents). */
static void scale_weights(double *w, int64_t n, int nw, int centre,
                          double D_model, double dt, double dr2)
{
    #pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
        for (int k = 0; k < nw; ++k)
            w[p * nw + k] = w[p * nw + k] * D_model * dt / dr2;
        w[p * nw + centre] += 1.0;
    }
}

static inline int m01(const int8_t *mesh, int64_t p) { return mesh[p] == 1; }

/* ------------------------------------------------------------------ */
/* isotropic weights                                                    */
/* ------------------------------------------------------------------ */

/* compute_component (isotropic_stencil_2d.py:135-158): d*m0*(m0+(m1==0)) */
static inline double icomp(double d, int m0, int m1)
{
    return d * (double)m0 * (double)(m0 + (m1 == 0));
}

/* IsotropicStencil2D.compute_weights (isotropic_stencil_2d.py:41-69,
 * 161-204).  Order: (i-1,j), (i,j-1), (i,j), (i,j+1), (i+1,j). */
EXPORT void fwo_weights_2d_iso5(const int8_t *mesh, const double *cond,
                                int64_t ni, int64_t nj, double D_model,
                                double dt, double dr2, double *w)
{
    int64_t n = ni * nj, shape[2] = {ni, nj};
    double *dxx = malloc(sizeof(double) * n), *dyy = malloc(sizeof(double) * n);
    half_iso(cond, shape, 2, 0, dxx);
    half_iso(cond, shape, 2, 1, dyy);
    memset(w, 0, sizeof(double) * n * 5);
    #pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
        int64_t i = p / nj, j = p % nj;
        if (!m01(mesh, p)) continue;
        int64_t im = (i - 1) * nj + j, ip = (i + 1) * nj + j;
        int64_t jm = i * nj + j - 1, jp = i * nj + j + 1;
        double *o = w + p * 5;
        o[0] = icomp(dxx[im], m01(mesh, im), m01(mesh, ip));
        o[1] = icomp(dyy[jm], m01(mesh, jm), m01(mesh, jp));
        o[3] = icomp(dyy[p], m01(mesh, jp), m01(mesh, jm));
        o[4] = icomp(dxx[p], m01(mesh, ip), m01(mesh, im));
        o[2] = -(o[0] + o[1] + o[3] + o[4]);
    }
    scale_weights(w, n, 5, 2, D_model, dt, dr2);
    free(dxx);
    free(dyy);
}

/* IsotropicStencil3D.compute_weights (cpuwave3D/stencil/isotropic_stencil_3d
 * .py:45-74, 113-149).  Order: (i-1), (j-1), (k-1), c, (k+1), (j+1), (i+1). */
EXPORT void fwo_weights_3d_iso7(const int8_t *mesh, const double *cond,
                                int64_t ni, int64_t nj, int64_t nk,
                                double D_model, double dt, double dr2,
                                double *w)
{
    int64_t n = ni * nj * nk, shape[3] = {ni, nj, nk};
    double *dxx = malloc(sizeof(double) * n), *dyy = malloc(sizeof(double) * n),
           *dzz = malloc(sizeof(double) * n);
    half_iso(cond, shape, 3, 0, dxx);
    half_iso(cond, shape, 3, 1, dyy);
    half_iso(cond, shape, 3, 2, dzz);
    memset(w, 0, sizeof(double) * n * 7);
    int64_t si = nj * nk, sj = nk;
    #pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
        if (!m01(mesh, p)) continue;
        double *o = w + p * 7;
        o[0] = icomp(dxx[p - si], m01(mesh, p - si), m01(mesh, p + si));
        o[1] = icomp(dyy[p - sj], m01(mesh, p - sj), m01(mesh, p + sj));
        o[2] = icomp(dzz[p - 1], m01(mesh, p - 1), m01(mesh, p + 1));
        o[4] = icomp(dzz[p], m01(mesh, p + 1), m01(mesh, p - 1));
        o[5] = icomp(dyy[p], m01(mesh, p + sj), m01(mesh, p - sj));
        o[6] = icomp(dxx[p], m01(mesh, p + si), m01(mesh, p - si));
        o[3] = -(o[0] + o[1] + o[2] + o[4] + o[5] + o[6]);
    }
    scale_weights(w, n, 7, 3, D_model, dt, dr2);
    free(dxx);
    free(dyy);
    free(dzz);
}

/* ------------------------------------------------------------------ */
/* anisotropic weights                                                  */
/* ------------------------------------------------------------------ */

/* minor_component (asymmetric_stencil_2d.py:204-259).  r[0..5] get the six
 * point weights, all zero when the face is not fully inside tissue. */
static inline void minor(double d, int m0, int m1, int m2, int m3, int m4,
                         int m5, double r[6])
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

/* AsymmetricStencil2D.compute_weights (asymmetric_stencil_2d.py:46-84) and
 * the njit accumulation (asymmetric_stencil_2d.py:291-433).  Point order
 * (i-1,j-1), (i-1,j), (i-1,j+1), (i,j-1), (i,j), (i,j+1), (i+1,j-1),
 * (i+1,j), (i+1,j+1).  fibers is (ni, nj, 2). */
EXPORT void fwo_weights_2d_aniso9(const int8_t *mesh, const double *cond,
                                  const double *fibers, int64_t ni, int64_t nj,
                                  double D_al, double D_ac, double D_model,
                                  double dt, double dr2, double *w)
{
    int64_t n = ni * nj, shape[2] = {ni, nj};
    double *dxx = malloc(sizeof(double) * n), *dxy = malloc(sizeof(double) * n),
           *dyx = malloc(sizeof(double) * n), *dyy = malloc(sizeof(double) * n);
    half_aniso(cond, fibers, shape, 2, 0, 0, D_al, D_ac, dxx);
    half_aniso(cond, fibers, shape, 2, 0, 1, D_al, D_ac, dxy);
    half_aniso(cond, fibers, shape, 2, 1, 0, D_al, D_ac, dyx);
    half_aniso(cond, fibers, shape, 2, 1, 1, D_al, D_ac, dyy);
    memset(w, 0, sizeof(double) * n * 9);
    #pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
        if (!m01(mesh, p)) continue;
        int64_t i = p / nj, j = p % nj;
#define M(a, b) m01(mesh, (i + (a)) * nj + (j + (b)))
#define AT(arr, a, b) arr[(i + (a)) * nj + (j + (b))]
        double *o = w + p * 9, r[6], q;
        /* q (i-1/2, j) */
        q = AT(dxx, -1, 0) * (double)M(-1, 0);
        o[1] += q; o[4] -= q;
        minor(AT(dxy, -1, 0), M(-1, -1), M(0, -1), M(-1, 0), M(0, 0),
              M(-1, 1), M(0, 1), r);
        o[0] -= r[0]; o[3] -= r[1]; o[1] -= r[2];
        o[4] -= r[3]; o[2] -= r[4]; o[5] -= r[5];
        /* q (i, j-1/2) */
        q = AT(dyy, 0, -1) * (double)M(0, -1);
        o[3] += q; o[4] -= q;
        minor(AT(dyx, 0, -1), M(-1, -1), M(-1, 0), M(0, -1), M(0, 0),
              M(1, -1), M(1, 0), r);
        o[0] -= r[0]; o[1] -= r[1]; o[3] -= r[2];
        o[4] -= r[3]; o[6] -= r[4]; o[7] -= r[5];
        /* q (i, j+1/2) */
        q = AT(dyy, 0, 0) * (double)M(0, 1);
        o[5] += q; o[4] -= q;
        minor(AT(dyx, 0, 0), M(-1, 1), M(-1, 0), M(0, 1), M(0, 0),
              M(1, 1), M(1, 0), r);
        o[2] += r[0]; o[1] += r[1]; o[5] += r[2];
        o[4] += r[3]; o[8] += r[4]; o[7] += r[5];
        /* q (i+1/2, j) */
        q = AT(dxx, 0, 0) * (double)M(1, 0);
        o[7] += q; o[4] -= q;
        minor(AT(dxy, 0, 0), M(1, -1), M(0, -1), M(1, 0), M(0, 0),
              M(1, 1), M(0, 1), r);
        o[6] += r[0]; o[3] += r[1]; o[7] += r[2];
        o[4] += r[3]; o[8] += r[4]; o[5] += r[5];
#undef M
#undef AT
    }
    scale_weights(w, n, 9, 4, D_model, dt, dr2);
    free(dxx); free(dxy); free(dyx); free(dyy);
}

/* AsymmetricStencil3D.compute_weights (cpuwave3D/stencil/asymmetric_
 * stencil_3d.py:61-105) and its serial njit accumulation (:164-458).
 * Point order is the 19-entry list at asymmetric_stencil_3d.py:25-44.
 * fibers is (ni, nj, nk, 3). */
EXPORT void fwo_weights_3d_aniso19(const int8_t *mesh, const double *cond,
                                   const double *fibers, int64_t ni,
                                   int64_t nj, int64_t nk, double D_al,
                                   double D_ac, double D_model, double dt,
                                   double dr2, double *w)
{
    int64_t n = ni * nj * nk, shape[3] = {ni, nj, nk};
    double *d[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            d[a][b] = malloc(sizeof(double) * n);
            half_aniso(cond, fibers, shape, 3, a, b, D_al, D_ac, d[a][b]);
        }
    memset(w, 0, sizeof(double) * n * 19);
    #pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
        if (!m01(mesh, p)) continue;
        int64_t i = p / (nj * nk), j = (p / nk) % nj, k = p % nk;
#define M(a, b, c) m01(mesh, ((i + (a)) * nj + (j + (b))) * nk + (k + (c)))
#define AT(x, y, a, b, c) d[x][y][((i + (a)) * nj + (j + (b))) * nk + (k + (c))]
        double *o = w + p * 19, r[6], q;
        /* q (i-1/2, j, k) */
        q = AT(0, 0, -1, 0, 0) * (double)M(-1, 0, 0);
        o[1] += q; o[4] -= q;
        minor(AT(0, 1, -1, 0, 0), M(-1, -1, 0), M(0, -1, 0), M(-1, 0, 0),
              M(0, 0, 0), M(-1, 1, 0), M(0, 1, 0), r);
        o[0] -= r[0]; o[3] -= r[1]; o[1] -= r[2];
        o[4] -= r[3]; o[2] -= r[4]; o[5] -= r[5];
        minor(AT(0, 2, -1, 0, 0), M(-1, 0, -1), M(0, 0, -1), M(-1, 0, 0),
              M(0, 0, 0), M(-1, 0, 1), M(0, 0, 1), r);
        o[15] -= r[0]; o[11] -= r[1]; o[1] -= r[2];
        o[4] -= r[3]; o[17] -= r[4]; o[12] -= r[5];
        /* q (i+1/2, j, k) */
        q = AT(0, 0, 0, 0, 0) * (double)M(1, 0, 0);
        o[7] += q; o[4] -= q;
        minor(AT(0, 1, 0, 0, 0), M(1, -1, 0), M(0, -1, 0), M(1, 0, 0),
              M(0, 0, 0), M(1, 1, 0), M(0, 1, 0), r);
        o[6] += r[0]; o[3] += r[1]; o[7] += r[2];
        o[4] += r[3]; o[8] += r[4]; o[5] += r[5];
        minor(AT(0, 2, 0, 0, 0), M(1, 0, -1), M(0, 0, -1), M(1, 0, 0),
              M(0, 0, 0), M(1, 0, 1), M(0, 0, 1), r);
        o[16] += r[0]; o[11] += r[1]; o[7] += r[2];
        o[4] += r[3]; o[18] += r[4]; o[12] += r[5];
        /* q (i, j-1/2, k) */
        q = AT(1, 1, 0, -1, 0) * (double)M(0, -1, 0);
        o[3] += q; o[4] -= q;
        minor(AT(1, 0, 0, -1, 0), M(-1, -1, 0), M(-1, 0, 0), M(0, -1, 0),
              M(0, 0, 0), M(1, -1, 0), M(1, 0, 0), r);
        o[0] -= r[0]; o[1] -= r[1]; o[3] -= r[2];
        o[4] -= r[3]; o[6] -= r[4]; o[7] -= r[5];
        minor(AT(1, 2, 0, -1, 0), M(0, -1, -1), M(0, 0, -1), M(0, -1, 0),
              M(0, 0, 0), M(0, -1, 1), M(0, 0, 1), r);
        o[9] -= r[0]; o[11] -= r[1]; o[3] -= r[2];
        o[4] -= r[3]; o[10] -= r[4]; o[12] -= r[5];
        /* q (i, j+1/2, k) */
        q = AT(1, 1, 0, 0, 0) * (double)M(0, 1, 0);
        o[5] += q; o[4] -= q;
        minor(AT(1, 0, 0, 0, 0), M(-1, 1, 0), M(-1, 0, 0), M(0, 1, 0),
              M(0, 0, 0), M(1, 1, 0), M(1, 0, 0), r);
        o[2] += r[0]; o[1] += r[1]; o[5] += r[2];
        o[4] += r[3]; o[8] += r[4]; o[7] += r[5];
        minor(AT(1, 2, 0, 0, 0), M(0, 1, -1), M(0, 0, -1), M(0, 1, 0),
              M(0, 0, 0), M(0, 1, 1), M(0, 0, 1), r);
        o[13] += r[0]; o[11] += r[1]; o[5] += r[2];
        o[4] += r[3]; o[14] += r[4]; o[12] += r[5];
        /* q (i, j, k-1/2) */
        q = AT(2, 2, 0, 0, -1) * (double)M(0, 0, -1);
        o[11] += q; o[4] -= q;
        minor(AT(2, 0, 0, 0, -1), M(-1, 0, -1), M(-1, 0, 0), M(0, 0, -1),
              M(0, 0, 0), M(1, 0, -1), M(1, 0, 0), r);
        o[15] -= r[0]; o[1] -= r[1]; o[11] -= r[2];
        o[4] -= r[3]; o[16] -= r[4]; o[7] -= r[5];
        minor(AT(2, 1, 0, 0, -1), M(0, -1, -1), M(0, -1, 0), M(0, 0, -1),
              M(0, 0, 0), M(0, 1, -1), M(0, 1, 0), r);
        o[9] -= r[0]; o[3] -= r[1]; o[11] -= r[2];
        o[4] -= r[3]; o[13] -= r[4]; o[5] -= r[5];
        /* q (i, j, k+1/2) */
        q = AT(2, 2, 0, 0, 0) * (double)M(0, 0, 1);
        o[12] += q; o[4] -= q;
        minor(AT(2, 0, 0, 0, 0), M(-1, 0, 1), M(-1, 0, 0), M(0, 0, 1),
              M(0, 0, 0), M(1, 0, 1), M(1, 0, 0), r);
        o[17] += r[0]; o[1] += r[1]; o[12] += r[2];
        o[4] += r[3]; o[18] += r[4]; o[7] += r[5];
        minor(AT(2, 1, 0, 0, 0), M(0, -1, 1), M(0, -1, 0), M(0, 0, 1),
              M(0, 0, 0), M(0, 1, 1), M(0, 1, 0), r);
        o[10] += r[0]; o[3] += r[1]; o[12] += r[2];
        o[4] += r[3]; o[14] += r[4]; o[5] += r[5];
#undef M
#undef AT
    }
    scale_weights(w, n, 19, 4, D_model, dt, dr2);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) free(d[a][b]);
}

/* ------------------------------------------------------------------ */
/* diffusion                                                            */
/* ------------------------------------------------------------------ */

/* diffusion_kernel_2d_iso (isotropic_stencil_2d.py:97-132) */
EXPORT void fwo_diffuse_2d_iso5(double *un, const double *u, const double *w,
                                const int64_t *idx, int64_t n_idx, int64_t ni,
                                int64_t nj)
{
    (void)ni;
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        int64_t p = idx[t];
        const double *o = w + p * 5;
        un[p] = u[p - nj] * o[0] + u[p - 1] * o[1] + u[p] * o[2] +
                u[p + 1] * o[3] + u[p + nj] * o[4];
    }
}

/* diffusion_kernel_2d_aniso (asymmetric_stencil_2d.py:164-201) */
EXPORT void fwo_diffuse_2d_aniso9(double *un, const double *u, const double *w,
                                  const int64_t *idx, int64_t n_idx,
                                  int64_t ni, int64_t nj)
{
    (void)ni;
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        int64_t p = idx[t];
        const double *o = w + p * 9;
        un[p] = u[p - nj - 1] * o[0] + u[p - nj] * o[1] + u[p - nj + 1] * o[2] +
                u[p - 1] * o[3] + u[p] * o[4] + u[p + 1] * o[5] +
                u[p + nj - 1] * o[6] + u[p + nj] * o[7] + u[p + nj + 1] * o[8];
    }
}

/* diffusion_kernel_3d_iso (cpuwave3D/stencil/isotropic_stencil_3d.py:78-109) */
EXPORT void fwo_diffuse_3d_iso7(double *un, const double *u, const double *w,
                                const int64_t *idx, int64_t n_idx, int64_t ni,
                                int64_t nj, int64_t nk)
{
    (void)ni;
    int64_t si = nj * nk, sj = nk;
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        int64_t p = idx[t];
        const double *o = w + p * 7;
        un[p] = u[p - si] * o[0] + u[p - sj] * o[1] + u[p - 1] * o[2] +
                u[p] * o[3] + u[p + 1] * o[4] + u[p + sj] * o[5] +
                u[p + si] * o[6];
    }
}

/* diffusion_kernel_3d_aniso (cpuwave3D/stencil/asymmetric_stencil_3d.py:
 * 108-160) */
EXPORT void fwo_diffuse_3d_aniso19(double *un, const double *u,
                                   const double *w, const int64_t *idx,
                                   int64_t n_idx, int64_t ni, int64_t nj,
                                   int64_t nk)
{
    (void)ni;
    int64_t si = nj * nk, sj = nk;
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        int64_t p = idx[t];
        const double *o = w + p * 19;
        un[p] = u[p - si - sj] * o[0] + u[p - si] * o[1] +
                u[p - si + sj] * o[2] + u[p - sj] * o[3] + u[p] * o[4] +
                u[p + sj] * o[5] + u[p + si - sj] * o[6] + u[p + si] * o[7] +
                u[p + si + sj] * o[8] + u[p - sj - 1] * o[9] +
                u[p - sj + 1] * o[10] + u[p - 1] * o[11] + u[p + 1] * o[12] +
                u[p + sj - 1] * o[13] + u[p + sj + 1] * o[14] +
                u[p - si - 1] * o[15] + u[p + si - 1] * o[16] +
                u[p - si + 1] * o[17] + u[p + si + 1] * o[18];
    }
}

/* ------------------------------------------------------------------ */
/* ionic models (node-local; the 2D and 3D kernels share one formula)    */
/* ------------------------------------------------------------------ */

/* Aliev-Panfilov: calc_v + ionic_kernel_2d (cpuwave2D/model/
 * aliev_panfilov_2d.py:337-406; 3D: cpuwave3D/model/aliev_panfilov_3d.py:
 * 53-84). */
EXPORT void fwo_ionic_ap(double *un, const double *u, double *v,
                         const int64_t *idx, int64_t n_idx, double dt,
                         double a, double k, double eap, double mu_1,
                         double mu_2)
{
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        int64_t p = idx[t];
        double uu = u[p], vv = v[p];
        vv += (-dt) * (eap + (mu_1 * vv) / (mu_2 + uu)) *
              (vv + k * uu * (uu - a - 1.0));
        v[p] = vv;
        un[p] += dt * ((-k) * uu * (uu - a) * (uu - 1.0) - uu * vv);
    }
}

/* Mitchell-Schaeffer: calc_h, calc_J_in, calc_J_out, ionic_kernel_2d
 * (cpuwave2D/model/mitchell_schaeffer_2d.py:102-217). */
EXPORT void fwo_ionic_ms(double *un, const double *u, double *h,
                         const int64_t *idx, int64_t n_idx, double dt,
                         double tau_close, double tau_open, double tau_in,
                         double tau_out, double u_gate)
{
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        int64_t p = idx[t];
        double uu = u[p], hh = h[p];
        hh += (uu < u_gate) ? dt * (1.0 - hh) / tau_open
                            : dt * (-hh) / tau_close;
        h[p] = hh;
        double C = (uu * uu) * (1.0 - uu);
        double J_in = hh * C / tau_in;
        double J_out = -uu / tau_out;
        un[p] += dt * (J_in + J_out);
    }
}

/* Fenton-Karma: calc_Jfi, calc_Jso, calc_Jsi, calc_v, calc_w,
 * ionic_kernel_2d (cpuwave2D/model/fenton_karma_2d.py:143-328).  As in the
 * reference (fenton_karma_2d.py:326), J_si is evaluated with v, not w. */
EXPORT void fwo_ionic_fk(double *un, const double *u, double *v, double *w,
                         const int64_t *idx, int64_t n_idx, double dt,
                         double tau_d, double tau_o, double tau_r,
                         double tau_si, double tau_v_m, double tau_v_p,
                         double tau_w_m, double tau_w_p, double k, double u_c,
                         double uc_si)
{
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_idx; ++t) {
        int64_t p = idx[t];
        double uu = u[p], vv = v[p], ww = w[p];
        double H1 = (u_c - uu) >= 0 ? 1.0 : 0.0;
        double H2 = (uu - u_c) >= 0 ? 1.0 : 0.0;
        vv += dt * (H1 * (1.0 - vv) / tau_v_m - H2 * vv / tau_v_p);
        ww += dt * (H1 * (1.0 - ww) / tau_w_m - H2 * ww / tau_w_p);
        v[p] = vv;
        w[p] = ww;
        double H = (uu - u_c) >= 0 ? 1.0 : 0.0;
        double J_fi = -(vv * H * (1.0 - uu) * (uu - u_c)) / tau_d;
        double J_so = uu * H1 / tau_o + H2 / tau_r;
        double J_si = (-vv) * (1.0 + tanh(k * (uu - uc_si))) / (2.0 * tau_si);
        un[p] += dt * (-J_fi - J_so - J_si);
    }
}

/* compute_ecg (cpuwave2D/tracker/ecg_2d_tracker.py:114-153 with dim 2,
 * cpuwave3D/tracker/ecg_3d_tracker.py:99-140 with dim 3): for every lead c,
 * the sum over myocytes in index order of (u_tr - u) / (d * dr) where d > 0.
 * Sequential: the reference's pure-Python order. */
EXPORT void fwo_ecg(const double *u_tr, const double *u, const double *coords,
                    int64_t n_c, double dr, const int64_t *idx, int64_t n_idx,
                    int64_t nj, int64_t nk, int dim, double *out)
{
    for (int64_t c = 0; c < n_c; ++c) {
        const double x = coords[3 * c], y = coords[3 * c + 1],
                     z = coords[3 * c + 2];
        double acc = 0.0;
        for (int64_t t = 0; t < n_idx; ++t) {
            const int64_t ii = idx[t];
            double i, j, k;
            if (dim == 2) {
                i = (double)(ii / nj);
                j = (double)(ii % nj);
                k = 0.0;
            } else {
                i = (double)(ii / (nj * nk));
                j = (double)((ii % (nj * nk)) / nk);
                k = (double)((ii % (nj * nk)) % nk);
            }
            const double d = dim == 2
                                 ? (x - i) * (x - i) + (y - j) * (y - j) + z * z
                                 : (x - i) * (x - i) + (y - j) * (y - j) +
                                       (z - k) * (z - k);
            if (d > 0) acc += (u_tr[ii] - u[ii]) / (d * dr);
        }
        out[c] = acc;
    }
}

/* SymmetricStencil2D.compute_weights (cpuwave2D/stencil/symmetric_stencil_2d.
 * py:31-250): D * conductivity averaged to the cell corners with np.roll
 * wrap, compute_components per corner cell, accumulated in the reference's
 * corner order, then weights *= (D_model * dt / dr**2) and +1 on w[4]. */
static void sym_corner(double dxx, double dxy, double dyx, double dyy, int m0,
                       int m1, int m2, int m3, int qx, int qy, double r[4])
{
    if (m0 + m1 + m2 + m3 < 3) {
        r[0] = r[1] = r[2] = r[3] = 0.0;
        return;
    }
    const double qdx = qx * dxx + qy * dyx;
    const double qdy = qx * dxy + qy * dyy;
    const double d0 = m0, d1 = m1, d2 = m2, d3 = m3;
    r[0] = 0.5 * ((-d0) / (d0 + d1) * qdx - d0 / (d0 + d2) * qdy);
    r[1] = 0.5 * ((-d1) / (d0 + d1) * qdx + d1 / (d1 + d3) * qdy);
    r[2] = 0.5 * (d2 / (d2 + d3) * qdx - d2 / (d0 + d2) * qdy);
    r[3] = 0.5 * (d3 / (d2 + d3) * qdx + d3 / (d1 + d3) * qdy);
}

EXPORT void fwo_weights_2d_sym9(const int8_t *mesh, const double *cond,
                                const double *fibers, int64_t ni, int64_t nj,
                                double D_al, double D_ac, double D_model,
                                double dt, double dr2, double *w)
{
    const int64_t n = ni * nj;
    const int64_t shape[2] = {ni, nj};
    double *D[4];
    for (int c = 0; c < 4; ++c) {
        D[c] = (double *)malloc(sizeof(double) * n);
        double *Dn = (double *)malloc(sizeof(double) * n);
        const int c0 = c / 2, c1 = c % 2;
        for (int64_t p = 0; p < n; ++p)
            Dn[p] = dcomp(fibers, p, 2, c0, c1, D_al, D_ac) * cond[p];
        for (int64_t i = 0; i < ni; ++i)
            for (int64_t j = 0; j < nj; ++j) {
                const int64_t i1 = (i + 1) % ni, j1 = (j + 1) % nj;
                D[c][i * nj + j] = 0.25 * (Dn[i * nj + j] + Dn[i1 * nj + j] +
                                           Dn[i * nj + j1] + Dn[i1 * nj + j1]);
            }
        free(Dn);
    }
    (void)shape;
#define M(i, j) (mesh[(i) * nj + (j)] == 1)
    for (int64_t p = 0; p < n * 9; ++p) w[p] = 0.0;
    const double scale = D_model * dt / dr2;
    for (int64_t i = 1; i + 1 < ni; ++i)
        for (int64_t j = 1; j + 1 < nj; ++j) {
            if (!M(i, j)) continue;
            double *o = w + (i * nj + j) * 9, r[4];
            int64_t q = (i - 1) * nj + (j - 1);
            sym_corner(D[0][q], D[1][q], D[2][q], D[3][q], M(i - 1, j - 1),
                       M(i - 1, j), M(i, j - 1), M(i, j), -1, -1, r);
            o[0] += r[0]; o[1] += r[1]; o[3] += r[2]; o[4] += r[3];
            q = (i - 1) * nj + j;
            sym_corner(D[0][q], D[1][q], D[2][q], D[3][q], M(i - 1, j),
                       M(i - 1, j + 1), M(i, j), M(i, j + 1), -1, 1, r);
            o[1] += r[0]; o[2] += r[1]; o[4] += r[2]; o[5] += r[3];
            q = i * nj + (j - 1);
            sym_corner(D[0][q], D[1][q], D[2][q], D[3][q], M(i, j - 1),
                       M(i, j), M(i + 1, j - 1), M(i + 1, j), 1, -1, r);
            o[3] += r[0]; o[4] += r[1]; o[6] += r[2]; o[7] += r[3];
            q = i * nj + j;
            sym_corner(D[0][q], D[1][q], D[2][q], D[3][q], M(i, j),
                       M(i, j + 1), M(i + 1, j), M(i + 1, j + 1), 1, 1, r);
            o[4] += r[0]; o[5] += r[1]; o[7] += r[2]; o[8] += r[3];
        }
#undef M
    for (int64_t p = 0; p < n; ++p) {
        for (int k = 0; k < 9; ++k) w[p * 9 + k] *= scale;
        w[p * 9 + 4] += 1.0;
    }
    for (int c = 0; c < 4; ++c) free(D[c]);
}
