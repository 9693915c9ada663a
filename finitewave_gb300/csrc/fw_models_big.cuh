// fw_models_big.cuh -- the detailed ionic models: ten Tusscher-Panfilov 2006
// (TP06) and Courtemanche 1998, in the interface of fw_models.cuh.
//
// Template parameter T is the type of the potential, the gates, the
// currents and the concentration rates; the ion-concentration state (TP06:
// Ca_i, Ca_SR, Ca_ss, Na_i, K_i; Courtemanche: Na_i, K_i, Ca_i, Ca_up,
// Ca_rel; Luo-Rudy 1991: Ca_i) takes 8 bytes per node in both forms.  Under
// FW_F64 every quantity is float64 and the expressions follow the
// reference's evaluation order, with CUDA's exp/log/sqrt/pow (a few ulp from
// the C library's).  Under FW_F32 everything is computed in float32 from the
// concentrations rounded to float, and the accumulation `c += dt * rate`
// -- increments ~1e-6 of the value, below float32's resolution -- is
// compensated (CPair below), so no float64 arithmetic (a small fraction of
// GB300's float32 rate) is left in the per-node work.
//
// Reference quirks kept: TP06 never updates Ca_i (tp06_2d.py:1098 assigns the
// new value and then the old one); Courtemanche's IKr conductance is fixed
// at 0.0294 (courtemanche_2d.py:420-422) and the model's `xs` array is the
// IKr gate, `xr` the IKs gate (its run_ionic_kernel passes xr, xs to the
// kernel's xs, xr arguments, courtemanche_2d.py:152-160 against :581).
#pragma once

#include <math.h>
#include <stdint.h>

#include "fw_models.cuh"

namespace fw {

// Transcendentals of the two precisions.  float64: CUDA's exp / log / pow
// (the reference's expressions, within a few ulp of the C library).
// float32: the SFU forms (__expf, __logf: a few ulp, growing by about one
// ulp per unit of |x| for exp, CUDA's documented bound) and the integer and
// half-integer powers as products -- the float32 form is compared with
// float64 by tolerance, and these calls are most of its instructions.
__device__ __forceinline__ float mexp(float x) { return __expf(x); }
__device__ __forceinline__ double mexp(double x) { return exp(x); }
__device__ __forceinline__ float mlog(float x) { return __logf(x); }
__device__ __forceinline__ double mlog(double x) { return log(x); }
// x / (e^x - 1), continuous through x = 0 where it is 1.  Several rates are
// written in the reference as a difference quotient such as
// (u - u0) / (exp(k (u - u0)) - 1), which is 0 / 0 at u = u0; in float64
// that point is never met in practice, but in float32 the exponential
// rounds to exactly 1 within ~1e-6 mV of u0 and the quotient becomes
// inf or NaN.  The float32 forms use this function instead (series
// 1 - x / 2 for |x| < 1e-4, where the next term is below 1e-9).
__device__ __forceinline__ float x_expm1(float x)
{
    return fabsf(x) < 1e-4f ? 1.f - 0.5f * x : x / expm1f(x);
}

__device__ __forceinline__ float pow3(float x) { return x * x * x; }
__device__ __forceinline__ double pow3(double x) { return pow(x, 3.0); }
__device__ __forceinline__ float pow15(float x) { return x * sqrtf(x); }
__device__ __forceinline__ double pow15(double x) { return pow(x, 1.5); }

// Instantaneous buffering (Rapid buffer approximation): the free
// concentration c after adding d to the total c + B c / (c + K) solves
// c^2 + (B - T + K) c - K T = 0 with T = c0 + B c0 / (c0 + K) + d
// (tp06_2d.py:793-873).  With c = c0 + delta the constant term becomes
// -(c0 + K) d, so delta solves delta^2 + p delta - (c0 + K) d = 0 with
// p = c0 + K + B K / (c0 + K) - d; its root near zero, in the form without
// cancellation, is 2 (c0 + K) d / (p + sqrt(p^2 + 4 (c0 + K) d)).
__device__ __forceinline__ float buffered_step(float c0, float B, float K,
                                               float d)
{
    const float kc = c0 + K;
    const float p = kc + B * K / kc - d;
    const float q = kc * d;
    return 2.f * q / (p + sqrtf(fmaxf(p * p + 4.f * q, 0.f)));
}

// ---------------------------------------------------------------- accumulators
// The ion-concentration accumulators.  float64 form: a double.  float32
// form: a compensated pair of floats, the value hi + lo with |lo| at most
// half an ulp of hi (about 48 bits of mantissa), kept in the 8 bytes per
// node a double would take (float2 per node).  An increment d, ~1e-7 of the
// value and below float32's resolution of it, is added with Knuth's
// two-sum error-free transformation -- the rounding error of hi + d is
// recovered exactly and carried in lo -- so the accumulation runs on the
// float32 pipe (GB300's float64 rate is a small fraction of it).  The
// rates see the value rounded to float (hi).
struct CPair {
    float hi, lo;
    __device__ __forceinline__ explicit operator float() const { return hi; }
    __device__ __forceinline__ CPair &operator+=(float d)
    {
        const float s = hi + d;
        const float bp = s - hi;
        const float e = (hi - (s - bp)) + (d - bp);
        const float l = lo + e;
        hi = s + l;
        lo = l - (hi - s);
        return *this;
    }
};

template <class T>
struct ConcOf {
    using type = double;
};
template <>
struct ConcOf<float> {
    using type = CPair;
};
template <class T>
using Conc = typename ConcOf<T>::type;

__device__ __forceinline__ void conc_load(double &c, const void *a, int64_t p)
{
    c = ((const double *)a)[p];
}
__device__ __forceinline__ void conc_load(CPair &c, const void *a, int64_t p)
{
    const float2 v = ((const float2 *)a)[p];
    c.hi = v.x;
    c.lo = v.y;
}
__device__ __forceinline__ void conc_store(void *a, int64_t p, double c)
{
    ((double *)a)[p] = c;
}
__device__ __forceinline__ void conc_store(void *a, int64_t p, const CPair &c)
{
    ((float2 *)a)[p] = make_float2(c.hi, c.lo);
}
__device__ __forceinline__ double conc_probe(double c) { return c; }
__device__ __forceinline__ double conc_probe(const CPair &c)
{
    return (double)c.hi + (double)c.lo;
}

// ---------------------------------------------------------------- TP06
// Parameters in the order of tp06_2d.py's ionic_kernel_2d signature
// (:1003-1012); state in TP062D.state_vars order minus u (:77-79).
struct ModelTP06 {
    static constexpr int NS = 19, NP = 49;
    static constexpr int kMinBlocksF32 = 4;  // 64 registers, no spills
    enum {
        ko, cao, nao, Vc, Vsr, Vss, Bufc, Kbufc, Bufsr, Kbufsr, Bufss, Kbufss,
        Vmaxup, Kup, Vrel, k1_, k2_, k3, k4, EC, maxsr, minsr, Vleak, Vxfer, R,
        F, T_, RTONF, CAPACITANCE, gkr, pKNa, gk1, gna, gbna, KmK, KmNa, knak,
        gcal, gbca, knaca, KmNai, KmCa, ksat, n_, gpca, KpCa, gpk, gto, gks
    };
    enum { s_cai, s_casr, s_cass, s_nai, s_Ki, s_m, s_h, s_j, s_xr1, s_xr2,
           s_xs, s_r, s_s, s_d, s_f, s_f2, s_fcass, s_rr, s_oo };
    static constexpr bool is_conc(int i) { return i <= s_Ki; }

    template <class T>
    struct St {
        Conc<T> cai, casr, cass, nai, Ki;
        T m, h, j, xr1, xr2, xs, r, s, d, f, f2, fcass, rr, oo;
    };
    template <class T>
    __device__ static __forceinline__ St<T> load(void *const *S, int64_t p)
    {
        St<T> x;
        conc_load(x.cai, S[s_cai], p);
        conc_load(x.casr, S[s_casr], p);
        conc_load(x.cass, S[s_cass], p);
        conc_load(x.nai, S[s_nai], p);
        conc_load(x.Ki, S[s_Ki], p);
        x.m = ((const T *)S[s_m])[p];
        x.h = ((const T *)S[s_h])[p];
        x.j = ((const T *)S[s_j])[p];
        x.xr1 = ((const T *)S[s_xr1])[p];
        x.xr2 = ((const T *)S[s_xr2])[p];
        x.xs = ((const T *)S[s_xs])[p];
        x.r = ((const T *)S[s_r])[p];
        x.s = ((const T *)S[s_s])[p];
        x.d = ((const T *)S[s_d])[p];
        x.f = ((const T *)S[s_f])[p];
        x.f2 = ((const T *)S[s_f2])[p];
        x.fcass = ((const T *)S[s_fcass])[p];
        x.rr = ((const T *)S[s_rr])[p];
        x.oo = ((const T *)S[s_oo])[p];
        return x;
    }
    template <class T>
    __device__ static __forceinline__ void store(void *const *S, int64_t p,
                                                 const St<T> &x)
    {
        // Ca_i is not written: the reference never changes it
        conc_store(S[s_casr], p, x.casr);
        conc_store(S[s_cass], p, x.cass);
        conc_store(S[s_nai], p, x.nai);
        conc_store(S[s_Ki], p, x.Ki);
        ((T *)S[s_m])[p] = x.m;
        ((T *)S[s_h])[p] = x.h;
        ((T *)S[s_j])[p] = x.j;
        ((T *)S[s_xr1])[p] = x.xr1;
        ((T *)S[s_xr2])[p] = x.xr2;
        ((T *)S[s_xs])[p] = x.xs;
        ((T *)S[s_r])[p] = x.r;
        ((T *)S[s_s])[p] = x.s;
        ((T *)S[s_d])[p] = x.d;
        ((T *)S[s_f])[p] = x.f;
        ((T *)S[s_f2])[p] = x.f2;
        ((T *)S[s_fcass])[p] = x.fcass;
        ((T *)S[s_rr])[p] = x.rr;
        ((T *)S[s_oo])[p] = x.oo;
    }
    template <class T>
    __device__ static __forceinline__ double probe(const St<T> &x, int i)
    {
        switch (i) {
        case s_cai: return conc_probe(x.cai);
        case s_casr: return conc_probe(x.casr);
        case s_cass: return conc_probe(x.cass);
        case s_nai: return conc_probe(x.nai);
        case s_Ki: return conc_probe(x.Ki);
        case s_m: return x.m;
        case s_h: return x.h;
        case s_j: return x.j;
        case s_xr1: return x.xr1;
        case s_xr2: return x.xr2;
        case s_xs: return x.xs;
        case s_r: return x.r;
        case s_s: return x.s;
        case s_d: return x.d;
        case s_f: return x.f;
        case s_f2: return x.f2;
        case s_fcass: return x.fcass;
        case s_rr: return x.rr;
        default: return x.oo;
        }
    }

    // ionic_kernel_2d and the calc_* helpers (tp06_2d.py:242-1103)
    template <class T>
    __device__ static __forceinline__ T update(T u, T un, St<T> &x,
                                               const Params<T, NP> &P, T dt)
    {
        const T c1 = (T)1.0;
        const T cass = (T)x.cass, cai = (T)x.cai, casr = (T)x.casr;
        const T nai = (T)x.nai, Ki = (T)x.Ki;
        const T inverseVcF = c1 / (P.v[Vc] * P.v[F]);
        const T inversevssF2 = c1 / ((T)2 * P.v[Vss] * P.v[F]);

        const T Ek = P.v[RTONF] * mlog(P.v[ko] / Ki);
        const T Ena = P.v[RTONF] * mlog(P.v[nao] / nai);
        const T Eks = P.v[RTONF] * mlog((P.v[ko] + P.v[pKNa] * P.v[nao]) /
                                          (Ki + P.v[pKNa] * nai));
        const T Eca = (T)0.5 * P.v[RTONF] * mlog(P.v[cao] / cai);

        // calc_ina
        T ina;
        {
            const T am = c1 / (c1 + mexp(((T)(-60.0) - u) / (T)5.0));
            const T beta_m = (T)0.1 / (c1 + mexp((u + (T)35.0) / (T)5.0)) +
                             (T)0.1 / (c1 + mexp((u - (T)50.0) / (T)200.0));
            const T tau_m = am * beta_m;
            const T e_m = mexp(((T)(-56.86) - u) / (T)9.03);
            const T m_inf = c1 / ((c1 + e_m) * (c1 + e_m));
            T alpha_h, beta_h, alpha_j, beta_j;
            if (u >= (T)(-40.0)) {
                alpha_h = (T)0;
                beta_h = (T)0.77 / ((T)0.13 * (c1 + mexp(-(u + (T)10.66) / (T)11.1)));
                alpha_j = (T)0;
                beta_j = (T)0.6 * mexp((T)0.057 * u) /
                         (c1 + mexp((T)(-0.1) * (u + (T)32.0)));
            } else {
                alpha_h = (T)0.057 * mexp(-(u + (T)80.0) / (T)6.8);
                beta_h = (T)2.7 * mexp((T)0.079 * u) +
                         (T)310000.0 * mexp((T)0.3485 * u);
                alpha_j = ((T)(-25428.0) * mexp((T)0.2444 * u) -
                           (T)6.948e-06 * mexp((T)(-0.04391) * u)) *
                          (u + (T)37.78) / (c1 + mexp((T)0.311 * (u + (T)79.23)));
                beta_j = (T)0.02424 * mexp((T)(-0.01052) * u) /
                         (c1 + mexp((T)(-0.1378) * (u + (T)40.14)));
            }
            const T tau_h = c1 / (alpha_h + beta_h);
            const T e_h = mexp((u + (T)71.55) / (T)7.43);
            const T h_inf = c1 / ((c1 + e_h) * (c1 + e_h));
            const T tau_j = c1 / (alpha_j + beta_j);
            const T j_inf = h_inf;
            x.m = m_inf - (m_inf - x.m) * mexp(-dt / tau_m);
            x.h = h_inf - (h_inf - x.h) * mexp(-dt / tau_h);
            x.j = j_inf - (j_inf - x.j) * mexp(-dt / tau_j);
            ina = P.v[gna] * x.m * x.m * x.m * x.h * x.j * (u - Ena);
        }
        // calc_ical
        T ical;
        {
            const T FF = P.v[F], RT = P.v[R] * P.v[T_];
            const T d_inf = c1 / (c1 + mexp(((T)(-8) - u) / (T)7.5));
            const T Ad = (T)1.4 / (c1 + mexp(((T)(-35) - u) / (T)13)) + (T)0.25;
            const T Bd = (T)1.4 / (c1 + mexp((u + (T)5) / (T)5));
            const T Cd = c1 / (c1 + mexp(((T)50 - u) / (T)20));
            const T tau_d = Ad * Bd + Cd;
            const T f_inf = c1 / (c1 + mexp((u + (T)20) / (T)7));
            const T Af = (T)1102.5 * mexp(-(u + (T)27) * (u + (T)27) / (T)225);
            const T Bf = (T)200.0 / (c1 + mexp(((T)13 - u) / (T)10.0));
            const T Cf = (T)180.0 / (c1 + mexp((u + (T)30) / (T)10)) + (T)20;
            const T tau_f = Af + Bf + Cf;
            const T f2_inf = (T)0.67 / (c1 + mexp((u + (T)35) / (T)7)) + (T)0.33;
            const T Af2 = (T)600 * mexp(-(u + (T)25) * (u + (T)25) / (T)170);
            const T Bf2 = (T)31 / (c1 + mexp(((T)25 - u) / (T)10));
            const T Cf2 = (T)16 / (c1 + mexp((u + (T)30) / (T)10));
            const T tau_f2 = Af2 + Bf2 + Cf2;
            const T q = cass / (T)0.05 * (cass / (T)0.05);
            const T fcass_inf = (T)0.6 / (c1 + q) + (T)0.4;
            const T tau_fcass = (T)80.0 / (c1 + q) + (T)2.0;
            x.d = d_inf - (d_inf - x.d) * mexp(-dt / tau_d);
            x.f = f_inf - (f_inf - x.f) * mexp(-dt / tau_f);
            x.f2 = f2_inf - (f2_inf - x.f2) * mexp(-dt / tau_f2);
            x.fcass = fcass_inf - (fcass_inf - x.fcass) * mexp(-dt / tau_fcass);
            const T z = (T)2 * (u - (T)15) * FF / RT;
            const T e2 = mexp(z);
            if constexpr (sizeof(T) == 8) {
                ical = P.v[gcal] * x.d * x.f * x.f2 * x.fcass * (T)4 *
                       (u - (T)15) * (FF * FF / RT) *
                       ((T)0.25 * e2 * cass - P.v[cao]) / (e2 - c1);
            } else {
                // 4 (u - 15) F^2 / RT / (e2 - 1) = 2 F z / (e^z - 1)
                ical = P.v[gcal] * x.d * x.f * x.f2 * x.fcass * (T)2 * FF *
                       x_expm1(z) * ((T)0.25 * e2 * cass - P.v[cao]);
            }
        }
        // calc_ito
        T ito;
        {
            const T r_inf = c1 / (c1 + mexp(((T)20 - u) / (T)6.0));
            const T s_inf = c1 / (c1 + mexp((u + (T)20) / (T)5.0));
            const T tau_r =
                (T)9.5 * mexp(-(u + (T)40.0) * (u + (T)40.0) / (T)1800.0) + (T)0.8;
            const T tau_s =
                (T)85.0 * mexp(-(u + (T)45.0) * (u + (T)45.0) / (T)320.0) +
                (T)5.0 / (c1 + mexp((u - (T)20.0) / (T)5.0)) + (T)3.0;
            x.s = s_inf - (s_inf - x.s) * mexp(-dt / tau_s);
            x.r = r_inf - (r_inf - x.r) * mexp(-dt / tau_r);
            ito = P.v[gto] * x.r * x.s * (u - Ek);
        }
        // calc_ikr
        T ikr;
        {
            const T xr1_inf = c1 / (c1 + mexp(((T)(-26.0) - u) / (T)7.0));
            const T axr1 = (T)450.0 / (c1 + mexp(((T)(-45.0) - u) / (T)10.0));
            const T bxr1 = (T)6.0 / (c1 + mexp((u - (T)(-30.0)) / (T)11.5));
            const T tau_xr1 = axr1 * bxr1;
            const T xr2_inf = c1 / (c1 + mexp((u - (T)(-88.0)) / (T)24.0));
            const T axr2 = (T)3.0 / (c1 + mexp(((T)(-60.0) - u) / (T)20.0));
            const T bxr2 = (T)1.12 / (c1 + mexp((u - (T)60.0) / (T)20.0));
            const T tau_xr2 = axr2 * bxr2;
            x.xr1 = xr1_inf - (xr1_inf - x.xr1) * mexp(-dt / tau_xr1);
            x.xr2 = xr2_inf - (xr2_inf - x.xr2) * mexp(-dt / tau_xr2);
            ikr = P.v[gkr] * fw_sqrt(P.v[ko] / (T)5.4) * x.xr1 * x.xr2 * (u - Ek);
        }
        // calc_iks
        T iks;
        {
            const T Axs = (T)1400.0 / fw_sqrt(c1 + mexp(((T)5.0 - u) / (T)6));
            const T Bxs = c1 / (c1 + mexp((u - (T)35.0) / (T)15.0));
            const T tau_xs = Axs * Bxs + (T)80;
            const T xs_inf = c1 / (c1 + mexp(((T)(-5.0) - u) / (T)14.0));
            x.xs = xs_inf - (xs_inf - x.xs) * mexp(-dt / tau_xs);
            iks = P.v[gks] * x.xs * x.xs * (u - Eks);
        }
        // calc_ik1
        const T ak1 = (T)0.1 / (c1 + mexp((T)0.06 * (u - Ek - (T)200)));
        const T bk1 = ((T)3.0 * mexp((T)0.0002 * (u - Ek + (T)100)) +
                       mexp((T)0.1 * (u - Ek - (T)10))) /
                      (c1 + mexp((T)(-0.5) * (u - Ek)));
        const T ik1 = P.v[gk1] * (ak1 / (ak1 + bk1)) * (u - Ek);
        // calc_inaca, calc_inak
        const T RT = P.v[R] * P.v[T_];
        const T inaca =
            P.v[knaca] *
            (c1 / (P.v[KmNai] * P.v[KmNai] * P.v[KmNai] +
                   P.v[nao] * P.v[nao] * P.v[nao])) *
            (c1 / (P.v[KmCa] + P.v[cao])) *
            (c1 / (c1 + P.v[ksat] * mexp((P.v[n_] - c1) * u * P.v[F] / RT))) *
            (mexp(P.v[n_] * u * P.v[F] / RT) * nai * nai * nai * P.v[cao] -
             mexp((P.v[n_] - c1) * u * P.v[F] / RT) * P.v[nao] * P.v[nao] *
                 P.v[nao] * cai * (T)2.5);
        const T rec_iNaK = c1 / (c1 + (T)0.1245 * mexp((T)(-0.1) * u * P.v[F] / RT) +
                                 (T)0.0353 * mexp(-u * P.v[F] / RT));
        const T inak = P.v[knak] * (P.v[ko] / (P.v[ko] + P.v[KmK])) *
                       (nai / (nai + P.v[KmNa])) * rec_iNaK;
        const T ipca = P.v[gpca] * cai / (P.v[KpCa] + cai);
        const T ipk = P.v[gpk] * (c1 / (c1 + mexp(((T)25 - u) / (T)5.98))) * (u - Ek);
        const T ibna = P.v[gbna] * (u - Ena);
        const T ibca = P.v[gbca] * (u - Eca);
        // calc_irel
        const T kCaSR = P.v[maxsr] - (P.v[maxsr] - P.v[minsr]) /
                                         (c1 + P.v[EC] / casr * (P.v[EC] / casr));
        const T k1 = P.v[k1_] / kCaSR;
        const T k2 = P.v[k2_] * kCaSR;
        const T drr = P.v[k4] * (c1 - x.rr) - k2 * cass * x.rr;
        x.rr += dt * drr;
        x.oo = k1 * cass * cass * x.rr / (P.v[k3] + k1 * cass * cass);
        const T irel = P.v[Vrel] * x.oo * (casr - cass);
        const T ileak = P.v[Vleak] * (casr - cai);
        const T iup = P.v[Vmaxup] / (c1 + P.v[Kup] * P.v[Kup] / (cai * cai));
        const T ixfer = P.v[Vxfer] * (cass - cai);
        // calc_casr, calc_cass (tp06_2d.py:793-873), calc_nai, calc_ki
        // (:924-966); calc_cai is discarded by the reference
        const T dCaSR = dt * (iup - irel - ileak);
        const T dCaSS = dt * (-ixfer * (P.v[Vc] / P.v[Vss]) +
                              irel * (P.v[Vsr] / P.v[Vss]) +
                              -ical * inversevssF2 * P.v[CAPACITANCE]);
        const T dNai = dt * (-(ina + ibna + (T)3 * inak + (T)3 * inaca) *
                             inverseVcF * P.v[CAPACITANCE]);
        const T dKi = dt * (-(ik1 + ito + ikr + iks - (T)2 * inak + ipk) *
                            inverseVcF * P.v[CAPACITANCE]);
        if constexpr (sizeof(T) == 8) {
            // the reference's quadratic for the free SR / subspace calcium
            const T CaCSQN = P.v[Bufsr] * casr / (casr + P.v[Kbufsr]);
            const T bjsr = P.v[Bufsr] - CaCSQN - dCaSR - casr + P.v[Kbufsr];
            const T cjsr = P.v[Kbufsr] * (CaCSQN + dCaSR + casr);
            const T CaSSBuf = P.v[Bufss] * cass / (cass + P.v[Kbufss]);
            const T bcss = P.v[Bufss] - CaSSBuf - dCaSS - cass + P.v[Kbufss];
            const T ccss = P.v[Kbufss] * (CaSSBuf + dCaSS + cass);
            x.casr = (fw_sqrt(bjsr * bjsr + 4 * cjsr) - bjsr) / 2;
            x.cass = (fw_sqrt(bcss * bcss + 4 * ccss) - bcss) / 2;
            x.nai += dNai;
            x.Ki += dKi;
        } else {
            // float32 rates, compensated accumulation: the new free calcium
            // is c0 + delta, delta the root near zero of the same quadratic
            // shifted to c0 (see buffered_step), so only the addition needs
            // the accumulator's precision
            x.casr += buffered_step(casr, P.v[Bufsr], P.v[Kbufsr], dCaSR);
            x.cass += buffered_step(cass, P.v[Bufss], P.v[Kbufss], dCaSS);
            x.nai += dNai;
            x.Ki += dKi;
        }
        return un - dt * (ikr + iks + ik1 + ito + ina + ibna + ical + ibca + inak +
                          inaca + ipca + ipk);
    }
};

// ---------------------------------------------------------------- Courtemanche
// Parameters in the order of courtemanche_2d.py's ionic_kernel_2d signature
// (:569-577); state in Courtemanche2D.state_vars order minus u (:118-120).
struct ModelCRN {
    static constexpr int NS = 21, NP = 39;
    static constexpr int kMinBlocksF32 = 3;  // 4 would spill
    enum {
        gna, gnab, gk1, gkr, gks, gto, gcal, gcab, gkur_coeff, F, T_, R, Vc, Vj,
        Vup, Vrel, ibk, cao, nao, ko, caupmax, kup, kmnai, kmko, kmnancx,
        kmcancx, ksatncx, kmcmdn, kmtrpn, kmcsqn, trpnmax, cmdnmax, csqnmax,
        inacamax, inakmax, ipcamax, krel, iupmax, kq10
    };
    enum { s_nai, s_ki, s_cai, s_caup, s_carel, s_m, s_h, s_j, s_d, s_f, s_oa,
           s_oi, s_ua, s_ui, s_xr, s_xs, s_fca, s_irel, s_vrel, s_urel, s_wrel };
    static constexpr bool is_conc(int i) { return i <= s_carel; }

    template <class T>
    struct St {
        Conc<T> nai, ki, cai, caup, carel;
        T m, h, j, d, f, oa, oi, ua, ui, xr, xs, fca, irel, vrel, urel, wrel;
    };
    template <class T>
    __device__ static __forceinline__ St<T> load(void *const *S, int64_t p)
    {
        St<T> x;
        conc_load(x.nai, S[s_nai], p);
        conc_load(x.ki, S[s_ki], p);
        conc_load(x.cai, S[s_cai], p);
        conc_load(x.caup, S[s_caup], p);
        conc_load(x.carel, S[s_carel], p);
        x.m = ((const T *)S[s_m])[p];
        x.h = ((const T *)S[s_h])[p];
        x.j = ((const T *)S[s_j])[p];
        x.d = ((const T *)S[s_d])[p];
        x.f = ((const T *)S[s_f])[p];
        x.oa = ((const T *)S[s_oa])[p];
        x.oi = ((const T *)S[s_oi])[p];
        x.ua = ((const T *)S[s_ua])[p];
        x.ui = ((const T *)S[s_ui])[p];
        x.xr = ((const T *)S[s_xr])[p];
        x.xs = ((const T *)S[s_xs])[p];
        x.fca = ((const T *)S[s_fca])[p];
        x.irel = ((const T *)S[s_irel])[p];
        x.vrel = ((const T *)S[s_vrel])[p];
        x.urel = ((const T *)S[s_urel])[p];
        x.wrel = ((const T *)S[s_wrel])[p];
        return x;
    }
    template <class T>
    __device__ static __forceinline__ void store(void *const *S, int64_t p,
                                                 const St<T> &x)
    {
        conc_store(S[s_nai], p, x.nai);
        conc_store(S[s_ki], p, x.ki);
        conc_store(S[s_cai], p, x.cai);
        conc_store(S[s_caup], p, x.caup);
        conc_store(S[s_carel], p, x.carel);
        ((T *)S[s_m])[p] = x.m;
        ((T *)S[s_h])[p] = x.h;
        ((T *)S[s_j])[p] = x.j;
        ((T *)S[s_d])[p] = x.d;
        ((T *)S[s_f])[p] = x.f;
        ((T *)S[s_oa])[p] = x.oa;
        ((T *)S[s_oi])[p] = x.oi;
        ((T *)S[s_ua])[p] = x.ua;
        ((T *)S[s_ui])[p] = x.ui;
        ((T *)S[s_xr])[p] = x.xr;
        ((T *)S[s_xs])[p] = x.xs;
        ((T *)S[s_fca])[p] = x.fca;
        ((T *)S[s_irel])[p] = x.irel;
        ((T *)S[s_vrel])[p] = x.vrel;
        ((T *)S[s_urel])[p] = x.urel;
        ((T *)S[s_wrel])[p] = x.wrel;
    }
    template <class T>
    __device__ static __forceinline__ double probe(const St<T> &x, int i)
    {
        switch (i) {
        case s_nai: return conc_probe(x.nai);
        case s_ki: return conc_probe(x.ki);
        case s_cai: return conc_probe(x.cai);
        case s_caup: return conc_probe(x.caup);
        case s_carel: return conc_probe(x.carel);
        case s_m: return x.m;
        case s_h: return x.h;
        case s_j: return x.j;
        case s_d: return x.d;
        case s_f: return x.f;
        case s_oa: return x.oa;
        case s_oi: return x.oi;
        case s_ua: return x.ua;
        case s_ui: return x.ui;
        case s_xr: return x.xr;
        case s_xs: return x.xs;
        case s_fca: return x.fca;
        case s_irel: return x.irel;
        case s_vrel: return x.vrel;
        case s_urel: return x.urel;
        default: return x.wrel;
        }
    }
    template <class T>
    __device__ static __forceinline__ T gate(T x, T x_inf, T tau, T dt)
    {
        return x_inf - (x_inf - x) * mexp(-dt / tau);
    }

    // ionic_kernel_2d and its helpers (courtemanche_2d.py:180-641)
    template <class T>
    __device__ static __forceinline__ T update(T u, T un, St<T> &x,
                                               const Params<T, NP> &P, T dt)
    {
        const T c1 = (T)1;
        const T cai = (T)x.cai, nai = (T)x.nai, carel = (T)x.carel;
        const T caup = (T)x.caup, ki = (T)x.ki;
        const T RTF = P.v[R] * P.v[T_] / P.v[F];
        const T ena = RTF * mlog(P.v[nao] / nai);
        const T ek = RTF * mlog(P.v[ko] / ki);
        const T eca = P.v[R] * P.v[T_] / ((T)2 * P.v[F]) * mlog(P.v[cao] / cai);
        // calc_gating_m, calc_gating_h, calc_gating_j
        {
            T am;
            if constexpr (sizeof(T) == 8) {
                if (u == (T)(-47.13))
                    am = (T)3.2;
                else
                    am = (T)0.32 * (u + (T)47.13) /
                         (c1 - mexp((T)(-0.1) * (u + (T)47.13)));
            } else {
                am = (T)3.2 * x_expm1((T)(-0.1) * (u + (T)47.13));
            }
            const T bm = (T)0.08 * mexp(-u / (T)11);
            x.m = gate(x.m, am / (am + bm), c1 / (am + bm), dt);
            T ah = (T)0.135 * mexp(-((T)80 + u) / (T)6.8);
            T bh = (T)3.56 * mexp((T)0.079 * u) + (T)310000 * mexp((T)0.35 * u);
            T aj = ((T)(-127140) * mexp((T)0.2444 * u) -
                    (T)3.474e-05 * mexp((T)(-0.04391) * u)) *
                   (u + (T)37.78) / (c1 + mexp((T)0.311 * (u + (T)79.23)));
            T bj = (T)0.1212 * mexp((T)(-0.01052) * u) /
                   (c1 + mexp((T)(-0.1378) * (u + (T)40.14)));
            if (u >= (T)(-40)) {
                ah = (T)0;
                bh = c1 / ((T)0.13 * (c1 + mexp(-(u + (T)10.66) / (T)11.1)));
                aj = (T)0;
                bj = (T)0.3 * mexp((T)(-2.535e-07) * u) /
                     (c1 + mexp((T)(-0.1) * (u + (T)32)));
            }
            x.h = gate(x.h, ah / (ah + bh), c1 / (ah + bh), dt);
            const T j_inf = aj / (aj + bj);
            const T tau_j = c1 / (aj + bj);
            x.j = j_inf - (j_inf - x.j) * mexp(-dt / tau_j);
        }
        const T ina = P.v[gna] * pow3(x.m) * x.h * x.j * (u - ena);
        const T ik1 = P.v[gk1] * (u - ek) / (c1 + mexp((T)0.07 * (u + (T)80)));
        T ito, ikur;
        {
            const T ao = (T)0.65 / (mexp(-(u + (T)10) / (T)8.5) +
                                    mexp(-(u - (T)30) / (T)59.0));
            const T bo = (T)0.65 / ((T)2.5 + mexp((u + (T)82) / (T)17.0));
            const T tau_o = c1 / (P.v[kq10] * (ao + bo));
            const T o_inf = c1 / (c1 + mexp(-(u + (T)20.47) / (T)17.54));
            const T aoi = c1 / ((T)18.53 + mexp((u + (T)113.7) / (T)10.95));
            const T boi = c1 / ((T)35.56 + mexp(-(u + (T)1.26) / (T)7.44));
            const T tau_oi = c1 / (P.v[kq10] * (aoi + boi));
            const T oi_inf = c1 / (c1 + mexp((u + (T)43.1) / (T)5.3));
            x.oa = gate(x.oa, o_inf, tau_o, dt);
            x.oi = gate(x.oi, oi_inf, tau_oi, dt);
            ito = P.v[gto] * pow3(x.oa) * x.oi * (u - ek);
            const T gkur = (T)0.005 + (T)0.05 / (c1 + mexp(-(u - (T)15) / (T)13.0));
            const T tau_ua = c1 / (P.v[kq10] * (ao + bo));
            const T ua_inf = c1 / (c1 + mexp(-(u + (T)30.3) / (T)9.6));
            const T aui = c1 / ((T)21 + mexp(-(u - (T)185) / (T)28.0));
            const T bui = mexp((u - (T)158) / (T)16.0);
            const T tau_ui = c1 / (P.v[kq10] * (aui + bui));
            const T ui_inf = c1 / (c1 + mexp((u - (T)99.45) / (T)27.48));
            x.ua = gate(x.ua, ua_inf, tau_ua, dt);
            x.ui = gate(x.ui, ui_inf, tau_ui, dt);
            ikur = P.v[gkur_coeff] * gkur * pow3(x.ua) * x.ui * (u - ek);
        }
        T ikr, iks;
        {
            // the model's xs holds the IKr gate, xr the IKs gate
            T axr, bxr;
            if constexpr (sizeof(T) == 8) {
                axr = (T)0.0003 * (u + (T)14.1) /
                      (c1 - mexp(-(u + (T)14.1) / (T)5));
                bxr = (T)7.3898e-05 * (u - (T)3.3328) /
                      (mexp((u - (T)3.3328) / (T)5.1237) - c1);
            } else {
                axr = (T)(0.0003 * 5) * x_expm1(-(u + (T)14.1) / (T)5);
                bxr = (T)(7.3898e-05 * 5.1237) *
                      x_expm1((u - (T)3.3328) / (T)5.1237);
            }
            const T tau_xr = c1 / (axr + bxr);
            const T xr_inf = c1 / (c1 + mexp(-(u + (T)14.1) / (T)6.5));
            x.xs = gate(x.xs, xr_inf, tau_xr, dt);
            ikr = (T)0.0294 * x.xs * (u - ek) / (c1 + mexp((u + (T)15) / (T)22.4));
            T axs, bxs;
            if constexpr (sizeof(T) == 8) {
                axs = (T)4e-05 * (u - (T)19.9) /
                      (c1 - mexp(-(u - (T)19.9) / (T)17));
                bxs = (T)3.5e-05 * (u - (T)19.9) /
                      (mexp((u - (T)19.9) / (T)9) - c1);
            } else {
                axs = (T)(4e-05 * 17) * x_expm1(-(u - (T)19.9) / (T)17);
                bxs = (T)(3.5e-05 * 9) * x_expm1((u - (T)19.9) / (T)9);
            }
            const T tau_xs = c1 / ((T)2 * (axs + bxs));
            const T xs_inf = c1 / fw_sqrt(c1 + mexp(-(u - (T)19.9) / (T)12.7));
            x.xr = gate(x.xr, xs_inf, tau_xs, dt);
            iks = P.v[gks] * (x.xr * x.xr) * (u - ek);
        }
        T ical;
        {
            const T e = mexp(-(u + (T)10) / (T)6.24);
            T tau_d;
            if constexpr (sizeof(T) == 8) {
                tau_d = (c1 - e) / ((T)0.035 * (u + (T)10) * (c1 + e));
            } else {
                // (1 - e^-v) / v = 1 / x_expm1(-v), v = (u + 10) / 6.24
                tau_d = c1 / ((T)(0.035 * 6.24) *
                              x_expm1(-(u + (T)10) / (T)6.24) * (c1 + e));
            }
            const T d_inf = c1 / (c1 + mexp(-(u + (T)10) / (T)8.0));
            const T tau_f = (T)9 / ((T)0.0197 * mexp(-((T)0.0337 * (T)0.0337) *
                                                      ((u + (T)10) * (u + (T)10))) +
                                    (T)0.02);
            const T f_inf = c1 / (c1 + mexp((u + (T)28) / (T)6.9));
            const T fca_inf = c1 / (c1 + cai / (T)0.00035);
            x.d = gate(x.d, d_inf, tau_d, dt);
            x.f = gate(x.f, f_inf, tau_f, dt);
            x.fca = gate(x.fca, fca_inf, (T)2, dt);
            ical = P.v[gcal] * x.d * x.f * x.fca * (u - (T)65);
        }
        const T RT = P.v[R] * P.v[T_];
        T inak, inaca;
        {
            const T s = c1 / (T)7.0 * (mexp(P.v[nao] / (T)67.3) - c1);
            const T fnak = c1 / (c1 + (T)0.1245 * mexp((T)(-0.1) * (P.v[F] * u) / RT) +
                                 (T)0.0365 * s * mexp(-(P.v[F] * u) / RT));
            inak = P.v[inakmax] * fnak * (c1 / (c1 + pow15(P.v[kmnai] / nai))) *
                   (P.v[ko] / (P.v[ko] + P.v[kmko]));
            const T gamma = (T)0.35;
            const T exp_term = mexp(gamma * (P.v[F] * u) / RT);
            const T exp_rev_term = mexp((gamma - c1) * (P.v[F] * u) / RT);
            const T numerator = P.v[inacamax] *
                                (exp_term * pow3(nai) * P.v[cao] -
                                 exp_rev_term * pow3(P.v[nao]) * cai);
            const T term1 = pow3(P.v[kmnancx]) + pow3(P.v[nao]);
            const T term2 = P.v[kmcancx] + P.v[cao];
            const T term3 = c1 + P.v[ksatncx] * exp_rev_term;
            inaca = numerator / (term1 * term2 * term3);
        }
        const T ibca = P.v[gcab] * (u - eca);
        const T ibna = P.v[gnab] * (u - ena);
        const T ipca = P.v[ipcamax] * cai / (cai + (T)0.0005);
        {
            const T Fn = (T)1e-12 * P.v[Vrel] * x.irel -
                         (T)5 * (T)1e-13 / P.v[F] * ((T)0.5 * ical - (T)0.2 * inaca);
            const T u_inf = c1 / (c1 + mexp(-(Fn - (T)3.4175e-13) / (T)1.367e-15));
            const T tau_v = (T)1.91 + (T)2.09 / (c1 + mexp(-(Fn - (T)3.4175e-13) /
                                                           (T)1.367e-15));
            const T v_inf = c1 - c1 / (c1 + mexp(-(Fn - (T)6.835e-14) / (T)1.367e-15));
            const T ew = mexp(-(u - (T)7.9) / (T)5.0);
            T tau_w;
            if constexpr (sizeof(T) == 8) {
                tau_w = (T)6 * (c1 - ew) / ((c1 + (T)0.3 * ew) * (u - (T)7.9));
            } else {
                tau_w = (T)(6.0 / 5.0) /
                        ((c1 + (T)0.3 * ew) * x_expm1(-(u - (T)7.9) / (T)5.0));
            }
            const T w_inf = c1 - c1 / (c1 + mexp(-(u - (T)40) / (T)17.0));
            x.urel = gate(x.urel, u_inf, (T)8, dt);
            x.vrel = gate(x.vrel, v_inf, tau_v, dt);
            x.wrel = gate(x.wrel, w_inf, tau_w, dt);
            x.irel = P.v[krel] * (x.urel * x.urel) * x.vrel * x.wrel * (carel - cai);
        }
        const T itr = (caup - carel) / (T)180;
        const T iup = P.v[iupmax] / (c1 + P.v[kup] / cai);
        const T iupleak = caup / P.v[caupmax] * P.v[iupmax];
        // calc_caup, calc_nai, calc_ki, calc_cai, calc_carel
        // (courtemanche_2d.py:219-253); under float32 the rates are float32
        // and only the accumulation is float64
        const T FVj = P.v[F] * P.v[Vj];
        const T dCaup = dt * (iup - iupleak - itr * (P.v[Vrel] / P.v[Vup]));
        const T dNai = dt * (((T)(-3) * inak - (T)3 * inaca - ibna - ina) / FVj);
        const T dKi = dt * (((T)2 * inak - ik1 - ito - ikur - ikr - iks -
                             P.v[ibk]) / FVj);
        const T ktr = P.v[kmtrpn], kcm = P.v[kmcmdn];
        const T B1 = ((T)2 * inaca - ipca - ical - ibca) / ((T)2 * FVj) +
                     (P.v[Vup] * (iupleak - iup) + x.irel * P.v[Vrel]) / P.v[Vj];
        const T B2 = c1 + P.v[trpnmax] * ktr / ((cai + ktr) * (cai + ktr)) +
                     P.v[cmdnmax] * kcm / ((cai + kcm) * (cai + kcm));
        const T dCai = dt * (B1 / B2);
        const T kcs = P.v[kmcsqn];
        const T dCarel = dt * ((itr - x.irel) /
                               (c1 + P.v[csqnmax] * kcs /
                                         ((carel + kcs) * (carel + kcs))));
        x.caup += dCaup;
        x.nai += dNai;
        x.ki += dKi;
        x.cai += dCai;
        x.carel += dCarel;
        return un - dt * (ina + ik1 + ito + ikur + ikr + iks + ical + ipca + inak +
                          inaca + ibna + ibca);
    }
};

// ---------------------------------------------------------------- LR91
// Luo-Rudy 1991.  Parameters in the order of luo_rudy91_2d.py's
// ionic_kernel_2d signature: gna, gsi, gk, gk1, gkp, gb, ko, ki, nai, nao,
// cao, R, T, F, PR_NaK; state m, h, j, d, f, x, cai (LuoRudy912D.state_vars
// minus u).  calc_ina uses the updated m, h, j; calc_isk and calc_ik the
// gates before their update, as the reference does.  Under FW_F32 Ca_i is
// stored as float64 and only its accumulation is float64.
struct ModelLR91 {
    static constexpr int NS = 7, NP = 15;
    enum { gna, gsi, gk, gk1, gkp, gb, ko, ki, nai, nao, cao, R, T_, F, PR_NaK };
    enum { s_m, s_h, s_j, s_d, s_f, s_x, s_cai };
    static constexpr bool is_conc(int i) { return i == s_cai; }

    template <class T>
    struct St {
        T m, h, j, d, f, x;
        Conc<T> cai;
    };
    template <class T>
    __device__ static __forceinline__ St<T> load(void *const *S, int64_t p)
    {
        St<T> x;
        x.m = ((const T *)S[s_m])[p];
        x.h = ((const T *)S[s_h])[p];
        x.j = ((const T *)S[s_j])[p];
        x.d = ((const T *)S[s_d])[p];
        x.f = ((const T *)S[s_f])[p];
        x.x = ((const T *)S[s_x])[p];
        conc_load(x.cai, S[s_cai], p);
        return x;
    }
    template <class T>
    __device__ static __forceinline__ void store(void *const *S, int64_t p,
                                                 const St<T> &x)
    {
        ((T *)S[s_m])[p] = x.m;
        ((T *)S[s_h])[p] = x.h;
        ((T *)S[s_j])[p] = x.j;
        ((T *)S[s_d])[p] = x.d;
        ((T *)S[s_f])[p] = x.f;
        ((T *)S[s_x])[p] = x.x;
        conc_store(S[s_cai], p, x.cai);
    }
    template <class T>
    __device__ static __forceinline__ double probe(const St<T> &x, int i)
    {
        switch (i) {
        case s_m: return x.m;
        case s_h: return x.h;
        case s_j: return x.j;
        case s_d: return x.d;
        case s_f: return x.f;
        case s_x: return x.x;
        default: return conc_probe(x.cai);
        }
    }
    // calc_gating_var (luo_rudy91_2d.py): tau = 1 / (a + b),
    // inf = a / (a + b), var += dt (inf - var) / tau
    template <class T>
    __device__ static __forceinline__ T gating(T var, T dt, T a, T b)
    {
        const T tau = (T)1. / (a + b);
        const T inf = a / (a + b);
        return var + dt * (inf - var) / tau;
    }

    template <class T>
    __device__ static __forceinline__ T update(T u, T un, St<T> &x,
                                               const Params<T, NP> &P, T dt)
    {
        const T c1 = (T)1;
        const T RTF = P.v[R] * P.v[T_] / P.v[F];
        const T E_Na = RTF * mlog(P.v[nao] / P.v[nai]);
        // calc_ina
        T ina;
        {
            T alpha_h = 0, beta_h = 0, beta_J = 0, alpha_J = 0;
            if (u >= (T)(-40.)) {
                beta_h = (T)1. / ((T)0.13 * (c1 + mexp((u + (T)10.66) / (T)(-11.1))));
                beta_J = (T)0.3 * mexp((T)(-2.535) * (T)1e-07 * u) /
                         (c1 + mexp((T)(-0.1) * (u + (T)32)));
            } else {
                alpha_h = (T)0.135 * mexp(((T)80 + u) / (T)(-6.8));
                beta_h = (T)3.56 * mexp((T)0.079 * u) +
                         (T)3.1 * (T)1e5 * mexp((T)0.35 * u);
                beta_J = (T)0.1212 * mexp((T)(-0.01052) * u) /
                         (c1 + mexp((T)(-0.1378) * (u + (T)40.14)));
                alpha_J = ((T)(-1.2714) * (T)1e5 * mexp((T)0.2444 * u) -
                           (T)3.474 * (T)1e-5 * mexp((T)(-0.04391) * u)) *
                          (u + (T)37.78) / (c1 + mexp((T)0.311 * (u + (T)79.23)));
            }
            T alpha_m;
            if constexpr (sizeof(T) == 8)
                alpha_m = (T)0.32 * (u + (T)47.13) /
                          (c1 - mexp((T)(-0.1) * (u + (T)47.13)));
            else
                alpha_m = (T)3.2 * x_expm1((T)(-0.1) * (u + (T)47.13));
            const T beta_m = (T)0.08 * mexp(-u / (T)11);
            x.m = gating(x.m, dt, alpha_m, beta_m);
            x.h = gating(x.h, dt, alpha_h, beta_h);
            x.j = gating(x.j, dt, alpha_J, beta_J);
            ina = P.v[gna] * x.m * x.m * x.m * x.h * x.j * (u - E_Na);
        }
        // calc_isk (gates before the update)
        T isi;
        {
            const T cai = (T)x.cai;
            const T E_Si = (T)7.7 - (T)13.0287 * mlog(cai);
            isi = P.v[gsi] * x.d * x.f * (u - E_Si);
            const T alpha_d = (T)0.095 * mexp((T)(-0.01) * (u - (T)5)) /
                              (c1 + mexp((T)(-0.072) * (u - (T)5)));
            const T beta_d = (T)0.07 * mexp((T)(-0.017) * (u + (T)44)) /
                             (c1 + mexp((T)0.05 * (u + (T)44)));
            const T alpha_f = (T)0.012 * mexp((T)(-0.008) * (u + (T)28)) /
                              (c1 + mexp((T)0.15 * (u + (T)28)));
            const T beta_f = (T)0.0065 * mexp((T)(-0.02) * (u + (T)30)) /
                             (c1 + mexp((T)(-0.2) * (u + (T)30)));
            x.d = gating(x.d, dt, alpha_d, beta_d);
            x.f = gating(x.f, dt, alpha_f, beta_f);
            x.cai += dt * ((T)(-0.0001) * isi + (T)0.07 * ((T)0.0001 - cai));
        }
        // calc_ik (gate before the update)
        T ik;
        {
            const T E_K = RTF * mlog((P.v[ko] + P.v[PR_NaK] * P.v[nao]) /
                                     (P.v[ki] + P.v[PR_NaK] * P.v[nai]));
            const T G_K = P.v[gk] * fw_sqrt(P.v[ko] / (T)5.4);
            T Xi;
            if (u > (T)(-100)) {
                if constexpr (sizeof(T) == 8)
                    Xi = (T)2.837 * (mexp((T)0.04 * (u + (T)77)) - c1) /
                         ((u + (T)77) * mexp((T)0.04 * (u + (T)35)));
                else  // (e^z - 1) / (u + 77) = 0.04 / x_expm1(z)
                    Xi = (T)(2.837 * 0.04) /
                         (x_expm1((T)0.04 * (u + (T)77)) *
                          mexp((T)0.04 * (u + (T)35)));
            } else {
                Xi = c1;
            }
            ik = G_K * x.x * Xi * (u - E_K);
            const T alpha_x = (T)0.0005 * mexp((T)0.083 * (u + (T)50)) /
                              (c1 + mexp((T)0.057 * (u + (T)50)));
            const T beta_x = (T)0.0013 * mexp((T)(-0.06) * (u + (T)20)) /
                             (c1 + mexp((T)(-0.04) * (u + (T)20)));
            x.x = gating(x.x, dt, alpha_x, beta_x);
        }
        const T E_K1 = RTF * mlog(P.v[ko] / P.v[ki]);
        // calc_ik1
        const T alpha_K1 = (T)1.02 / (c1 + mexp((T)0.2385 * (u - E_K1 - (T)59.215)));
        const T beta_K1 = ((T)0.49124 * mexp((T)0.08032 * (u - E_K1 + (T)5.476)) +
                           mexp((T)0.06175 * (u - E_K1 - (T)594.31))) /
                          (c1 + mexp((T)(-0.5143) * (u - E_K1 + (T)4.753)));
        const T K_1x = alpha_K1 / (alpha_K1 + beta_K1);
        const T G_K1 = P.v[gk1] * fw_sqrt(P.v[ko] / (T)5.4);
        const T ik1 = G_K1 * K_1x * (u - E_K1);
        // calc_ikp, calc_ib
        const T K_p = (T)1. / (c1 + mexp(((T)7.488 - u) / (T)5.98));
        const T ikp = P.v[gkp] * K_p * (u - E_K1);
        const T ib = P.v[gb] * (u + (T)59.87);
        const T ik1t = ik1 + ikp + ib;
        return un - dt * (ina + isi + ik1t + ik);
    }
};

}  // namespace fw
