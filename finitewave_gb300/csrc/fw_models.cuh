// fw_models.cuh -- node-local ionic updates of the phenomenological models.
//
// Each model restates the reference's per-node formula with its operation
// order kept term by term; compiled without FMA contraction (fw_exact.cu) the
// float64 results are bitwise the reference's for the models that use only
// + - * / (Aliev-Panfilov, Mitchell-Schaeffer).  The same code compiled with
// FMA contraction is the fast FP32 form.
//
// Interface of a model M:
//   M::NS, M::NP            number of state variables after u / parameters
//   M::St<T>                the node's state variables in registers
//   M::load<T>(s, p)        read state of node p from the arrays s[0..NS-1]
//   M::store<T>(s, p, x)    write it back
//   M::update<T>(u, un, x, P, dt)
//       u  : the node's potential at step n (after stimuli)
//       un : the diffusion result for the node
//       returns the new potential; x is advanced in place.
#pragma once

#include <math.h>
#include <stdint.h>

namespace fw {

template <class T, int N>
struct Params {
    T v[N];
};

// float32 operations with a fixed rounding -- to nearest even, subnormal
// inputs and results flushed to zero -- as inline PTX, so that neither FMA
// contraction nor the translation unit's flags change them.  The pair forms
// are Blackwell's two-wide f32x2 instructions (one issue for two lanes);
// each lane is rounded exactly as the scalar operation, so an update written
// once with f_* and once with f2_* gives the same bits per node.
__device__ __forceinline__ float f_add(float a, float b)
{
    float d;
    asm("add.rn.ftz.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
    return d;
}
__device__ __forceinline__ float f_mul(float a, float b)
{
    float d;
    asm("mul.rn.ftz.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
    return d;
}
__device__ __forceinline__ float f_fma(float a, float b, float c)
{
    float d;
    asm("fma.rn.ftz.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float2 f2_add(float2 a, float2 b)
{
    float2 d;
    asm("{\n .reg .b64 ra, rb, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
        " add.rn.ftz.f32x2 rd, ra, rb;\n mov.b64 {%0, %1}, rd;\n}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b)
{
    float2 d;
    asm("{\n .reg .b64 ra, rb, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
        " mul.rn.ftz.f32x2 rd, ra, rb;\n mov.b64 {%0, %1}, rd;\n}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c)
{
    float2 d;
    asm("{\n .reg .b64 ra, rb, rc, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
        " mov.b64 rc, {%6, %7};\n fma.rn.ftz.f32x2 rd, ra, rb, rc;\n mov.b64 {%0, %1}, rd;\n}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
__device__ __forceinline__ float2 f2_dup(float x) { return make_float2(x, x); }

// Precision-matched transcendental calls (float -> the float functions, so
// that no float64 arithmetic sneaks into the float32 kernels).
__device__ __forceinline__ float fw_tanh(float x) { return tanhf(x); }
__device__ __forceinline__ double fw_tanh(double x) { return tanh(x); }
__device__ __forceinline__ float fw_exp(float x) { return expf(x); }
__device__ __forceinline__ double fw_exp(double x) { return exp(x); }
__device__ __forceinline__ float fw_log(float x) { return logf(x); }
__device__ __forceinline__ double fw_log(double x) { return log(x); }
__device__ __forceinline__ float fw_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double fw_sqrt(double x) { return sqrt(x); }

template <class T, int N, class S>
__device__ __forceinline__ Params<T, N> load_params(const S *p)
{
    Params<T, N> r;
#pragma unroll
    for (int i = 0; i < N; ++i) r.v[i] = (T)p[i];
    return r;
}

// Aliev-Panfilov.  params: a, k, eap, mu_1, mu_2 (aliev_panfilov_2d.py:
// 290-295).  calc_v (:337-374), then the voltage update with the new v
// (ionic_kernel_2d :376-406).
struct ModelAP {
    static constexpr int NS = 1, NP = 5;
    template <class T>
    struct St {
        T v;
    };
    template <class T>
    __device__ static __forceinline__ St<T> load(void *const *s, int64_t p)
    {
        return {((const T *)s[0])[p]};
    }
    template <class T>
    __device__ static __forceinline__ void store(void *const *s, int64_t p,
                                                 const St<T> &x)
    {
        ((T *)s[0])[p] = x.v;
    }
    template <class T>
    __device__ static __forceinline__ double probe(const St<T> &x, int)
    {
        return (double)x.v;
    }
    template <class T>
    __device__ static __forceinline__ St<T> from_array(const T *a)
    {
        return {a[0]};
    }
    template <class T>
    __device__ static __forceinline__ T update(T u, T un, St<T> &x,
                                               const Params<T, NP> &P, T dt)
    {
        const T a = P.v[0], k = P.v[1], eap = P.v[2], mu_1 = P.v[3],
                mu_2 = P.v[4];
        T v = x.v;
        if constexpr (sizeof(T) == 4) {
            // float32: the same update with fewer operations -- u - a - 1
            // formed once for both equations, u (u - a) (u - 1) as
            // ((u - (a + 1)) u + a) u, and explicit FMAs; it rounds
            // differently from the float64 form, within float32 error
            const T ua1 = u - (a + (T)1.);
            const T q = __fdividef(mu_1 * v, mu_2 + u);
            const T g = fmaf(k * u, ua1, v);
            v = fmaf((-dt) * (eap + q), g, v);
            x.v = v;
            const T cub = fmaf(ua1, u, a) * u;
            return fmaf(dt, fmaf(-k, cub, -(u * v)), un);
        } else {
            v += (-dt) * (eap + (mu_1 * v) / (mu_2 + u)) *
                 (v + k * u * (u - a - (T)1.));
            x.v = v;
            return un + dt * ((-k) * u * (u - a) * (u - (T)1.) - u * v);
        }
    }
    // The float32 update of the fused and batched kernels: update<float>'s
    // rearrangement with every rounding explicit (-dt (k cub + u v) for
    // dt (-k cub - u v), the same value), and its two-node form, which
    // gives each node the same bits.
    __device__ static __forceinline__ float update_fused(float u, float un,
                                                         St<float> &x,
                                                         const Params<float, NP> &P,
                                                         float dt)
    {
        const float a = P.v[0], k = P.v[1], eap = P.v[2], mu_1 = P.v[3],
                    mu_2 = P.v[4];
        float v = x.v;
        const float ua1 = f_add(u, -(a + 1.f));
        const float q = __fdividef(f_mul(mu_1, v), f_add(mu_2, u));
        const float g = f_fma(f_mul(k, u), ua1, v);
        v = f_fma(f_mul(-dt, f_add(eap, q)), g, v);
        x.v = v;
        const float cub = f_mul(f_fma(ua1, u, a), u);
        return f_fma(-dt, f_fma(k, cub, f_mul(u, v)), un);
    }
    __device__ static __forceinline__ float2 update_pair(float2 u, float2 un,
                                                         St<float> &x0, St<float> &x1,
                                                         const Params<float, NP> &P,
                                                         float dt)
    {
        const float a = P.v[0], k = P.v[1], eap = P.v[2], mu_1 = P.v[3],
                    mu_2 = P.v[4];
        float2 v = make_float2(x0.v, x1.v);
        const float2 ua1 = f2_add(u, f2_dup(-(a + 1.f)));
        const float2 num = f2_mul(f2_dup(mu_1), v), den = f2_add(f2_dup(mu_2), u);
        const float2 q = make_float2(__fdividef(num.x, den.x), __fdividef(num.y, den.y));
        const float2 g = f2_fma(f2_mul(f2_dup(k), u), ua1, v);
        v = f2_fma(f2_mul(f2_dup(-dt), f2_add(f2_dup(eap), q)), g, v);
        x0.v = v.x;
        x1.v = v.y;
        const float2 cub = f2_mul(f2_fma(ua1, u, f2_dup(a)), u);
        return f2_fma(f2_dup(-dt), f2_fma(f2_dup(k), cub, f2_mul(u, v)), un);
    }
};

// Mitchell-Schaeffer.  params: tau_close, tau_open, tau_in, tau_out, u_gate
// (mitchell_schaeffer_2d.py:57-61).  calc_h, calc_J_in, calc_J_out,
// ionic_kernel_2d (:102-217).  u**2 is u*u as numba compiles it.
struct ModelMS {
    static constexpr int NS = 1, NP = 5;
    template <class T>
    struct St {
        T h;
    };
    template <class T>
    __device__ static __forceinline__ St<T> load(void *const *s, int64_t p)
    {
        return {((const T *)s[0])[p]};
    }
    template <class T>
    __device__ static __forceinline__ void store(void *const *s, int64_t p,
                                                 const St<T> &x)
    {
        ((T *)s[0])[p] = x.h;
    }
    template <class T>
    __device__ static __forceinline__ double probe(const St<T> &x, int)
    {
        return (double)x.h;
    }
    template <class T>
    __device__ static __forceinline__ St<T> from_array(const T *a)
    {
        return {a[0]};
    }
    template <class T>
    __device__ static __forceinline__ T update(T u, T un, St<T> &x,
                                               const Params<T, NP> &P, T dt)
    {
        const T tau_close = P.v[0], tau_open = P.v[1], tau_in = P.v[2],
                tau_out = P.v[3], u_gate = P.v[4];
        T h = x.h;
        h += (u < u_gate) ? dt * ((T)1.0 - h) / tau_open
                          : dt * (-h) / tau_close;
        x.h = h;
        T C = (u * u) * ((T)1 - u);
        T J_in = h * C / tau_in;
        T J_out = -u / tau_out;
        return un + dt * (J_in + J_out);
    }
};

// Fenton-Karma (MLR-I).  params: tau_d, tau_o, tau_r, tau_si, tau_v_m,
// tau_v_p, tau_w_m, tau_w_p, k, u_c, uc_si (fenton_karma_2d.py:86-97).
// calc_v, calc_w, calc_Jfi, calc_Jso, calc_Jsi, ionic_kernel_2d (:143-328);
// J_si takes the fast gate v, as the reference passes it (:326).
struct ModelFK {
    static constexpr int NS = 2, NP = 11;
    template <class T>
    struct St {
        T v, w;
    };
    template <class T>
    __device__ static __forceinline__ St<T> load(void *const *s, int64_t p)
    {
        return {((const T *)s[0])[p], ((const T *)s[1])[p]};
    }
    template <class T>
    __device__ static __forceinline__ void store(void *const *s, int64_t p,
                                                 const St<T> &x)
    {
        ((T *)s[0])[p] = x.v;
        ((T *)s[1])[p] = x.w;
    }
    template <class T>
    __device__ static __forceinline__ double probe(const St<T> &x, int i)
    {
        return i == 0 ? (double)x.v : (double)x.w;
    }
    template <class T>
    __device__ static __forceinline__ St<T> from_array(const T *a)
    {
        return {a[0], a[1]};
    }
    template <class T>
    __device__ static __forceinline__ T update(T u, T un, St<T> &x,
                                               const Params<T, NP> &P, T dt)
    {
        const T tau_d = P.v[0], tau_o = P.v[1], tau_r = P.v[2],
                tau_si = P.v[3], tau_v_m = P.v[4], tau_v_p = P.v[5],
                tau_w_m = P.v[6], tau_w_p = P.v[7], k = P.v[8], u_c = P.v[9],
                uc_si = P.v[10];
        const T one = (T)1;
        T H1 = (u_c - u) >= 0 ? one : (T)0;
        T H2 = (u - u_c) >= 0 ? one : (T)0;
        T v = x.v + dt * (H1 * (one - x.v) / tau_v_m - H2 * x.v / tau_v_p);
        T w = x.w + dt * (H1 * (one - x.w) / tau_w_m - H2 * x.w / tau_w_p);
        x.v = v;
        x.w = w;
        T J_fi = -(v * H2 * (one - u) * (u - u_c)) / tau_d;
        T J_so = u * H1 / tau_o + H2 / tau_r;
        T J_si = (-v) * (one + fw_tanh(k * (u - uc_si))) / ((T)2 * tau_si);
        return un + dt * (-J_fi - J_so - J_si);
    }
};

// Barkley.  params: a, b, eap (barkley_2d.py:69-71, ionic_kernel_2d
// signature :141); calc_v (:114-138) then the voltage update with the new v
// (:141-170).
struct ModelBK {
    static constexpr int NS = 1, NP = 3;
    template <class T>
    struct St {
        T v;
    };
    template <class T>
    __device__ static __forceinline__ St<T> load(void *const *s, int64_t p)
    {
        return {((const T *)s[0])[p]};
    }
    template <class T>
    __device__ static __forceinline__ void store(void *const *s, int64_t p,
                                                 const St<T> &x)
    {
        ((T *)s[0])[p] = x.v;
    }
    template <class T>
    __device__ static __forceinline__ double probe(const St<T> &x, int)
    {
        return (double)x.v;
    }
    template <class T>
    __device__ static __forceinline__ St<T> from_array(const T *a)
    {
        return {a[0]};
    }
    template <class T>
    __device__ static __forceinline__ T update(T u, T un, St<T> &x,
                                               const Params<T, NP> &P, T dt)
    {
        const T a = P.v[0], b = P.v[1], eap = P.v[2];
        T v = x.v;
        v += dt * (u - v);
        x.v = v;
        return un + dt * (u * ((T)1 - u) * (u - (v + b) / a)) / eap;
    }
};

// Bueno-Orovio (minimal ventricular).  params in ionic_kernel_2d's order
// (bueno_orovio_2d.py, signature after the state arrays): u_o, u_u,
// theta_v, theta_w, theta_v_m, theta_o, tau_v1_m, tau_v2_m, tau_v_p,
// tau_w1_m, tau_w2_m, k_w_m, u_w_m, tau_w_p, tau_fi, tau_o1, tau_o2,
// tau_so1, tau_so2, k_so, u_so, tau_s1, tau_s2, k_s, u_s, tau_si, tau_w_inf,
// w_inf_.  calc_v, calc_w, calc_s, J_fi, J_so, J_si with the updated gates
// (ionic_kernel_2d, bueno_orovio_2d.py).
struct ModelBO {
    static constexpr int NS = 3, NP = 28;
    enum {
        u_o, u_u, theta_v, theta_w, theta_v_m, theta_o, tau_v1_m, tau_v2_m,
        tau_v_p, tau_w1_m, tau_w2_m, k_w_m, u_w_m, tau_w_p, tau_fi, tau_o1,
        tau_o2, tau_so1, tau_so2, k_so, u_so, tau_s1, tau_s2, k_s, u_s, tau_si,
        tau_w_inf, w_inf_
    };
    template <class T>
    struct St {
        T v, w, s;
    };
    template <class T>
    __device__ static __forceinline__ St<T> load(void *const *s, int64_t p)
    {
        return {((const T *)s[0])[p], ((const T *)s[1])[p],
                ((const T *)s[2])[p]};
    }
    template <class T>
    __device__ static __forceinline__ void store(void *const *s, int64_t p,
                                                 const St<T> &x)
    {
        ((T *)s[0])[p] = x.v;
        ((T *)s[1])[p] = x.w;
        ((T *)s[2])[p] = x.s;
    }
    template <class T>
    __device__ static __forceinline__ double probe(const St<T> &x, int i)
    {
        return i == 0 ? (double)x.v : i == 1 ? (double)x.w : (double)x.s;
    }
    template <class T>
    __device__ static __forceinline__ St<T> from_array(const T *a)
    {
        return {a[0], a[1], a[2]};
    }
    template <class T>
    __device__ static __forceinline__ T update(T u, T un, St<T> &x,
                                               const Params<T, NP> &P, T dt)
    {
        const T one = (T)1, two = (T)2;
        // calc_v_inf, calc_tau_v_m, calc_v
        const T v_inf = u < P.v[theta_v_m] ? one : (T)0;
        const T tau_v_m = (u - P.v[theta_v_m]) < 0 ? P.v[tau_v1_m] : P.v[tau_v2_m];
        const T dv = (u - P.v[theta_v]) < 0 ? (v_inf - x.v) / tau_v_m
                                            : -x.v / P.v[tau_v_p];
        x.v += dt * dv;
        // calc_w_inf, calc_tau_w_m, calc_w
        const T w_inf = (u - P.v[theta_o]) < 0 ? one - u / P.v[tau_w_inf]
                                               : P.v[w_inf_];
        const T tau_w_m = P.v[tau_w1_m] + (P.v[tau_w2_m] - P.v[tau_w1_m]) *
                                              (one + fw_tanh(P.v[k_w_m] * (u - P.v[u_w_m]))) /
                                              two;
        const T dw = (u - P.v[theta_w]) < 0 ? (w_inf - x.w) / tau_w_m
                                            : -x.w / P.v[tau_w_p];
        x.w += dt * dw;
        // calc_tau_s, calc_s
        const T tau_s = (u - P.v[theta_w]) < 0 ? P.v[tau_s1] : P.v[tau_s2];
        x.s += dt * ((one + fw_tanh(P.v[k_s] * (u - P.v[u_s]))) / two - x.s) /
               tau_s;
        // calc_Jfi, calc_Jso (calc_tau_o, calc_tau_so), calc_Jsi
        const T Hv = (u - P.v[theta_v]) >= 0 ? one : (T)0;
        const T J_fi = -x.v * Hv * (u - P.v[theta_v]) * (P.v[u_u] - u) / P.v[tau_fi];
        const T tau_o = (u - P.v[theta_o]) < 0 ? P.v[tau_o1] : P.v[tau_o2];
        const T tau_so = P.v[tau_so1] + (P.v[tau_so2] - P.v[tau_so1]) *
                                            (one + fw_tanh(P.v[k_so] * (u - P.v[u_so]))) /
                                            two;
        const T Hw = (u - P.v[theta_w]) >= 0 ? one : (T)0;
        const T J_so = (u - P.v[u_o]) * (one - Hw) / tau_o + Hw / tau_so;
        const T J_si = -Hw * x.w * x.s / P.v[tau_si];
        return un + dt * (-J_fi - J_so - J_si);
    }
};

}  // namespace fw
