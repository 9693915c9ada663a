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
        v += (-dt) * (eap + (mu_1 * v) / (mu_2 + u)) *
             (v + k * u * (u - a - (T)1.));
        x.v = v;
        return un + dt * ((-k) * u * (u - a) * (u - (T)1.) - u * v);
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

}  // namespace fw
