// wg_cells.cuh — per-cell building blocks shared by the stepping kernels: field and
// mask accessors, coefficient sources, 16-byte vector loads, and the boundary-line
// rules of the native forms.
#pragma once
#include "wg_internal.h"

namespace wg {

// ---------------------------------------------------------------------------
// Accessors
// ---------------------------------------------------------------------------
template <class T>
struct Field {
    const T *a;
    int pitch;
    __device__ __forceinline__ T operator()(int i, int j) const { return a[(size_t)i * pitch + j]; }
};
// psi of an FP32 scene: phi - v in FP64
struct PsiOfVel {
    const float *x, *v;
    int pitch;
    __device__ __forceinline__ double operator()(int i, int j) const
    {
        const size_t o = (size_t)i * pitch + j;
        return S_((double)x[o], (double)v[o]);
    }
};
struct ActI16 {
    const int16_t *a;
    int pitch;
    __device__ __forceinline__ int operator()(int i, int j) const { return a[(size_t)i * pitch + j] != 0; }
};
struct ActBits {
    const uint32_t *w;
    int wpitch;
    __device__ __forceinline__ int operator()(int i, int j) const
    {
        return (w[(size_t)i * wpitch + (j >> 5)] >> (j & 31)) & 1u;
    }
};
template <class T>
struct CoefTab {
    const T *tcc_, *tc_, *tg_;
    int pitch;
    double gam;
    __device__ __forceinline__ double tcc(int i, int j) const { return (double)tcc_[(size_t)i * pitch + j]; }
    __device__ __forceinline__ double tc(int i, int j) const { return tc_ ? (double)tc_[(size_t)i * pitch + j] : 0.0; }
    __device__ __forceinline__ double tg(int i, int j) const { return tg_ ? (double)tg_[(size_t)i * pitch + j] : gam; }
};
struct CoefMask {
    ActBits act;
    double c2, c2b, gam, gamb, c, cb;
    __device__ __forceinline__ double tcc(int i, int j) const { return act(i, j) ? c2 : c2b; }
    __device__ __forceinline__ double tc(int i, int j) const { return act(i, j) ? c : cb; }
    __device__ __forceinline__ double tg(int i, int j) const { return act(i, j) ? gam : gamb; }
};

template <class T> struct Vec;
template <> struct Vec<float> { using type = float4; static constexpr int n = 4; };
template <> struct Vec<double> { using type = double2; static constexpr int n = 2; };

template <class T>
__device__ __forceinline__ void vload(const T *ptr, T (&v)[Vec<T>::n])
{
    typename Vec<T>::type t = *reinterpret_cast<const typename Vec<T>::type *>(ptr);
    const T *s = reinterpret_cast<const T *>(&t);
#pragma unroll
    for (int k = 0; k < Vec<T>::n; k++) v[k] = s[k];
}
template <class T>
__device__ __forceinline__ void vstore(T *ptr, const T (&v)[Vec<T>::n])
{
    typename Vec<T>::type t;
    T *d = reinterpret_cast<T *>(&t);
#pragma unroll
    for (int k = 0; k < Vec<T>::n; k++) d[k] = v[k];
    *reinterpret_cast<typename Vec<T>::type *>(ptr) = t;
}

// FP32 boundary-line cell: mirror, periodic and absorbing scenes by edge32 (the rule of
// the tiled and skewed FP32 steppers), neighbours read from the current level (wrapped
// around the grid for periodic scenes); the other boundary conditions by the reference
// rule of edge_cell in FP64 on psi = phi - v, the velocity being the FP64 change rounded
// once.  FLOOR on cells whose mask is nonzero.
template <int COEF>
__device__ inline XV fast_edge_v(const DevParams &p, const FastArgs<float> &a, int i, int j, long long time)
{
    const size_t o = (size_t)i * p.pitch + j;
    const float x = a.phi[o], y = a.psi[o];
    XV r;
    if (p.b_cond == WG_BC_DIRICHLET || p.b_cond == WG_BC_ABSORBING || p.b_cond == WG_BC_PERIODIC) {
        const bool per = p.b_cond == WG_BC_PERIODIC;
        const int ip = (i + 1 < p.nx) ? i + 1 : (per ? 0 : i), im = (i > 0) ? i - 1 : (per ? p.nx - 1 : i);
        const int jp = (j + 1 < p.ny) ? j + 1 : (per ? 0 : j), jm = (j > 0) ? j - 1 : (per ? p.ny - 1 : j);
        const float n = a.phi[(size_t)ip * p.pitch + j];
        const float sv = a.phi[(size_t)im * p.pitch + j];
        const float e = a.phi[(size_t)i * p.pitch + jp];
        const float w = a.phi[(size_t)i * p.pitch + jm];
        const bool act = ActBits{a.act, p.wpitch}(i, j);
        float ccv, tcv, g;
        if (COEF == WG_COEF_TABLE) {
            ccv = a.tcc[o];
            tcv = a.tc ? a.tc[o] : 0.f;
            g = a.tg ? a.tg[o] : a.gamf;
        } else {
            ccv = act ? a.c2f : a.c2bf;
            tcv = act ? a.courantf : a.courantbf;
            g = act ? a.gamf : a.gambf;
        }
        const Edge32K k{a.kappaf, a.ksf, a.ktf, a.gsf, a.gtf, a.vmaxf};
        r = edge32<false>(p, i, j, x, y, n, sv, e, w, ccv, tcv, g, act, k,
                          [&] { return (float)osc_bc(p, (int)time, j); });
    } else {
        Field<float> PHI{a.phi, p.pitch};
        PsiOfVel PSI{a.phi, a.psi, p.pitch};
        ActBits ACT{a.act, p.wpitch};
        double v;
        bool w;
        if (COEF == WG_COEF_MASK) {
            CoefMask CF{ACT, p.c2, p.c2b, p.gam, p.gamb, p.courant, p.courantb};
            w = edge_cell<float>(p, time, i, j, PHI, PSI, ACT, CF, &v);
        } else {
            CoefTab<float> CF{a.tcc, a.tc, a.tg, p.pitch, p.gam};
            w = edge_cell<float>(p, time, i, j, PHI, PSI, ACT, CF, &v);
        }
        r = w ? XV{(float)v, (float)S_(v, (double)x)} : keep32(x, y);
    }
    if (p.floor_clamp && ActBits{a.nz, p.wpitch}(i, j)) r = clamp32(x, r, a.vmaxf);
    return r;
}

// Boundary-line cell of the native FP64 form, reference rules.  Returns the value to
// store (the old psi value y when the reference writes nothing).
template <class T, int COEF>
__device__ inline T fast_edge(const DevParams &p, const FastArgs<T> &a, int i, int j, long long time, T y)
{
    Field<T> PHI{a.phi, p.pitch}, PSI{a.psi, p.pitch};
    ActBits ACT{a.act, p.wpitch}, NZ{a.nz, p.wpitch};
    double v;
    bool w;
    if (COEF == WG_COEF_MASK) {
        CoefMask CF{ACT, p.c2, p.c2b, p.gam, p.gamb, p.courant, p.courantb};
        w = edge_cell<T>(p, time, i, j, PHI, PSI, ACT, CF, &v);
    } else {
        CoefTab<T> CF{a.tcc, a.tc, a.tg, p.pitch, p.gam};
        w = edge_cell<T>(p, time, i, j, PHI, PSI, ACT, CF, &v);
    }
    if (!w) v = (double)y;
    if (p.floor_clamp && NZ(i, j)) v = floor_clamp(p, v);
    return (T)v;
}

}  // namespace wg
