// wg_kernels.cu — single-update stepping kernels, Neumann gather, point source,
// energy reductions and small utility kernels for sm_103a.
//
//  k_step_exact   drop-in form: int16 mask, FP64 tables, three buffers, writes exactly
//                 the cells wave_billiard.c:302-610 writes (bit-identical FP64).
//  k_step_bulk    native form, interior rows: 1-bit masks, 16-byte vector loads along
//                 j; FP64 (reference operation order) in place (the new level
//                 overwrites psi), or FP32 (phi and velocity, increment form) into the
//                 other pair of fields.
//  k_step_edge    native form, the four boundary lines and the point source.
//  k_neumann      Neumann gather of wave_billiard.c:379-389 for the active records.
//  k_energy_cols  compute_energy (wave_common.c:453-472) per cell, one warp per
//                 column: sums of j < ny/2 and j >= ny/2, box partials per block.
//  k_energy_final total and the six compute_energy_tblr boxes from the partials.
#include <type_traits>
#include "wg_internal.h"
#include "wg_cells.cuh"

namespace wg {

// ---------------------------------------------------------------------------
// Exact drop-in kernel
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_step_exact(DevParams p, const double *__restrict__ phi,
                                                    const double *__restrict__ psi, double *__restrict__ out,
                                                    const int16_t *__restrict__ xy, const double *__restrict__ tcc,
                                                    const double *__restrict__ tc, const double *__restrict__ tg,
                                                    long long time, int do_source)
{
    pdl_wait();  // launched by launch_pdl: the previous update has completed
    pdl_trigger();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= p.nx || j >= p.ny) return;
    const size_t c = (size_t)i * p.pitch + j;
    const int m = xy[c];
    double v = 0.0;
    bool w;
    if (i == 0 || i == p.nx - 1 || j == 0 || j == p.ny - 1) {
        Field<double> PHI{phi, p.pitch}, PSI{psi, p.pitch};
        ActI16 ACT{xy, p.pitch};
        CoefTab<double> CF{tcc, tc, tg, p.pitch, 0.0};
        w = edge_cell<double>(p, time, i, j, PHI, PSI, ACT, CF, &v);
    } else {
        w = p.twospeeds || m > 0;
        if (w) {
            const double x = phi[c], y = psi[c];
            const double delta = L4_(A_(A_(A_(phi[c + p.pitch], phi[c - p.pitch]), phi[c + 1]), phi[c - 1]), x);
            v = upd64(x, y, tcc[c], delta, p.kappa, tg[c]);
        }
    }
    if (p.floor_clamp && m != 0) {
        if (!w) { v = out[c]; w = true; }
        v = floor_clamp(p, v);
    }
    if (do_source && p.src_on && i == p.src_i && j == p.src_j) {
        if (!w) { v = out[c]; w = true; }
        v = A_(v, point_source(p, time));
    }
    if (w) out[c] = v;
}

// wave_energy's stepper (wave_energy.c:662-913) on the half domain j < ny/2, with
// its tables built from the mask (wave_energy.c:670-697).  The OSCILLATE_TOPBOT
// branch of that file reads outside its tables and is rejected on the host.
__global__ void __launch_bounds__(256) k_step_exact_energy(DevParams p, const double *__restrict__ phi,
                                                           const double *__restrict__ psi, double *__restrict__ out,
                                                           const int16_t *__restrict__ xy, long long time)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int NX = p.nx, jmid = p.ny / 2;
    if (i >= NX || j >= jmid) return;
    const int P = p.pitch;
    auto PHI = [&](int a, int b) { return phi[(size_t)a * P + b]; };
    auto XY = [&](int a, int b) { return (int)xy[(size_t)a * P + b]; };
    auto TCC = [&](int a, int b) { return XY(a, b) ? p.c2 : (p.twospeeds ? p.c2b : 0.0); };
    auto TC = [&](int a, int b) { return XY(a, b) ? p.courant : (p.twospeeds ? p.courantb : 0.0); };
    auto TG = [&](int a, int b) { return XY(a, b) ? p.gam : (p.twospeeds ? p.gamb : 0.0); };
    const size_t c = (size_t)i * P + j;
    const int m = XY(i, j);
    const bool active = p.twospeeds || m != 0;
    const double x = phi[c], y = psi[c];
    double v = 0.0, delta;
    bool w = false;
    if (j == jmid - 1 || j == 0) {
        const int jb = j, jn = (j == 0) ? 1 : jmid - 2, jw = (j == 0) ? jmid - 1 : 0;
        if (i == 0 && j == jmid - 1 && p.osc_left) { v = osc_bc(p, (int)time, j); w = true; }
        if (active) {
            int ip, im;
            switch (p.b_cond) {
            case 0:
                ip = i + 1; if (ip == NX) ip = NX - 1;
                im = i - 1; if (im == -1) im = 0;
                delta = S_(A_(A_(PHI(ip, jb), PHI(im, jb)), PHI(i, jn)), M_(3.0, x));
                v = upd64(x, y, TCC(i, jb), delta, p.kappa, TG(i, jb));
                break;
            case 1:
                ip = (i + 1) % NX; im = (i - 1) % NX; if (im < 0) im += NX;
                delta = S_(A_(A_(A_(PHI(ip, jb), PHI(im, jb)), PHI(i, jn)), PHI(i, jw)), M_(4.0, x));
                v = upd64(x, y, TCC(i, jb), delta, p.kappa, TG(i, jb));
                break;
            case 2:
                v = absorb64(x, y, TC(i, jb), PHI(i, jn), p.kappa_topbot, p.gamma_topbot);
                break;
            default:
                ip = i + 1; if (ip == NX) ip = NX - 1;
                im = i - 1; if (im == -1) im = 0;
                if (i == 0) v = absorb64(x, y, TC(0, jb), PHI(1, jb), p.kappa_sides, p.gamma_sides);
                else {
                    delta = S_(A_(A_(A_(PHI(ip, jb), PHI(im, jb)), PHI(i, jn)), PHI(i, jw)), M_(4.0, x));
                    v = upd64(x, y, TCC(i, jb), delta, p.kappa, TG(i, jb));
                }
                break;
            }
            w = true;
        }
    } else if (i == 0 && p.osc_left) {
        v = osc_bc(p, (int)time, j);
        w = true;
    } else if (i == 0 || i == NX - 1) {
        if (active) {
            const int in = (i == 0) ? 1 : NX - 2, iw = (i == 0) ? NX - 1 : 0;
            switch (p.b_cond) {
            case 0:
                delta = S_(A_(A_(PHI(in, j), PHI(i, j + 1)), PHI(i, j - 1)), M_(3.0, x));
                v = upd64(x, y, TCC(i, j), delta, p.kappa, TG(i, j));
                break;
            case 1:
                delta = S_(A_(A_(A_(PHI(in, j), PHI(iw, j)), PHI(i, j + 1)), PHI(i, j - 1)), M_(4.0, x));
                v = upd64(x, y, TCC(i, j), delta, p.kappa, TG(i, j));
                break;
            default:
                v = absorb64(x, y, TC(i, j), PHI(in, j), p.kappa_sides, p.gamma_sides);
                break;
            }
            w = true;
        }
    } else if (active) {
        delta = S_(A_(A_(A_(PHI(i + 1, j), PHI(i - 1, j)), PHI(i, j + 1)), PHI(i, j - 1)), M_(4.0, x));
        v = upd64(x, y, TCC(i, j), delta, p.kappa, TG(i, j));
        w = true;
    }
    if (p.floor_clamp && m != 0) {
        if (!w) { v = out[c]; w = true; }
        v = floor_clamp(p, v);
    }
    if (w) out[c] = v;
}

__global__ void k_cell_energy(DevParams p, const double *phi, const double *psi, const int16_t *xy, int i, int j,
                              double *out)
{
    const int NX = p.nx, NY = p.ny, P = p.pitch;
    const int ip = (i + 1 == NX) ? NX - 1 : i + 1, im = (i == 0) ? 0 : i - 1;
    const int jp = (j + 1 == NY) ? NY - 1 : j + 1, jm = (j == 0) ? 0 : j - 1;
    const size_t c = (size_t)i * P + j;
    *out = cell_energy(p, phi[c], psi[c], phi[(size_t)ip * P + j], phi[(size_t)im * P + j], phi[(size_t)i * P + jp],
                       phi[(size_t)i * P + jm], xy[c] != 0);
}

// Neumann gather for active records (drop-in form; records pre-validated to lie in
// 1..nx-2 x 1..ny-2 with in-range neighbours).
__global__ void k_neumann_exact(DevParams p, const double *__restrict__ phi, double *__restrict__ out,
                                const int16_t *__restrict__ xy, const wg_neumann_bc *__restrict__ rec, int n)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const wg_neumann_bc r = rec[q];
    if (!r.active) return;
    const size_t c = (size_t)r.i * p.pitch + r.j;
    double v = M_(r.nx, phi[(size_t)r.nbi1 * p.pitch + r.nbj1]);
    v = A_(v, M_(r.ny, phi[(size_t)r.nbi2 * p.pitch + r.nbj2]));
    if (p.floor_clamp && xy[c] != 0) v = floor_clamp(p, v);
    out[c] = v;
}

// vout (FP32 fields): the velocity takes the increment too.
template <class T>
__global__ void k_point_source(DevParams p, T *out, T *vout, long long time)
{
    const size_t c = (size_t)p.src_i * p.pitch + p.src_j;
    const double add = point_source(p, time);
    out[c] = (T)A_((double)out[c], add);
    if (vout) vout[c] = (T)A_((double)vout[c], add);
}

// ---------------------------------------------------------------------------
// Fast native kernel
// ---------------------------------------------------------------------------
// Interior rows 1..nx-2 of one update: each thread updates V = 16/sizeof(T) consecutive
// cells of row i with every load (three phi rows, psi or the velocity, tcc, the j-1 / j+V
// neighbours, the mask word) issued before the first use.  FP64: in place, the new level
// overwriting psi.  FP32: the new phi and velocity into the other pair.  Boundary-line
// cells (j = 0, j = ny-1) and padding take the rule of an unwritten cell; k_step_edge
// computes the boundary lines afterwards.
template <class T, int COEF, int Z = 0>
__global__ void __launch_bounds__(256) k_step_bulk(const __grid_constant__ DevParams p,
                                                   const __grid_constant__ FastArgs<T> a)
{
    constexpr int V = Vec<T>::n;
    pdl_wait();  // launched by launch_pdl: the previous update has completed
    pdl_trigger();
    const int i = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int j0 = (blockIdx.x * blockDim.x + threadIdx.x) * V;
    if (i >= p.nx - 1 || j0 >= p.pitch) return;
    const size_t row = (size_t)i * p.pitch;
    T c[V], y[V], n[V], s[V], cc[V];
    vload(a.phi + row + j0, c);
    vload(a.psi + row + j0, y);
    vload(a.phi + row + p.pitch + j0, n);
    vload(a.phi + row - p.pitch + j0, s);
    if (COEF == WG_COEF_TABLE) vload(a.tcc + row + j0, cc);
    const T wl = (j0 > 0) ? a.phi[row + j0 - 1] : (T)0;
    const T er = (j0 + V < p.pitch) ? a.phi[row + j0 + V] : (T)0;
    const uint32_t word = a.act[(size_t)i * p.wpitch + (j0 >> 5)] >> (j0 & 31);
    uint32_t nzw = 0;
    if (p.floor_clamp && a.has_ghosts) nzw = a.nz[(size_t)i * p.wpitch + (j0 >> 5)] >> (j0 & 31);
    T out[V], vo[V];
#pragma unroll
    for (int k = 0; k < V; k++) {
        const int j = j0 + k;
        const bool act = (word >> k) & 1u;
        const bool upd = j >= 1 && j < p.ny - 1 && (p.twospeeds || act);
        const bool clamp = p.floor_clamp && j >= 1 && j < p.ny - 1 && ((upd && act) || ((nzw >> k) & 1u));
        const T x = c[k];
        const T w = (k == 0) ? wl : c[k - 1];
        const T e = (k == V - 1) ? er : c[k + 1];
        if constexpr (sizeof(T) == 8) {
            double v = y[k];
            if (upd) {
                const double delta = L4_(A_(A_(A_(n[k], s[k]), e), w), x);
                const double ccv = (COEF == WG_COEF_TABLE) ? (double)cc[k] : (act ? p.c2 : p.c2b);
                double g;
                if (COEF == WG_COEF_TABLE) g = a.tg ? (double)a.tg[row + j] : p.gam;
                else g = act ? p.gam : p.gamb;
                v = upd64<Z>(x, y[k], ccv, delta, p.kappa, g);
            }
            if (clamp) v = floor_clamp(p, v);
            out[k] = (T)v;
        } else {
            XV r = keep32(x, y[k]);
            if (upd) {
                const float delta = ((n[k] - x) + (s[k] - x)) + ((e - x) + (w - x));
                const float ccv = (COEF == WG_COEF_TABLE) ? cc[k] : (act ? a.c2f : a.c2bf);
                float g;
                if (COEF == WG_COEF_TABLE) g = a.tg ? a.tg[row + j] : a.gamf;
                else g = act ? a.gamf : a.gambf;
                r = upd32(x, y[k], ccv, delta, a.kappaf, g);
            }
            if (clamp) r = clamp32(x, r, a.vmaxf);
            out[k] = r.x;
            vo[k] = r.v;
        }
    }
    vstore(a.out + row + j0, out);
    if constexpr (sizeof(T) == 4) vstore(a.vout + row + j0, vo);
}

// The four boundary lines of one update (one thread per cell, reference rules) and,
// in the last thread, the point source when it lies inside; runs after k_step_bulk
// (boundary cells read only phi and their own psi or velocity).
template <class T, int COEF>
__global__ void __launch_bounds__(256) k_step_edge(const __grid_constant__ DevParams p,
                                                   const __grid_constant__ FastArgs<T> a, long long time)
{
    pdl_wait();  // launched by launch_pdl: the bulk kernel of this update has completed
    pdl_trigger();
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int NX = p.nx, NY = p.ny;
    const int nedge = 2 * NX + 2 * (NY - 2);
    int i, j;
    if (idx < NX) { i = idx; j = 0; }
    else if (idx < 2 * NX) { i = idx - NX; j = NY - 1; }
    else if (idx < 2 * NX + (NY - 2)) { i = 0; j = idx - 2 * NX + 1; }
    else if (idx < nedge) { i = NX - 1; j = idx - 2 * NX - (NY - 2) + 1; }
    else {
        if (idx == nedge && a.do_source && p.src_on && p.src_i > 0 && p.src_i < NX - 1 && p.src_j > 0 &&
            p.src_j < NY - 1) {
            const size_t o = (size_t)p.src_i * p.pitch + p.src_j;
            const double add = point_source(p, time);
            a.out[o] = (T)A_((double)a.out[o], add);
            if constexpr (sizeof(T) == 4) a.vout[o] = (T)A_((double)a.vout[o], add);
        }
        return;
    }
    const size_t o = (size_t)i * p.pitch + j;
    const bool src = a.do_source && p.src_on && i == p.src_i && j == p.src_j;
    if constexpr (sizeof(T) == 8) {
        T v = fast_edge<T, COEF>(p, a, i, j, time, a.psi[o]);
        if (src) v = (T)A_((double)v, point_source(p, time));
        a.out[o] = v;
    } else {
        XV r = fast_edge_v<COEF>(p, a, i, j, time);
        if (src) r = source32(r, point_source(p, time));
        a.out[o] = r.x;
        a.vout[o] = r.v;
    }
}

// Native Neumann gather: active records only, from phi (level t) into the new level
// (vout: FP32 fields, the velocity of the gathered value against the cell's phi at level
// t, in FP64).
template <class T>
__global__ void k_neumann_fast(DevParams p, const T *__restrict__ phi, T *__restrict__ out, T *__restrict__ vout,
                               const int4 *__restrict__ idx, const double2 *__restrict__ w, int n)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int4 r = idx[q];       // cell, nb1, nb2 (element offsets), flags (bit0 floor, bit1 inactive)
    if (r.w & 2) return;
    const double2 cw = w[q];
    double v = M_(cw.x, (double)phi[r.y]);
    v = A_(v, M_(cw.y, (double)phi[r.z]));
    if (p.floor_clamp && (r.w & 1)) v = floor_clamp(p, v);
    out[r.x] = (T)v;
    if (vout) vout[r.x] = (T)S_(v, (double)phi[r.x]);
}

// ---------------------------------------------------------------------------
// Energy
// ---------------------------------------------------------------------------
// Error-free FP32 double-word ("double-float") accumulator: h + l carries the running
// sum to about 2^-48 relative.  Every addition is Knuth's TwoSum (the rounding error of
// h + x, recovered exactly, goes into l); merges add the two high words by TwoSum and
// renormalise.  All of it runs on the FP32 pipe: on this GPU an FP64 operation costs
// about 64 FP32 operations, so the FP32 fields' sums stay off the FP64 pipe and are
// converted to FP64 (exactly) only per column.
// An aggregate like Neu: start it as {0.f, 0.f}.
struct DF {
    float h, l;
    __device__ __forceinline__ void add(float x)
    {
        const float s = __fadd_rn(h, x);
        const float bp = __fsub_rn(s, h);
        const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bp)), __fsub_rn(x, bp));
        h = s;
        l = __fadd_rn(l, e);
    }
    __device__ __forceinline__ void merge(const DF &o)
    {
        const float s = __fadd_rn(h, o.h);
        const float bp = __fsub_rn(s, h);
        const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bp)), __fsub_rn(o.h, bp));
        const float t = __fadd_rn(__fadd_rn(l, o.l), e);
        h = __fadd_rn(s, t);                  // Fast2Sum renormalisation (|s| >= |t|)
        l = __fsub_rn(t, __fsub_rn(h, s));
    }
    __device__ __forceinline__ double value() const { return A_((double)h, (double)l); }
};

// compute_energy in FP32 for FP32 fields (same formula and order as cell_energy), with
// the stored velocity v in place of phi - psi.
__device__ __forceinline__ float cell_energy32(float es2, float hc2, float hc2b, int twospeeds, float x, float v,
                                               float e, float w, float n, float s, int m)
{
    float a = e - x, b = x - w, c = n - x, d = x - s;
    float g = (a * a + b * b) + (c * c + d * d);
    if (m) return es2 * (v * v + hc2 * g);
    if (twospeeds) return es2 * (v * v + hc2b * g);
    return 0.0f;
}

// Merges the accumulators of the 32 lanes into lane 0 (value and compensation travel).
__device__ __forceinline__ void warp_merge(Neu &a)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        Neu o = {0.0, 0.0};
        o.s = __shfl_down_sync(0xffffffffu, a.s, off);
        o.c = __shfl_down_sync(0xffffffffu, a.c, off);
        a.merge(o);
    }
}
__device__ __forceinline__ void warp_merge(DF &a)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        DF o = {0.f, 0.f};
        o.h = __shfl_down_sync(0xffffffffu, a.h, off);
        o.l = __shfl_down_sync(0xffffffffu, a.l, off);
        a.merge(o);
    }
}
__device__ __forceinline__ void acc_add(Neu &a, double x) { a.add(x); }
__device__ __forceinline__ void acc_add(DF &a, float x) { a.add(x); }
__device__ __forceinline__ void acc_merge(Neu &a, const Neu &o) { a.merge(o); }
__device__ __forceinline__ void acc_merge(DF &a, const DF &o) { a.merge(o); }

// One warp per column i, eight columns per block.  MASK: 0 = int16 (xy != 0), 1 =
// "nonzero" bit plane.  Per cell compute_energy (wave_common.c:453-472): FP64 for FP64
// fields, FP32 for FP32 fields.  Every reduction is compensated: FP64 fields add their
// cell energies into FP64 Neumaier accumulators; FP32 fields into the error-free FP32
// double-word accumulator DF above.  Lanes merge (value and compensation) into the
// column sums of compute_energy_x (wave_energy.c:292-302); the block merges the six
// boxes of compute_energy_tblr (sub_wave_comp.c:1752-1800) over its columns, and its
// total.  cols[i] = (sum over j < ny/2, sum over j >= ny/2); part[6 b + k] = box k of
// block b (0..2 top left/mid/right, 3..5 bottom); the block's total overwrites
// cols[8 b].y (already folded into the boxes).  FP32 fields: psi is the velocity.
#define ENERGY_COLS_PER_BLOCK 8
template <class T, int MASK>
__global__ void __launch_bounds__(32 * ENERGY_COLS_PER_BLOCK)
    k_energy_cols(const __grid_constant__ DevParams p, const T *__restrict__ phi, const T *__restrict__ psi,
                  const int16_t *__restrict__ xy, const uint32_t *__restrict__ nz, int ileft, int iright,
                  double2 *__restrict__ cols, double *__restrict__ part)
{
    using Acc = typename std::conditional<sizeof(T) == 8, Neu, DF>::type;
    __shared__ Acc sh[ENERGY_COLS_PER_BLOCK][2];
    __shared__ Acc sbx[6];
    __shared__ int sbox[ENERGY_COLS_PER_BLOCK];
    pdl_wait();  // launched by launch_pdl: the update that wrote the fields has completed
    pdl_trigger();
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * ENERGY_COLS_PER_BLOCK + wid;
    Acc ab = {0, 0}, at = {0, 0};  // bottom (j < ny/2) and top halves of the column
    if (i < p.nx) {
        const int NX = p.nx, NY = p.ny, jmid = NY / 2;
        const size_t row = (size_t)i * p.pitch;
        const int ip = (i + 1 == NX) ? NX - 1 : i + 1, im = (i == 0) ? 0 : i - 1;
        const T *re = phi + (size_t)ip * p.pitch, *rw = phi + (size_t)im * p.pitch, *rc = phi + row, *ry = psi + row;
        const float es2 = (float)p.e_scale2, hc2 = (float)p.ehalf_c2, hc2b = (float)p.ehalf_c2b;
        if (sizeof(T) == 4 && MASK == 1) {
            // FP32 fields: four cells per lane and step as 16-byte loads of the rows i-1, i, i+1
            // and the velocity; the j-1 / j+1 neighbours from the adjacent lanes (the row pitch is a
            // multiple of 128 elements, so every load stays in the row)
            const float *fc = (const float *)rc, *fy = (const float *)ry, *fe = (const float *)re,
                        *fw = (const float *)rw;
            const uint32_t *nzr = nz + (size_t)i * p.wpitch;
            for (int base = 0; base < NY; base += 128) {
                const int j0 = base + 4 * lane;
                const float4 c4 = *reinterpret_cast<const float4 *>(fc + j0);
                const float4 y4 = *reinterpret_cast<const float4 *>(fy + j0);
                const float4 e4 = *reinterpret_cast<const float4 *>(fe + j0);
                const float4 w4 = *reinterpret_cast<const float4 *>(fw + j0);
                float left = __shfl_up_sync(0xffffffffu, c4.w, 1), right = __shfl_down_sync(0xffffffffu, c4.x, 1);
                if (lane == 0) left = (j0 > 0) ? fc[j0 - 1] : c4.x;
                if (lane == 31) right = (j0 + 4 < NY) ? fc[j0 + 4] : c4.w;
                const uint32_t bits = (nzr[j0 >> 5] >> (j0 & 31)) & 0xFu;
                const float xs[4] = {c4.x, c4.y, c4.z, c4.w}, ys[4] = {y4.x, y4.y, y4.z, y4.w};
                const float es[4] = {e4.x, e4.y, e4.z, e4.w}, ws[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int j = j0 + k;
                    if (j >= NY) break;
                    float jn = (k < 3) ? xs[k < 3 ? k + 1 : 3] : right;
                    float js = (k > 0) ? xs[k > 0 ? k - 1 : 0] : left;
                    if (j == NY - 1) jn = xs[k];  // clamped at the boundary lines
                    if (j == 0) js = xs[k];
                    const float en = cell_energy32(es2, hc2, hc2b, p.twospeeds, xs[k], ys[k], es[k], ws[k], jn, js,
                                                   (int)((bits >> k) & 1u));
                    acc_add(j < jmid ? ab : at, en);
                }
            }
        } else {
#pragma unroll 4
            for (int j = lane; j < NY; j += 32) {
                const int jp = (j + 1 == NY) ? NY - 1 : j + 1, jm = (j == 0) ? 0 : j - 1;
                int m;
                if (MASK == 0) m = xy[row + j] != 0;
                else m = (nz[(size_t)i * p.wpitch + (j >> 5)] >> (j & 31)) & 1u;
                if (sizeof(T) == 8) {
                    const double en = cell_energy(p, (double)rc[j], (double)ry[j], (double)re[j], (double)rw[j],
                                                  (double)rc[jp], (double)rc[jm], m);
                    acc_add(j < jmid ? ab : at, en);
                } else {
                    const float en = cell_energy32(es2, hc2, hc2b, p.twospeeds, (float)rc[j], (float)ry[j],
                                                   (float)re[j], (float)rw[j], (float)rc[jp], (float)rc[jm], m);
                    acc_add(j < jmid ? ab : at, en);
                }
            }
        }
    }
    warp_merge(ab);
    warp_merge(at);
    if (lane == 0) {
        if (i < p.nx) cols[i] = make_double2(ab.value(), at.value());
        sh[wid][0] = ab;
        sh[wid][1] = at;
        sbox[wid] = (i < ileft) ? 0 : (i < iright ? 1 : 2);
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x, box = k % 3, half = k < 3 ? 1 : 0;  // top boxes sum j >= ny/2
        Acc acc = {0, 0};
#pragma unroll
        for (int w = 0; w < ENERGY_COLS_PER_BLOCK; w++)
            if (sbox[w] == box) acc_merge(acc, sh[w][half]);
        part[(size_t)blockIdx.x * 6 + k] = acc.value();
        sbx[k] = acc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        Acc t = {0, 0};
#pragma unroll
        for (int k = 0; k < 6; k++) acc_merge(t, sbx[k]);
        cols[(size_t)blockIdx.x * ENERGY_COLS_PER_BLOCK].y = t.value();
    }
}

// One warp per output: block k < 6 merges box k over the blocks of k_energy_cols into
// out[1 + k] (top left/mid/right, bottom left/mid/right); block 6 merges the blocks'
// totals into out[0]; all of them copy the column sums over j < ny/2 into out[7..7+nx).
// FP64 Neumaier per lane, then merged across the warp.
__global__ void __launch_bounds__(32) k_energy_final(int nx, int nblocks, const double2 *__restrict__ cols,
                                                     const double *__restrict__ part, double *__restrict__ out)
{
    pdl_wait();  // launched by launch_pdl: k_energy_cols has completed
    pdl_trigger();
    const int k = blockIdx.x, lane = threadIdx.x;
    for (int i = k * 32 + lane; i < nx; i += 7 * 32) out[7 + i] = cols[i].x;
    Neu acc = {0.0, 0.0};
    for (int b = lane; b < nblocks; b += 32)
        acc.add(k < 6 ? part[(size_t)b * 6 + k] : cols[(size_t)b * ENERGY_COLS_PER_BLOCK].y);
    warp_merge(acc);
    if (lane == 0) out[k < 6 ? 1 + k : 0] = acc.value();
}

// ---------------------------------------------------------------------------
// Utilities
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_count_nonfinite(int nx, int ny, int pitch, const T *__restrict__ a, unsigned long long *count)
{
    unsigned long long local = 0;
    const size_t total = (size_t)nx * pitch;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < total; c += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(c % pitch);
        if (j < ny && !isfinite((double)a[c])) local++;
    }
    if (local) atomicAdd(count, local);
}

// Packs the int16 mask into the "active" plane (bulk test xy > 0, boundary-line test
// xy != 0) and the "nonzero" plane (xy != 0).  One thread per 32-bit word.
__global__ void k_pack_mask(int nx, int ny, int wpitch, const int16_t *__restrict__ xy, uint32_t *__restrict__ act,
                            uint32_t *__restrict__ nz)
{
    const int wj = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (wj >= wpitch || i >= nx) return;
    uint32_t a = 0, z = 0;
    for (int b = 0; b < 32; b++) {
        const int j = wj * 32 + b;
        if (j >= ny) break;
        const int m = xy[(size_t)i * ny + j];
        const bool edge = (i == 0 || i == nx - 1 || j == 0 || j == ny - 1);
        if (edge ? (m != 0) : (m > 0)) a |= 1u << b;
        if (m != 0) z |= 1u << b;
    }
    act[(size_t)i * wpitch + wj] = a;
    nz[(size_t)i * wpitch + wj] = z;
}

// Dense FP64 [nx][ny] -> pitched T [nx][pitch] (padding zeroed).
template <class T>
__global__ void k_convert_in(int nx, int ny, int pitch, const double *__restrict__ src, T *__restrict__ dst)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= pitch || i >= nx) return;
    dst[(size_t)i * pitch + j] = (j < ny) ? (T)src[(size_t)i * ny + j] : (T)0;
}
// Dense [nx][ny] rows of the field precision into the pitched layout (padding zeroed).
template <class T>
__global__ void k_repack_in(int nx, int ny, int pitch, const T *__restrict__ src, T *__restrict__ dst)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= pitch || i >= nx) return;
    dst[(size_t)i * pitch + j] = (j < ny) ? src[(size_t)i * ny + j] : (T)0;
}
template <class T>
__global__ void k_convert_out(int nx, int ny, int pitch, const T *__restrict__ src, double *__restrict__ dst)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= ny || i >= nx) return;
    dst[(size_t)i * ny + j] = (double)src[(size_t)i * pitch + j];
}

// a - b of two floats rounded once to FP32, i.e. the FP32 subtraction.  The difference
// computed in FP64 and then rounded to FP32 is the same value (53 >= 2*24 + 2 bits, so the
// double rounding is innocuous for a sum of two floats), without the FP64 pipe.
__device__ __forceinline__ float dif32(float a, float b) { return __fsub_rn(a, b); }

// FP32 state from host (phi, psi) rows, dense [nx][ny] of H = double or float: phi
// rounded once, the velocity phi - psi computed exactly and rounded once (FP64 rows: in
// FP64; FP32 rows: dif32); padding zeroed.  The rows may be the caller's page-locked
// host memory, read in place.
template <class H>
__global__ void k_state_in32(int nx, int ny, int pitch, const H *__restrict__ phi, const H *__restrict__ psi,
                             float *__restrict__ x, float *__restrict__ v)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= pitch || i >= nx) return;
    const size_t o = (size_t)i * pitch + j, c = (size_t)i * ny + j;
    if constexpr (sizeof(H) == 4) {
        const float a = j < ny ? phi[c] : 0.f, b = j < ny ? psi[c] : 0.f;
        x[o] = a;
        v[o] = dif32(a, b);
    } else {
        const double a = j < ny ? phi[c] : 0.0, b = j < ny ? psi[c] : 0.0;
        x[o] = (float)a;
        v[o] = (float)S_(a, b);
    }
}
// The same for FP32 host rows four columns per thread (ny a multiple of 4, so every dense
// row starts on 16 bytes), padding zeroed.
__global__ void k_state_in32_v4(int nx, int ny, int pitch, const float4 *__restrict__ phi,
                                const float4 *__restrict__ psi, float *__restrict__ x, float *__restrict__ v)
{
    const int j = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int i = blockIdx.y;
    if (j >= pitch || i >= nx) return;
    const size_t o = (size_t)i * pitch + j;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (j < ny) {
        const size_t c = ((size_t)i * ny + j) / 4;
        a = phi[c];
        b = psi[c];
    }
    const float4 dv = make_float4(dif32(a.x, b.x), dif32(a.y, b.y), dif32(a.z, b.z), dif32(a.w, b.w));
    *reinterpret_cast<float4 *>(x + o) = a;
    *reinterpret_cast<float4 *>(v + o) = dv;
}

// FP32 state to host rows: phi, and psi = phi - v computed exactly and rounded once to H
// (FP64 rows: in FP64; FP32 rows: dif32); either may be NULL.  The rows may be the caller's
// page-locked host memory, written in place.
template <class H>
__global__ void k_state_out32(int nx, int ny, int pitch, const float *__restrict__ x, const float *__restrict__ v,
                              H *__restrict__ phi, H *__restrict__ psi)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= ny || i >= nx) return;
    const size_t o = (size_t)i * pitch + j, c = (size_t)i * ny + j;
    const float a = x[o];
    if (phi) phi[c] = (H)a;
    if constexpr (sizeof(H) == 4) {
        if (psi) psi[c] = dif32(a, v[o]);
    } else {
        if (psi) psi[c] = S_((double)a, (double)v[o]);
    }
}
// The same into FP32 host rows four columns per thread (ny a multiple of 4).
__global__ void k_state_out32_v4(int nx, int ny, int pitch, const float *__restrict__ x, const float *__restrict__ v,
                                 float4 *__restrict__ phi, float4 *__restrict__ psi)
{
    const int j = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int i = blockIdx.y;
    if (j >= ny || i >= nx) return;
    const size_t o = (size_t)i * pitch + j, c = ((size_t)i * ny + j) / 4;
    const float4 a = *reinterpret_cast<const float4 *>(x + o);
    if (phi) phi[c] = a;
    if (psi) {
        const float4 b = *reinterpret_cast<const float4 *>(v + o);
        psi[c] = make_float4(dif32(a.x, b.x), dif32(a.y, b.y), dif32(a.z, b.z), dif32(a.w, b.w));
    }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
void launch_step_exact(const DevParams &p, const double *phi, const double *psi, double *out, const int16_t *xy,
                       const double *tcc, const double *tc, const double *tg, long long time, int do_source,
                       cudaStream_t st)
{
    dim3 blk(64, 4), grd((p.ny + 63) / 64, (p.nx + 3) / 4);
    launch_pdl(k_step_exact, grd, blk, 0, st, p, phi, psi, out, xy, tcc, tc, tg, time, do_source);
}

void launch_step_exact_energy(const DevParams &p, const double *phi, const double *psi, double *out,
                              const int16_t *xy, long long time, cudaStream_t st)
{
    dim3 blk(64, 4), grd((p.ny / 2 + 63) / 64, (p.nx + 3) / 4);
    k_step_exact_energy<<<grd, blk, 0, st>>>(p, phi, psi, out, xy, time);
}

void launch_cell_energy(const DevParams &p, const double *phi, const double *psi, const int16_t *xy, int i, int j,
                        double *out, cudaStream_t st)
{
    k_cell_energy<<<1, 1, 0, st>>>(p, phi, psi, xy, i, j, out);
}

void launch_neumann_exact(const DevParams &p, const double *phi, double *out, const int16_t *xy,
                          const wg_neumann_bc *rec, int n, cudaStream_t st)
{
    if (n <= 0) return;
    k_neumann_exact<<<(n + 255) / 256, 256, 0, st>>>(p, phi, out, xy, rec, n);
}

template <class T>
void launch_point_source(const DevParams &p, T *out, T *vout, long long time, cudaStream_t st)
{
    k_point_source<T><<<1, 1, 0, st>>>(p, out, vout, time);
}
template void launch_point_source<float>(const DevParams &, float *, float *, long long, cudaStream_t);
template void launch_point_source<double>(const DevParams &, double *, double *, long long, cudaStream_t);

// FP64: the bulk update without the terms whose coefficient is zero on every cell
// (upd64's Z flags: KAPPA = 0; GAMMA = 0 as a uniform value); the values are unchanged.
template <class T, int COEF>
static void launch_bulk(const DevParams &p, const FastArgs<T> &a, dim3 grd, dim3 blk, cudaStream_t st)
{
    if constexpr (sizeof(T) == 8) {
        const bool g0 = (COEF == WG_COEF_TABLE) ? (!a.tg && p.gam == 0.0) : (p.gam == 0.0 && p.gamb == 0.0);
        switch ((p.kappa == 0.0 ? Z_KAPPA : 0) | (g0 ? Z_GAMMA : 0)) {
        case Z_KAPPA: launch_pdl(k_step_bulk<T, COEF, Z_KAPPA>, grd, blk, 0, st, p, a); return;
        case Z_GAMMA: launch_pdl(k_step_bulk<T, COEF, Z_GAMMA>, grd, blk, 0, st, p, a); return;
        case Z_KAPPA | Z_GAMMA: launch_pdl(k_step_bulk<T, COEF, Z_KAPPA | Z_GAMMA>, grd, blk, 0, st, p, a); return;
        default: break;
        }
    }
    launch_pdl(k_step_bulk<T, COEF>, grd, blk, 0, st, p, a);
}

template <class T>
void launch_step_fast(const DevParams &p, const FastArgs<T> &a, int coef_mode, long long time, cudaStream_t st)
{
    constexpr int V = Vec<T>::n;
    dim3 blk(64, 4), grd((p.pitch / V + 63) / 64, (p.nx - 2 + 3) / 4);
    const int nedge = 2 * p.nx + 2 * (p.ny - 2) + 1;
    if (coef_mode == WG_COEF_MASK) {
        launch_bulk<T, WG_COEF_MASK>(p, a, grd, blk, st);
        launch_pdl(k_step_edge<T, WG_COEF_MASK>, dim3((nedge + 255) / 256), dim3(256), 0, st, p, a, time);
    } else {
        launch_bulk<T, WG_COEF_TABLE>(p, a, grd, blk, st);
        launch_pdl(k_step_edge<T, WG_COEF_TABLE>, dim3((nedge + 255) / 256), dim3(256), 0, st, p, a, time);
    }
}
template void launch_step_fast<float>(const DevParams &, const FastArgs<float> &, int, long long, cudaStream_t);
template void launch_step_fast<double>(const DevParams &, const FastArgs<double> &, int, long long, cudaStream_t);

template <class T>
void launch_neumann_fast(const DevParams &p, const T *phi, T *out, T *vout, const int4 *idx, const double2 *w, int n,
                         cudaStream_t st)
{
    if (n <= 0) return;
    k_neumann_fast<T><<<(n + 255) / 256, 256, 0, st>>>(p, phi, out, vout, idx, w, n);
}
template void launch_neumann_fast<float>(const DevParams &, const float *, float *, float *, const int4 *, const double2 *, int, cudaStream_t);
template void launch_neumann_fast<double>(const DevParams &, const double *, double *, double *, const int4 *, const double2 *, int, cudaStream_t);

template <class T>
void launch_energy(const DevParams &p, const T *phi, const T *psi, const int16_t *xy, const uint32_t *nz,
                   double2 *bot, double2 *top, int ileft, int iright, double *out, cudaStream_t st)
{
    // bot: per-column sums; top (2 nx doubles): six box partials per block of 8 columns
    const int nblocks = (p.nx + ENERGY_COLS_PER_BLOCK - 1) / ENERGY_COLS_PER_BLOCK;
    double *part = reinterpret_cast<double *>(top);
    const dim3 g(nblocks), b(32 * ENERGY_COLS_PER_BLOCK);
    if (xy) launch_pdl(k_energy_cols<T, 0>, g, b, 0, st, p, phi, psi, xy, nz, ileft, iright, bot, part);
    else launch_pdl(k_energy_cols<T, 1>, g, b, 0, st, p, phi, psi, xy, nz, ileft, iright, bot, part);
    launch_pdl(k_energy_final, dim3(7), dim3(32), 0, st, p.nx, nblocks, (const double2 *)bot, (const double *)part, out);
}
template void launch_energy<float>(const DevParams &, const float *, const float *, const int16_t *, const uint32_t *, double2 *, double2 *, int, int, double *, cudaStream_t);
template void launch_energy<double>(const DevParams &, const double *, const double *, const int16_t *, const uint32_t *, double2 *, double2 *, int, int, double *, cudaStream_t);

template <class T>
void launch_count_nonfinite(int nx, int ny, int pitch, const T *a, unsigned long long *count, cudaStream_t st)
{
    k_count_nonfinite<T><<<4 * 152, 256, 0, st>>>(nx, ny, pitch, a, count);
}
template void launch_count_nonfinite<float>(int, int, int, const float *, unsigned long long *, cudaStream_t);
template void launch_count_nonfinite<double>(int, int, int, const double *, unsigned long long *, cudaStream_t);

void launch_pack_mask(int nx, int ny, int wpitch, const int16_t *xy, uint32_t *act, uint32_t *nz, cudaStream_t st)
{
    dim3 grd((wpitch + 127) / 128, nx);
    k_pack_mask<<<grd, 128, 0, st>>>(nx, ny, wpitch, xy, act, nz);
}

template <class T>
void launch_convert_in(int nx, int ny, int pitch, const double *src, T *dst, cudaStream_t st)
{
    dim3 grd((pitch + 255) / 256, nx);
    k_convert_in<T><<<grd, 256, 0, st>>>(nx, ny, pitch, src, dst);
}
template <class T>
void launch_convert_out(int nx, int ny, int pitch, const T *src, double *dst, cudaStream_t st)
{
    dim3 grd((ny + 255) / 256, nx);
    k_convert_out<T><<<grd, 256, 0, st>>>(nx, ny, pitch, src, dst);
}
template <class T>
void launch_repack_in(int nx, int ny, int pitch, const T *src, T *dst, cudaStream_t st)
{
    dim3 grd((pitch + 255) / 256, nx);
    k_repack_in<T><<<grd, 256, 0, st>>>(nx, ny, pitch, src, dst);
}
template void launch_repack_in<float>(int, int, int, const float *, float *, cudaStream_t);
template void launch_repack_in<double>(int, int, int, const double *, double *, cudaStream_t);
template void launch_convert_in<float>(int, int, int, const double *, float *, cudaStream_t);
template void launch_convert_in<double>(int, int, int, const double *, double *, cudaStream_t);
template void launch_convert_out<float>(int, int, int, const float *, double *, cudaStream_t);
template void launch_convert_out<double>(int, int, int, const double *, double *, cudaStream_t);

// dense FP32 rows of ny % 4 == 0 columns from 16-byte aligned bases take the 4-wide kernels
static bool rows_v4(int ny, const void *a, const void *b)
{
    return ny % 4 == 0 && ((uintptr_t)a & 15) == 0 && ((uintptr_t)b & 15) == 0;
}
template <class H>
void launch_state_in32(int nx, int ny, int pitch, const H *phi, const H *psi, float *x, float *v, cudaStream_t st)
{
    if (sizeof(H) == 4 && rows_v4(ny, phi, psi)) {
        dim3 grd((pitch / 4 + 255) / 256, nx);
        k_state_in32_v4<<<grd, 256, 0, st>>>(nx, ny, pitch, (const float4 *)phi, (const float4 *)psi, x, v);
        return;
    }
    dim3 grd((pitch + 255) / 256, nx);
    k_state_in32<H><<<grd, 256, 0, st>>>(nx, ny, pitch, phi, psi, x, v);
}
template <class H>
void launch_state_out32(int nx, int ny, int pitch, const float *x, const float *v, H *phi, H *psi, cudaStream_t st)
{
    if (sizeof(H) == 4 && rows_v4(ny, phi ? (const void *)phi : (const void *)psi, psi ? (const void *)psi : (const void *)phi)) {
        dim3 grd((ny / 4 + 255) / 256, nx);
        k_state_out32_v4<<<grd, 256, 0, st>>>(nx, ny, pitch, x, v, (float4 *)phi, (float4 *)psi);
        return;
    }
    dim3 grd((ny + 255) / 256, nx);
    k_state_out32<H><<<grd, 256, 0, st>>>(nx, ny, pitch, x, v, phi, psi);
}
template void launch_state_in32<float>(int, int, int, const float *, const float *, float *, float *, cudaStream_t);
template void launch_state_in32<double>(int, int, int, const double *, const double *, float *, float *, cudaStream_t);
template void launch_state_out32<float>(int, int, int, const float *, const float *, float *, float *, cudaStream_t);
template void launch_state_out32<double>(int, int, int, const float *, const float *, double *, double *, cudaStream_t);

}  // namespace wg
