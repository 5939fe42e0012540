// wg_tb.cu — temporal blocking of the FP32 leapfrog stepper, and its autotuner.
//
// k_step_tb<COEF>: one CTA owns an extended tile of L rows (i) x W columns (j, W =
// blockDim.x = 128 or 256; L = 16..64), i.e. a core of (L-2K) x (W-2K) cells plus a
// halo of K.  The tile's phi (two levels, alternating) and velocity sit in shared
// memory; K leapfrog updates run on the shrinking region [s, L-s) x [s, W-s) (the new
// phi goes to the other phi level, the velocity is updated in place at the cell itself,
// so a sub-step has no hazards), each thread marching down its column with the i+-1
// neighbours in a register window.  Then the core of phi and the velocity is stored.
// HBM traffic per K updates: one read of phi, the velocity (and the tcc table) over the
// extended tile and one write of both over the core.
//
// The per-cell rules are the reference's (wave_billiard.c:361-590) for the boundary
// conditions whose stencils stay inside the tile: the mirror "Dirichlet" box edges,
// absorbing edges, OSCILLATE_LEFT / OSCILLATE_TOPBOT, FLOOR and the point source.
// Periodic and VPER_HABS boundaries (which read the opposite side of the grid) and
// Neumann gathers use the single-step kernel.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include "wg_scene.h"
#include "wg_batch.h"
#include "wg_tma.cuh"

namespace wg {


constexpr int TB_AW = 12;  // mask words loaded per tile row (covers 256 + 3*32 columns)

struct TbArgs {
    const float *phi, *psi;   // phi(t) and the velocity phi(t) - phi(t-1)
    float *phi_out, *psi_out; // the same after the pass (distinct buffers)
    const uint32_t *act;      // active plane
    const float *tcc, *tc;    // tables (WG_COEF_TABLE)
    float c2, c2b, gam, gamb, kappa, ks, kt, gs, gt, vmax, courant, courantb;
    long long t0;             // step counter before the pass
    const float *osc;         // oscillating_bc values of the pass, [K][ny]
    const double *src;        // point-source increments of the pass, [K]
    int *err;                 // set to 1 when a bounded wait gives up
};

// FP32 phi and velocity of one boundary-line or point-source cell after update t, with
// the reference rules for non-wrapping boundaries (wave_billiard.c:393-590): the mirror
// "Dirichlet" edge and OSCILLATE_TOPBOT rows are the bulk update with the missing
// neighbours replaced by the cell itself, absorbing edges use their inward neighbour,
// oscillating cells take the precomputed oscillating_bc value; keep32 where the
// reference writes nothing.
template <int COEF>
__device__ __forceinline__ XV tb_general(const DevParams &p, const TbArgs &a, int gi, int gj, int s, float x,
                                         float v, float nip, float nim, float njp, float njm, float cc, int act)
{
    const float ccv = (COEF == WG_COEF_TABLE) ? cc : (act ? a.c2 : a.c2b);
    const float g = (COEF == WG_COEF_TABLE) ? a.gam : (act ? a.gam : a.gamb);
    const float tcv = (COEF == WG_COEF_TABLE) ? (a.tc ? a.tc[(size_t)gi * p.pitch + gj] : 0.f)
                                              : (act ? a.courant : a.courantb);
    const Edge32K k{a.kappa, a.ks, a.kt, a.gs, a.gt, a.vmax};
    XV r = edge32<true>(p, gi, gj, x, v, nip, nim, njp, njm, ccv, tcv, g, act != 0, k,
                        [&] { return a.osc[(size_t)(s - 1) * p.ny + gj]; });
    if (p.src_on && gi == p.src_i && gj == p.src_j) r = source32(r, a.src[s - 1]);
    return r;
}

// One sub-step down this thread's column for a tile with no boundary-line or source
// cell: rows [r0, r1), the i+-1 neighbours in a register window, shared-memory
// addressing by constant offsets.  P: phi of the previous level; Q: phi of the new
// level; Vs: the velocity, in place.  ACT: the cell's mask bit selects coefficients and
// whether it is written (otherwise every cell is written with its tcc).
template <int COEF, bool ACT>
__device__ __forceinline__ void tb_rows_interior(const DevParams &p, const TbArgs &a, const float *__restrict__ P,
                                                 float *__restrict__ Q, float *__restrict__ Vs,
                                                 const float *__restrict__ Cs, int Bw, int c, int r0, int r1,
                                                 uint64_t actb)
{
    int idx = r0 * Bw + c;
    float up = P[idx - Bw], mid = P[idx];
    uint64_t am = actb >> r0;
    const int n = r1 - r0;
#pragma unroll 4
    for (int q = 0; q < n; q++, idx += Bw) {
        const float dn = P[idx + Bw], e = P[idx + 1], w = P[idx - 1], y = Vs[idx];
        const float delta = ((dn - mid) + (up - mid)) + ((e - mid) + (w - mid));
        XV r;
        if (!ACT) {
            r = upd32(mid, y, Cs[idx], delta, a.kappa, a.gam);
        } else {
            const bool act = am & 1u;
            am >>= 1;
            const float ccv = (COEF == WG_COEF_TABLE) ? Cs[idx] : (act ? a.c2 : a.c2b);
            const float g = (COEF == WG_COEF_TABLE) ? a.gam : (act ? a.gam : a.gamb);
            r = keep32(mid, y);
            if (p.twospeeds || act) {
                r = upd32(mid, y, ccv, delta, a.kappa, g);
                if (p.floor_clamp && act) r = clamp32(mid, r, a.vmax);
            }
        }
        Q[idx] = r.x;
        Vs[idx] = r.v;
        up = mid;
        mid = dn;
    }
}

// oscillating_bc(t0 + s, j) for s = 1..n (when OSCILLATE_LEFT) and the point-source
// increment of update t0 + s, rounded to FP32, for the passes of one step() call.
__global__ void k_boundary_values(const __grid_constant__ DevParams p, long long t0, int n, float *osc, double *src)
{
    pdl_wait();  // launched by launch_pdl: the previous pass, which read these arrays, has completed
    pdl_trigger();
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (p.osc_left && idx < n * p.ny) {
        const int s = idx / p.ny, j = idx % p.ny;
        osc[idx] = (float)osc_bc(p, (int)(t0 + s + 1), j);
    }
    if (p.src_on && idx < n) src[idx] = point_source(p, t0 + idx + 1);
}

// Shared-memory layout of one tile: F0, F1 (phi, alternating levels), Vs (velocity),
// Cs (tcc, table mode), Aw (the active-plane words covering the tile), one mbarrier.
// F0, Vs, Cs and Aw are loaded; F1 is written before it is read.
struct TbLayout {
    int f0, f1, vs, cs, aw, bar, bytes, tma_bytes;
};
__host__ __device__ inline TbLayout tb_layout(int coef, int L, int Bw)
{
    TbLayout t;
    const int fb = L * Bw * 4;
    t.f0 = 0;
    t.f1 = fb;
    t.vs = 2 * fb;
    t.cs = 3 * fb;
    t.aw = (coef == WG_COEF_TABLE ? 4 : 3) * fb;
    t.bar = t.aw + ((L * TB_AW * 4 + 15) / 16) * 16;
    t.bytes = t.bar + 16;
    t.tma_bytes = (coef == WG_COEF_TABLE ? 3 : 2) * fb + L * TB_AW * 4;
    return t;
}

template <int COEF>
__global__ void __launch_bounds__(256) k_step_tb(const __grid_constant__ DevParams p, const __grid_constant__ TbArgs a,
                                                 const __grid_constant__ CUtensorMap m_phi,
                                                 const __grid_constant__ CUtensorMap m_psi,
                                                 const __grid_constant__ CUtensorMap m_tcc,
                                                 const __grid_constant__ CUtensorMap m_act, int K, int Kh, int L)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const int Bw = blockDim.x;
    const TbLayout lay = tb_layout(COEF, L, Bw);
    float *F0 = (float *)(smem + lay.f0), *F1 = (float *)(smem + lay.f1), *Vs = (float *)(smem + lay.vs),
          *Cs = (float *)(smem + lay.cs);
    const uint32_t *Aw = (const uint32_t *)(smem + lay.aw);
    uint64_t *bar = (uint64_t *)(smem + lay.bar);
    const int c = threadIdx.x;
    const int core_w = Bw - 2 * Kh, core_h = L - 2 * K;
    const int x0 = blockIdx.x * core_w - Kh;   // first column of the tile (a multiple of 4)
    const int gi0 = blockIdx.y * core_h - K;   // first row of the tile
    const int w0 = (x0 >> 5) & ~3;             // first mask word of the tile (a multiple of 4)
    const int gj = x0 + c;
    const bool col_ok = gj >= 0 && gj < p.ny;
    const bool col_special = (gj == 0 || gj == p.ny - 1);

    // TMA destinations must be 128-byte aligned; refuse (flag) rather than issue otherwise
    if (smem_u32(smem) & 127u) {
        if (c == 0) atomicExch(a.err, 2);
        return;
    }
    // TMA: the extended tile of phi, the velocity (tcc) and the mask words, zero outside the grid
    if (c == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (c == 0) {
        mbar_arrive_expect_tx(bar, (unsigned)lay.tma_bytes);
        tma_load_2d(F0, &m_phi, x0, gi0, bar);
        tma_load_2d(Vs, &m_psi, x0, gi0, bar);
        if (COEF == WG_COEF_TABLE) tma_load_2d(Cs, &m_tcc, x0, gi0, bar);
        tma_load_2d((void *)Aw, &m_act, w0, gi0, bar);
    }
    const bool ok = mbar_wait_bounded(bar, 0, 1u << 24);
    if (__syncthreads_or(!ok)) {
        // the copies did not land in time: flag it, let them drain (bounded), leave
        if (c == 0) atomicExch(a.err, 1);
        mbar_wait_bounded(bar, 0, 1u << 24);
        return;
    }

    uint64_t actb = 0;
    if (col_ok) {
        const int wi = (gj >> 5) - w0;
#pragma unroll 8
        for (int r = 0; r < L; r++) actb |= (uint64_t)((Aw[r * TB_AW + wi] >> (gj & 31)) & 1u) << r;
    }

    // a tile with no boundary line and no source cell runs the lean interior loop
    const bool interior_tile = gi0 >= 1 && gi0 + L <= p.nx - 1 && x0 >= 1 && x0 + Bw <= p.ny - 1 &&
                               !(p.src_on && p.src_i >= gi0 && p.src_i < gi0 + L && p.src_j >= x0 && p.src_j < x0 + Bw);
    const bool no_act = COEF == WG_COEF_TABLE && p.twospeeds && !p.floor_clamp;

    for (int s = 1; s <= K; s++) {
        const float *P = (s & 1) ? F0 : F1;  // phi of level t+s-1
        float *Q = (s & 1) ? F1 : F0;        // phi of level t+s-2, becomes level t+s
        const bool in_region = c >= Kh - K + s && c < Bw - Kh + K - s;
        if (interior_tile) {
            if (in_region) {
                if (no_act) tb_rows_interior<COEF, false>(p, a, P, Q, Vs, Cs, Bw, c, s, L - s, actb);
                else tb_rows_interior<COEF, true>(p, a, P, Q, Vs, Cs, Bw, c, s, L - s, actb);
            }
        } else if (col_ok && in_region && !col_special) {
            // a boundary tile, interior column: lean segments between the special rows
            // (gi = 0, gi = nx-1, the source row), the special rows one at a time
            const int lo = max(s, -gi0), hi = min(L - s, p.nx - gi0);
            const int ra = -gi0, rb = p.nx - 1 - gi0;
            const int rs = (p.src_on && gj == p.src_j) ? p.src_i - gi0 : -1;
            int r = lo;
            while (r < hi) {
                if (r == ra || r == rb || r == rs) {
                    const int gi = gi0 + r, o = r * Bw + c;
                    const float cc = (COEF == WG_COEF_TABLE) ? Cs[o] : 0.f;
                    const XV res = tb_general<COEF>(p, a, gi, gj, s, P[o], Vs[o], P[o + Bw], P[o - Bw], P[o + 1],
                                                    P[o - 1], cc, (int)((actb >> r) & 1u));
                    Q[o] = res.x;
                    Vs[o] = res.v;
                    r++;
                } else {
                    int nxt = hi;
                    if (ra > r && ra < nxt) nxt = ra;
                    if (rb > r && rb < nxt) nxt = rb;
                    if (rs > r && rs < nxt) nxt = rs;
                    if (no_act) tb_rows_interior<COEF, false>(p, a, P, Q, Vs, Cs, Bw, c, r, nxt, actb);
                    else tb_rows_interior<COEF, true>(p, a, P, Q, Vs, Cs, Bw, c, r, nxt, actb);
                    r = nxt;
                }
            }
        } else if (col_ok && in_region) {
            int r = s;
            float up = P[(r - 1) * Bw + c], mid = P[r * Bw + c];
#pragma unroll 4
            for (; r < L - s; r++) {
                const float dn = P[(r + 1) * Bw + c];
                const int gi = gi0 + r;
                if (gi >= 0 && gi < p.nx) {
                    const int o = r * Bw + c;
                    const float e = P[o + 1], w = P[o - 1];
                    const float y = Vs[o];
                    const float cc = (COEF == WG_COEF_TABLE) ? Cs[o] : 0.f;
                    const int act = (int)((actb >> r) & 1u);
                    XV res = keep32(mid, y);
                    if (col_special || gi == 0 || gi == p.nx - 1 || (p.src_on && gi == p.src_i && gj == p.src_j)) {
                        res = tb_general<COEF>(p, a, gi, gj, s, mid, y, dn, up, e, w, cc, act);
                    } else if (p.twospeeds || act) {
                        const float ccv = (COEF == WG_COEF_TABLE) ? cc : (act ? a.c2 : a.c2b);
                        const float g = (COEF == WG_COEF_TABLE) ? a.gam : (act ? a.gam : a.gamb);
                        res = upd32(mid, y, ccv, ((dn - mid) + (up - mid)) + ((e - mid) + (w - mid)), a.kappa, g);
                        if (p.floor_clamp && act) res = clamp32(mid, res, a.vmax);
                    }
                    Q[o] = res.x;
                    Vs[o] = res.v;
                }
                up = mid;
                mid = dn;
            }
        }
        __syncthreads();
    }

    // store the core: phi of level t+K and the velocity
    if (col_ok && c >= Kh && c < Bw - Kh) {
        const float *newest = (K & 1) ? F1 : F0;
#pragma unroll 4
        for (int r = K; r < L - K; r++) {
            const int gi = gi0 + r;
            if (gi < p.nx) {
                const size_t o = (size_t)gi * p.pitch + gj;
                a.phi_out[o] = newest[r * Bw + c];
                a.psi_out[o] = Vs[r * Bw + c];
            }
        }
    }
}

// One FP32 cell of level s at (gi, gj) from level s-1 (phi x, its neighbours n = i+1,
// sv = i-1, e = j+1, w = j-1, and the velocity y).  cc is the cell's tcc, tcv its tc
// (table mode).  GEN = false: a cell off the boundary lines and the source; PLAIN
// additionally promises twospeeds and no FLOOR clamp, so every such cell takes the
// leapfrog update.  INL: oscillating values and source increments are computed here
// (batches) instead of read from the per-call arrays; both are the same double values,
// rounded the same way.
// Out of line: they are rare, and inlined copies per level would crowd the instruction cache.
__device__ __noinline__ float osc_inl(const DevParams &p, long long t, int j) { return (float)osc_bc(p, (int)t, j); }
__device__ __noinline__ double src_inl(const DevParams &p, long long t) { return point_source(p, t); }

template <int COEF, bool GEN, bool PLAIN, bool INL = false, bool KZ = false>
__device__ __forceinline__ XV skew_cell(const DevParams &p, const TbArgs &a, int gi, int gj, int s, float x, float y,
                                        float n, float sv, float e, float w, float cc, float tcv, bool act)
{
    const float ccv = (COEF == WG_COEF_TABLE) ? cc : (act ? a.c2 : a.c2b);
    const float g = (COEF == WG_COEF_TABLE) ? a.gam : (act ? a.gam : a.gamb);
    if (!GEN && PLAIN && KZ) return upd32_k0(x, y, ccv, ((n - x) + (sv - x)) + ((e - x) + (w - x)), g);
    if (!GEN && PLAIN) return upd32(x, y, ccv, ((n - x) + (sv - x)) + ((e - x) + (w - x)), a.kappa, g);
    if (!GEN) {
        XV r = keep32(x, y);
        if (p.twospeeds || act) {
            r = upd32(x, y, ccv, ((n - x) + (sv - x)) + ((e - x) + (w - x)), a.kappa, g);
            if (p.floor_clamp && act) r = clamp32(x, r, a.vmax);
        }
        return r;
    }
    const float tce = (COEF == WG_COEF_TABLE) ? tcv : (act ? a.courant : a.courantb);
    const Edge32K k{a.kappa, a.ks, a.kt, a.gs, a.gt, a.vmax};
    XV r = edge32<true>(p, gi, gj, x, y, n, sv, e, w, ccv, tce, g, act, k, [&] {
        return INL ? osc_inl(p, a.t0 + s, gj) : a.osc[(size_t)(s - 1) * p.ny + gj];
    });
    if (p.src_on && gi == p.src_i && gj == p.src_j) r = source32(r, INL ? src_inl(p, a.t0 + s) : a.src[s - 1]);
    return r;
}


// Paired FP32 arithmetic: the two-wide add, sub and fma of this GPU (.f32x2) round each
// element exactly as the scalar instruction does, so two cells computed together get the
// same bits as two computed one at a time, for one instruction issued instead of two.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
// element c (0..3) of a lane's four cells held as the pairs (0, 1) and (2, 3)
__device__ __forceinline__ float el(const float2 (&q)[2], int c)
{
    return (c & 2) ? ((c & 1) ? q[1].y : q[1].x) : ((c & 1) ? q[0].y : q[0].x);
}

// skew_cell's inner rule (GEN = false) for the two cells of a pair, with the Laplacian
// given in differences.  Vertical: vert = dn - dp with dn = n - x and dp = x - sv, which
// equals (n - x) + (sv - x) exactly (round to nearest is symmetric, so sv - x == -(x - sv));
// dp is the previous row's dn, so each row's difference is formed once per column.
// Horizontal: hh = he - hw with he = e - x and hw = x - w, (e - x) + (w - x) == he - hw
// exactly, and a lane's four cells share the five differences of their row.  x, y, vert,
// cc: the cells' phi, velocity, vertical part and tcc.  New phi in xo, new velocity in vo:
// upd32_k0 (PLAIN, KZ), upd32 (PLAIN) or updkeep32 and clamp32, element by element.
template <int COEF, bool PLAIN, bool KZ = false>
__device__ __forceinline__ void skew_inner2(const DevParams &p, const TbArgs &a, float2 x, float2 y, float2 vert,
                                            float2 hh, float2 cc, bool act0, bool act1, float2 &xo, float2 &vo)
{
    const float2 ccv = (COEF == WG_COEF_TABLE) ? cc : make_float2(act0 ? a.c2 : a.c2b, act1 ? a.c2 : a.c2b);
    const float2 ng = (COEF == WG_COEF_TABLE) ? make_float2(-a.gam, -a.gam)
                                              : make_float2(act0 ? -a.gam : -a.gamb, act1 ? -a.gam : -a.gamb);
    const float2 lap = add2(vert, hh);
    float2 vn;
    if (PLAIN && KZ) {
        vn = fma2(ccv, lap, fma2(ng, y, y));                                    // upd32_k0
    } else {
        vn = fma2(ccv, lap, fma2(make_float2(-a.kappa, -a.kappa), x, fma2(ng, y, y)));  // vel32
        if (!PLAIN) {                                                           // updkeep32
            if (!(p.twospeeds || act0)) vn.x = -y.x;
            if (!(p.twospeeds || act1)) vn.y = -y.y;
        }
    }
    xo = add2(x, vn);
    vo = vn;
    if (!PLAIN && p.floor_clamp) {
        if (act0) {
            const XV r = clamp32(x.x, XV{xo.x, vo.x}, a.vmax);
            xo.x = r.x;
            vo.x = r.v;
        }
        if (act1) {
            const XV r = clamp32(x.y, XV{xo.y, vo.y}, a.vmax);
            xo.y = r.x;
            vo.y = r.v;
        }
    }
}

// ---------------------------------------------------------------------------
// Time-skewed streaming (k_step_skew): every warp owns a tile of 128 columns (four
// adjacent columns j per lane, loaded as float4; a column halo of H = K rounded up to 4
// on each side) and a strip of S rows (i), and marches down the strip once.  At input
// row m it computes level s at row m - s for s = 1..K (level 0 = phi(t) and its
// velocity), so each level keeps only a window of three phi rows and one velocity row in
// registers (plus the new velocity row of the level just computed, held until the next
// level has read the row it replaces).  Column neighbours inside a lane are registers;
// across lanes they are one warp shuffle each way.  Input rows are prefetched QD rows
// ahead through a per-warp shared-memory ring; table scenes also keep the tcc values of
// the last K+1 rows in a second small ring.  One row per loop trip (SKEW_UNROLL): longer
// trips turn the window rotation into register renaming but miss the instruction cache.
// Core columns [H, 128-H) store phi and the velocity of level K for the rows in the strip.
//
// Tiles that reach an edge row or column or hold the point source (edge tiles) take three
// extra steps after the common update: the lane holding column 0 or ny-1 redoes that
// cell by the column rule; rows 0 and nx-1 (warp-uniform) are redone by the general
// rule; the source cell gets its increment.  Cells outside the domain keep whatever
// they got: no cell inside reads them and none is stored.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float pick4(float a0, float a1, float a2, float a3, int c)
{
    return c == 0 ? a0 : (c == 1 ? a1 : (c == 2 ? a2 : a3));
}

// Column 0 (right = false) or ny-1 (right = true) at a row 1..nx-2: the boundary rule of
// evolve_wave_half for the top/bottom lines (wave_billiard.c:366-452, B_COND Dirichlet or
// absorbing, OSCILLATE_TOPBOT), same branches as skew_cell's general form.  vert: the
// vertical part of the Laplacian, (n - x) + (sv - x), as skew_inner2 takes it.
template <int COEF>
__device__ __forceinline__ XV col_edge_cell(const DevParams &p, const TbArgs &a, int gi, float x, float y, float vert,
                                            float e, float w, float cc, float tcv, bool act, bool right)
{
    const float ccv = (COEF == WG_COEF_TABLE) ? cc : (act ? a.c2 : a.c2b);
    const float g = (COEF == WG_COEF_TABLE) ? a.gam : (act ? a.gam : a.gamb);
    int mode = 0;
    if (p.osc_topbot && gi < p.tb_ilim) {
        e = x;
        w = x;
    } else if (p.b_cond == WG_BC_DIRICHLET) {
        if (right) e = x; else w = x;
    } else {
        mode = 1;
    }
    XV r = keep32(x, y);
    if (p.twospeeds || act) {
        if (mode == 0)
            r = upd32(x, y, ccv, vert + ((e - x) + (w - x)), a.kappa, g);
        else
            r = absorb32(x, y, (COEF == WG_COEF_TABLE) ? tcv : (act ? a.courant : a.courantb), right ? w : e, a.kt, a.gt);
        if (p.floor_clamp && act) r = clamp32(x, r, a.vmax);
    }
    return r;
}

// Asynchronous global->shared copies of one lane's 16 (or 4) bytes to a 32-bit shared-window
// address; with src_bytes 0 nothing is read and the destination is zero-filled.
__device__ __forceinline__ void cp_async16s(unsigned d, const void *src, int src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async4s(unsigned d, const void *src, int src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Row slot of a warp's shared-memory ring (floats): phi[128], psi[128], tcc[128] (table
// scenes), then one active word and one edge-column tc per lane.
#ifndef SKEW_UNROLL
#define SKEW_UNROLL 1  // rows per loop trip (2 and 3 measured slower)
#endif
template <int COEF> struct SkewSlot {
    static constexpr int PSI = 128, TCC = 256, ACT = (COEF == WG_COEF_TABLE) ? 384 : 256, TCE = ACT + 32, SIZE = TCE + 32;
    // ring slots: 4 for table scenes (measured against 3, 5 and 6 on 3840x2160: +1% at K = 5,
    // +4% at K = 4 over 6), 8 for the batches' mask form (4 and 6 measured slower)
    static constexpr int DEPTH = (COEF == WG_COEF_TABLE) ? 4 : 8;
};

// GEN = false: inner tiles (fix = false) and tiles of column 0, of column ny-1 when ny is
// a multiple of 4, or of the point source (fix = true), all away from rows 0 and nx-1.
// GEN = true (fix = true): the others, with the general rule on rows 0 and nx-1.
// Columns [lo, hi) of the tile are stored (lo, hi multiples of 4 but for hi = ny).
// wrap: a periodic scene in the ghost layout (batches): rows -BATCH_GHOST_ROWS..nx +
// BATCH_GHOST_ROWS - 1 and columns -BATCH_GHOST_COLS..ny + BATCH_GHOST_COLS - 1 hold the
// wrapped field, so every cell takes the bulk rule and no edge rule applies.
// KZ (with PLAIN): KAPPA = 0, the bulk update without its kappa term.
// (a runtime flag, so that periodic and other inner tiles share one loop in the
// instruction cache).
template <int COEF, int K, bool PLAIN, bool GEN, bool INL = false, bool KZ = false>
__device__ __forceinline__ void skew_strip(const DevParams &p, const TbArgs &a, int i_s, int i_e, int gj0, int lane,
                                           float *ring, float *tring, bool edge, int lo, int hi, bool wrap = false)
{
    using SL = SkewSlot<COEF>;
    constexpr int D = SL::DEPTH;
    constexpr int QD = D - 1;                    // rows in flight ahead of the one in use
    constexpr bool NEED_ACT = !(PLAIN && COEF == WG_COEF_TABLE);  // the plain table update ignores the mask
    const bool need_tce = edge && COEF == WG_COEF_TABLE;           // tc of this lane's boundary column
    const int m0 = i_s - K - 1, m1 = i_e + K;                      // input rows [m0, m1)
    const bool lane_core = gj0 >= lo && gj0 < hi;
    const bool grp_ok = gj0 >= 0 && gj0 < p.ny;  // the group holds at least one domain column
    // edge tiles: the lane's boundary column (0..3), or -1; the domain has ny >= 8 columns
    const int cr = p.ny - 1 - gj0;  // column ny-1 within the lane's group when 0..3
    const int ce = !edge ? -1 : (gj0 == 0 ? 0 : (cr >= 0 && cr <= 3 ? cr : -1));
    const bool src_lane = edge && p.src_on && p.src_j >= gj0 && p.src_j < gj0 + 4;

    // The lane's four cells are held as two pairs, (gj0, gj0+1) and (gj0+2, gj0+3), for
    // the paired instructions; el(q, c) reads cell c.
    float2 W[K + 1][3][2];  // W[s][k] = phi of level s at row m-s-2+k (k = 0: GEN only)
    // Dp[s] = phi_s(m-s-1) - phi_s(m-s-2): the vertical difference level s+1 formed in the
    // previous trip, its dp in this one (not GEN)
    float2 Dp[K][2];
    // V[s] = velocity of level s at row m-s-1, until level s+1 of the trip for row m has
    // read it; pend = the new velocity row of the level just computed.  (Kept in a per-warp
    // shared-memory row per level instead, the single-grid pass ran as fast at its best
    // depth and the batch passes 8% slower.)
    float2 V[K][2], pend[2];
    // tcc at rows m, m-1, ..., m-K (table scenes): the warp's shared ring tring of K+1 rows
    // (slot ts holds row m), each lane writing and reading back only its own 16 bytes
    int ts = 0;
    float TE[K + 1];       // tc of the lane's boundary column at the same rows (edge tiles, table)
    uint32_t aq = 0;       // bits 4d..4d+3 = active bits of row m-d
#pragma unroll
    for (int q = 0; q <= K; q++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            W[q][0][h] = W[q][1][h] = W[q][2][h] = make_float2(0.f, 0.f);
            if (q < K) V[q][h] = Dp[q][h] = make_float2(0.f, 0.f);
        }
        TE[q] = 0.f;
    }

    // row m goes to slot (m - m0) % D; each lane copies, and later reads, only its own bytes
    // shared-memory addresses of this lane's bytes in slot 0 (a slot is SL::SIZE floats)
    const unsigned s16 = (unsigned)__cvta_generic_to_shared(ring) + 16u * lane;
    const unsigned s4 = (unsigned)__cvta_generic_to_shared(ring) + 4u * lane;
    auto issue = [&](int m, int slot) {
        const unsigned so = (unsigned)(slot * SL::SIZE * 4);
        const bool ok = wrap ? (gj0 >= -BATCH_GHOST_COLS && gj0 < p.ny + BATCH_GHOST_COLS && m >= -BATCH_GHOST_ROWS &&
                                m < p.nx + BATCH_GHOST_ROWS)
                             : (grp_ok && (unsigned)m < (unsigned)p.nx);
        const long long o = ok ? (long long)m * p.pitch + gj0 : 0;
        const int n16 = ok ? 16 : 0;
        cp_async16s(s16 + so, a.phi + o, n16);
        cp_async16s(s16 + so + 4 * SL::PSI, a.psi + o, n16);
        if (COEF == WG_COEF_TABLE) cp_async16s(s16 + so + 4 * SL::TCC, a.tcc + o, n16);
        // mask word of the group: floor division, so that the ghost columns left of column 0
        // read the row's ghost word (index -1)
        if (NEED_ACT)
            cp_async4s(s4 + so + 4 * SL::ACT, a.act + (ok ? (long long)m * p.wpitch + ((gj0 + 32) / 32 - 1) : 0),
                       ok ? 4 : 0);
        if (need_tce) {
            const bool te = ok && ce >= 0 && a.tc;  // the table exists with an absorbing boundary
            cp_async4s(s4 + so + 4 * SL::TCE, te ? a.tc + o + (unsigned)ce : a.phi, te ? 4 : 0);
        }
        cp_async_commit();
    };
#pragma unroll
    for (int q = 0; q < QD; q++) issue(m0 + q, q);
    int slot = 0;  // slot of row m

    for (int mb = m0; mb < m1; mb += SKEW_UNROLL) {
#pragma unroll
        for (int u = 0; u < SKEW_UNROLL; u++) {
            const int m = mb + u;
            if (m >= m1) break;  // warp-uniform
            cp_async_wait<QD - 1>();  // row m has landed
            const float *b = ring + slot * SL::SIZE;
            const float4 xq = *reinterpret_cast<const float4 *>(b + 4 * lane);
            const float4 yq = *reinterpret_cast<const float4 *>(b + SL::PSI + 4 * lane);
            const float4 cq = (COEF == WG_COEF_TABLE) ? *reinterpret_cast<const float4 *>(b + SL::TCC + 4 * lane)
                                                      : make_float4(0.f, 0.f, 0.f, 0.f);
            const uint32_t aw = NEED_ACT ? reinterpret_cast<const uint32_t *>(b)[SL::ACT + lane] : 0u;
            const float tein = need_tce ? b[SL::TCE + lane] : 0.f;
            const float2 xin[2] = {make_float2(xq.x, xq.y), make_float2(xq.z, xq.w)};
            const float2 yin[2] = {make_float2(yq.x, yq.y), make_float2(yq.z, yq.w)};
            if (COEF == WG_COEF_TABLE) *reinterpret_cast<float4 *>(tring + ts * 128 + 4 * lane) = cq;
            if (NEED_ACT) aq = (aq << 4) | ((aw >> (gj0 & 31)) & 0xFu);
            // the slot of row m-1 (read in the previous row) takes row m+QD
            issue(m + QD, slot == 0 ? D - 1 : slot - 1);
            slot = (slot == D - 1) ? 0 : slot + 1;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (GEN) W[0][0][h] = W[0][1][h];
                W[0][1][h] = W[0][2][h];
                W[0][2][h] = xin[h];
                pend[h] = yin[h];
            }
            if (need_tce) {  // warp-uniform: only tiles that hold a boundary column read TE
#pragma unroll
                for (int q = K; q > 0; q--) TE[q] = TE[q - 1];
                TE[0] = tein;
            }
#pragma unroll
            for (int lv = 1; lv <= K; lv++) {
                const int r = m - lv;  // row of this level's new value
                XV v[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
                // vertical part of the Laplacian of level lv-1 at row r: from the kept
                // difference (formed in every trip, so that the first active trip of the
                // level finds its dp), or from the three rows in GEN strips, which keep them
                // for the general rule
                float2 vt2[2];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    if (GEN) {
                        vt2[h] = add2(sub2(W[lv - 1][2][h], W[lv - 1][1][h]), sub2(W[lv - 1][0][h], W[lv - 1][1][h]));
                    } else {
                        const float2 dn = sub2(W[lv - 1][2][h], W[lv - 1][1][h]);
                        vt2[h] = sub2(dn, Dp[lv - 1][h]);
                        Dp[lv - 1][h] = dn;
                    }
                }
                // Level lv at row r reaches the stored rows only from r >= i_s - K + lv on, i.e.
                // from input row m0 + 2 lv + 1: in the pipeline fill the earlier levels are skipped
                // (warp-uniform), and their window slots hold zeros that nothing reads.
                if (m - m0 >= 2 * lv + 1) {
                // per-cell views of the pairs, for the horizontal differences and the edge rules
                const float Wc[4] = {W[lv - 1][1][0].x, W[lv - 1][1][0].y, W[lv - 1][1][1].x, W[lv - 1][1][1].y};
                const float Yl[4] = {V[lv - 1][0].x, V[lv - 1][0].y, V[lv - 1][1].x, V[lv - 1][1].y};  // row r
                const float vt[4] = {vt2[0].x, vt2[0].y, vt2[1].x, vt2[1].y};
                float2 Tl2[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};  // tcc at row r
                if (COEF == WG_COEF_TABLE) {
                    const int tsl = ts >= lv ? ts - lv : ts - lv + K + 1;
                    const float4 tq = *reinterpret_cast<const float4 *>(tring + tsl * 128 + 4 * lane);
                    Tl2[0] = make_float2(tq.x, tq.y);
                    Tl2[1] = make_float2(tq.z, tq.w);
                }
                const float Tl[4] = {Tl2[0].x, Tl2[0].y, Tl2[1].x, Tl2[1].y};
                const float e3 = __shfl_down_sync(0xffffffffu, Wc[0], 1);
                const float w0 = __shfl_up_sync(0xffffffffu, Wc[3], 1);
                // hd[c] = x(gj0+c) - x(gj0+c-1): cell c's e - x is hd[c+1], its x - w is hd[c];
                // the horizontal part of cell c is hd[c+1] - hd[c]
                const float hd[5] = {Wc[0] - w0, Wc[1] - Wc[0], Wc[2] - Wc[1], Wc[3] - Wc[2], e3 - Wc[3]};
                const float2 hh[2] = {make_float2(hd[1] - hd[0], hd[2] - hd[1]), make_float2(hd[3] - hd[2], hd[4] - hd[3])};
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const bool a0 = NEED_ACT ? ((aq >> (4 * lv + 2 * h)) & 1u) : true;
                    const bool a1 = NEED_ACT ? ((aq >> (4 * lv + 2 * h + 1)) & 1u) : true;
                    float2 xo, vo;
                    skew_inner2<COEF, PLAIN, KZ>(p, a, W[lv - 1][1][h], V[lv - 1][h], vt2[h], hh[h], Tl2[h], a0, a1, xo, vo);
                    v[2 * h] = XV{xo.x, vo.x};
                    v[2 * h + 1] = XV{xo.y, vo.y};
                }
                if (!GEN && edge) {  // warp-uniform
                    if (ce >= 0 && r > 0 && r < p.nx - 1) {  // the lane holding column 0 (c = 0) or ny-1 (c = 3)
                        const bool lf = ce == 0;
                        const XV res = col_edge_cell<COEF>(
                            p, a, r, lf ? Wc[0] : Wc[3], lf ? Yl[0] : Yl[3], lf ? vt[0] : vt[3], lf ? Wc[1] : e3,
                            lf ? w0 : Wc[2],
                            lf ? Tl[0] : Tl[3], TE[lv], NEED_ACT ? ((aq >> (4 * lv + ce)) & 1u) : true, !lf);
                        v[0] = lf ? res : v[0];
                        v[3] = lf ? v[3] : res;
                    }
                    if (src_lane && r == p.src_i) {
                        const double add = INL ? src_inl(p, a.t0 + lv) : a.src[lv - 1];
                        const int cs = p.src_j - gj0;
#pragma unroll
                        for (int c = 0; c < 4; c++) v[c] = (cs == c) ? source32(v[c], add) : v[c];
                    }
                }
                if (GEN) {
                    const bool row_edge = r == 0 || r == p.nx - 1;  // warp-uniform
                    if (ce >= 0 && r > 0 && r < p.nx - 1) {  // the lane holding column 0 or ny-1: picked by index
                        const XV res = col_edge_cell<COEF>(
                            p, a, r, pick4(Wc[0], Wc[1], Wc[2], Wc[3], ce), pick4(Yl[0], Yl[1], Yl[2], Yl[3], ce),
                            pick4(vt[0], vt[1], vt[2], vt[3], ce),
                            pick4(Wc[1], Wc[2], Wc[3], e3, ce), pick4(w0, Wc[0], Wc[1], Wc[2], ce),
                            pick4(Tl[0], Tl[1], Tl[2], Tl[3], ce), TE[lv],
                            NEED_ACT ? ((aq >> (4 * lv + ce)) & 1u) : true, gj0 != 0);
                        v[0] = (ce == 0) ? res : v[0];
                        v[1] = (ce == 1) ? res : v[1];
                        v[2] = (ce == 2) ? res : v[2];
                        v[3] = (ce == 3) ? res : v[3];
                    }
                    if (row_edge) {  // rows 0 and nx-1 by the general rule, one cell at a time
#pragma unroll 1
                        for (int c = 0; c < 4; c++) {
                            const int gj = gj0 + c;
                            if (gj < 0 || gj >= p.ny) continue;
                            const float tcv = (COEF == WG_COEF_TABLE && a.tc) ? a.tc[(size_t)r * p.pitch + gj] : 0.f;
                            const XV res = skew_cell<COEF, true, false, INL>(
                                p, a, r, gj, lv, pick4(Wc[0], Wc[1], Wc[2], Wc[3], c), pick4(Yl[0], Yl[1], Yl[2], Yl[3], c),
                                pick4(el(W[lv - 1][2], 0), el(W[lv - 1][2], 1), el(W[lv - 1][2], 2), el(W[lv - 1][2], 3), c),
                                pick4(el(W[lv - 1][0], 0), el(W[lv - 1][0], 1), el(W[lv - 1][0], 2), el(W[lv - 1][0], 3), c),
                                pick4(Wc[1], Wc[2], Wc[3], e3, c), pick4(w0, Wc[0], Wc[1], Wc[2], c),
                                pick4(Tl[0], Tl[1], Tl[2], Tl[3], c), tcv,
                                NEED_ACT ? ((aq >> (4 * lv + c)) & 1u) : true);
                            v[0] = (c == 0) ? res : v[0];
                            v[1] = (c == 1) ? res : v[1];
                            v[2] = (c == 2) ? res : v[2];
                            v[3] = (c == 3) ? res : v[3];
                        }
                    } else if (src_lane && r == p.src_i) {  // the general rule adds it on rows 0 and nx-1
                        const double add = INL ? src_inl(p, a.t0 + lv) : a.src[lv - 1];
                        const int cs = p.src_j - gj0;
#pragma unroll
                        for (int c = 0; c < 4; c++) v[c] = (cs == c) ? source32(v[c], add) : v[c];
                    }
                }
                }  // levels in use
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    if (GEN) W[lv][0][h] = W[lv][1][h];
                    W[lv][1][h] = W[lv][2][h];
                    W[lv][2][h] = make_float2(v[2 * h].x, v[2 * h + 1].x);
                    V[lv - 1][h] = pend[h];  // level lv-1's row r+1: level lv has read row r
                    pend[h] = make_float2(v[2 * h].v, v[2 * h + 1].v);
                }
            }
            ts = (ts == K) ? 0 : ts + 1;  // row m+1's tcc slot
            const int r = m - K;
            if (lane_core && r >= i_s && r < i_e) {
                const size_t o = (size_t)r * p.pitch + gj0;
                if (gj0 + 3 < p.ny) {
                    if (grp_ok) {
                        *reinterpret_cast<float4 *>(a.phi_out + o) = make_float4(W[K][2][0].x, W[K][2][0].y, W[K][2][1].x, W[K][2][1].y);
                        *reinterpret_cast<float4 *>(a.psi_out + o) = make_float4(pend[0].x, pend[0].y, pend[1].x, pend[1].y);
                    }
                } else if (grp_ok) {
#pragma unroll
                    for (int c = 0; c < 4; c++)
                        if (gj0 + c < p.ny) {
                            a.phi_out[o + c] = el(W[K][2], c);
                            a.psi_out[o + c] = el(pend, c);
                        }
                }
            }
        }
    }
    cp_async_wait<0>();  // rows prefetched past the strip land before the ring is reused
}

// One warp per task: column tile tj (x), rows [i_s, i_e) (y, z), and its kind (w): 0 inner,
// 1 column 0 / column ny-1 / point source, 2 rows 0 and nx-1 or a column ny-1 that is not
// a group's last.  The task list fills one wave of resident warps.  PL: 0 general, 1 PLAIN,
// 2 PLAIN with KAPPA = 0.
template <int COEF, int K, int PL>
__global__ void __launch_bounds__(128, 4) k_step_skew(const __grid_constant__ DevParams p, const __grid_constant__ TbArgs a,
                                                      const int4 *__restrict__ tasks, int ntasks)
{
    constexpr int H = (K + 3) & ~3, STEP = 128 - 2 * H;
    extern __shared__ float4 skew_smem[];
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (warp >= ntasks) return;  // warp-uniform
    float *ring = reinterpret_cast<float *>(skew_smem) + (threadIdx.x >> 5) * SkewSlot<COEF>::DEPTH * SkewSlot<COEF>::SIZE;
    float *tring = reinterpret_cast<float *>(skew_smem) + 4 * SkewSlot<COEF>::DEPTH * SkewSlot<COEF>::SIZE +
                   (threadIdx.x >> 5) * (K + 1) * 128;  // table scenes: tcc of the last K+1 rows
    const int4 t = tasks[warp];
    const int gj0 = t.x * STEP - H + 4 * lane;
    const int lo = t.x * STEP, hi = lo + STEP;  // the core columns of tile t.x
    constexpr bool PLAIN = PL >= 1, KZ = PL == 2;
    // Programmatic dependent launch: this pass may be launched while the previous one is
    // finishing (its blocks take the SMs the previous pass's blocks leave); it reads and
    // writes the fields only after the previous pass has completed and its writes are
    // visible.  The next pass may be launched from here on.
    pdl_wait();
    pdl_trigger();
    if (t.w == 2) skew_strip<COEF, K, PLAIN, true, false, KZ>(p, a, t.y, t.z, gj0, lane, ring, tring, true, lo, hi);
    else skew_strip<COEF, K, PLAIN, false, false, KZ>(p, a, t.y, t.z, gj0, lane, ring, tring, t.w == 1, lo, hi);
}

// dynamic shared memory of k_step_skew: 4 warps x (row ring + tcc ring of K+1 rows, table scenes)
template <int COEF, int K>
constexpr size_t skew_smem_bytes()
{
    return 4 * (SkewSlot<COEF>::DEPTH * SkewSlot<COEF>::SIZE + (COEF == WG_COEF_TABLE ? (K + 1) * 128 : 0)) * sizeof(float);
}

static bool skew_shape_ok(const DevParams &p, int K, int S)
{
    return K >= 2 && K <= WG_SKEW_MAX_K && S >= 8 && S <= 4096 && p.ny >= 8 && p.nx >= 2;
}

static int sm_count()
{
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <int COEF, int K, int PL>
static int skew_capacity()
{
    constexpr size_t smem = skew_smem_bytes<COEF, K>();
    static int per_sm = 0;
    if (!per_sm) {
        cudaFuncSetAttribute(k_step_skew<COEF, K, PL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_step_skew<COEF, K, PL>, 128, smem);
        per_sm = nb > 0 ? nb : 1;
    }
    return per_sm * sm_count() * 4;
}

template <int COEF, int K, int PL>
static void launch_skew_k(const DevParams &p, const TbArgs &a, const int4 *tasks, int ntasks, cudaStream_t st)
{
    constexpr size_t smem = skew_smem_bytes<COEF, K>();
    skew_capacity<COEF, K, PL>();  // sets the shared-memory attribute once
    launch_pdl(k_step_skew<COEF, K, PL>, dim3((unsigned)((ntasks + 3) / 4)), dim3(128), smem, st, p, a, tasks, ntasks);
}

template <int COEF, int PL>
static int skew_dispatch(const DevParams &p, const TbArgs *a, int K, const int4 *tasks, int ntasks, cudaStream_t st)
{
    // a == nullptr: return the number of resident warps instead of launching
    switch (K) {
    case 2: if (!a) return skew_capacity<COEF, 2, PL>(); launch_skew_k<COEF, 2, PL>(p, *a, tasks, ntasks, st); break;
    case 3: if (!a) return skew_capacity<COEF, 3, PL>(); launch_skew_k<COEF, 3, PL>(p, *a, tasks, ntasks, st); break;
    case 4: if (!a) return skew_capacity<COEF, 4, PL>(); launch_skew_k<COEF, 4, PL>(p, *a, tasks, ntasks, st); break;
    case 5: if (!a) return skew_capacity<COEF, 5, PL>(); launch_skew_k<COEF, 5, PL>(p, *a, tasks, ntasks, st); break;
    default: if (!a) return skew_capacity<COEF, 6, PL>(); launch_skew_k<COEF, 6, PL>(p, *a, tasks, ntasks, st); break;
    }
    return 0;
}

static int skew_call(const DevParams &p, const TbArgs *a, int coef, int K, const int4 *tasks, int ntasks, cudaStream_t st)
{
    const bool plain = p.twospeeds && !p.floor_clamp;
    const int pl = !plain ? 0 : (p.kappa == 0.0 ? 2 : 1);
    if (coef == WG_COEF_TABLE) {
        if (pl == 2) return skew_dispatch<WG_COEF_TABLE, 2>(p, a, K, tasks, ntasks, st);
        return pl ? skew_dispatch<WG_COEF_TABLE, 1>(p, a, K, tasks, ntasks, st)
                  : skew_dispatch<WG_COEF_TABLE, 0>(p, a, K, tasks, ntasks, st);
    }
    if (pl == 2) return skew_dispatch<WG_COEF_MASK, 2>(p, a, K, tasks, ntasks, st);
    return pl ? skew_dispatch<WG_COEF_MASK, 1>(p, a, K, tasks, ntasks, st)
              : skew_dispatch<WG_COEF_MASK, 0>(p, a, K, tasks, ntasks, st);
}

// Task list of a skewed pass.  Every column tile is cut into a top and a bottom segment
// of R rows (kind 2) and row chunks in between; a chunk costs its rows plus 2K+1 rows of
// pipeline fill, and a row of a boundary column tile about SKEW_EDGE_COST rows of an
// inner one.  Chunks are sized so that all warps carry about the same cost and the list
// fills the resident warps once (inner chunks of at least min_rows rows).  Tasks are
// ordered by row band so that the boundary chunks spread over the SMs.
// shifted = false: tile tj spans columns [tj*step - H, tj*step - H + 128) and stores
// [tj*step, (tj+1)*step).  shifted = true (batches): tile tj starts at column tj*step, so
// the first tile needs no halo on the left and the last none on the right (column 0 and
// ny-1 read no column outside the grid); a scene of 128 columns or fewer is one tile.
#define SKEW_EDGE_COST 1.9  // per-warp timing of the 3840x2160 passes: 1.87 (K 4), 1.90 (K 5)
static std::vector<int4> skew_plan(const DevParams &p, int K, int min_rows, int cap, bool shifted = false)
{
    const int H = (K + 3) & ~3, step = 128 - 2 * H, F = 2 * K + 1, sh = shifted ? 0 : H;
    const int nx = p.nx;
    const int tiles_j = shifted ? 1 + std::max(0, (p.ny - 128 + step - 1) / step) : (p.ny + step - 1) / step;
    // rows of a top or bottom segment (the halo of a middle chunk stays off rows 0 and nx-1):
    // K+1 for single grids (+3% on 3840x2160), at least 8 for batches of small scenes (+2%)
    const int R = shifted ? std::max(K + 1, 8) : K + 1;
    const bool segs = nx >= 2 * R + 1;  // else every task is of kind 2
    const int mid0 = segs ? R : 0, mid1 = segs ? nx - R : nx, nmid = mid1 - mid0;
    std::vector<int> col_kind(tiles_j);  // 0 inner, 1 column 0 or ny-1 (last of a group), 2 ny-1 elsewhere
    int n_edge = 0;
    for (int tj = 0; tj < tiles_j; tj++) {
        const int t0 = tj * step - sh;
        const bool left = t0 < 1, right = t0 + 128 > p.ny - 1;
        col_kind[tj] = (right && (p.ny & 3) != 0) ? 2 : ((left || right) ? 1 : 0);
        n_edge += col_kind[tj] != 0;
    }
    const int n_inner = tiles_j - n_edge;
    const int nseg = segs ? 2 * tiles_j : 0;
    const int capm = std::max(cap - nseg, tiles_j);
    auto edge_chunks = [&](int nl) {
        const double rows_l = std::ceil((double)nmid / nl) + F;
        const double re = rows_l / SKEW_EDGE_COST - F;
        return re >= 1.0 ? std::min(nmid, (int)std::ceil(nmid / re)) : nmid;
    };
    int nl = 1;
    const int nl_max = std::max(1, nmid / std::max(min_rows, 1));
    for (int c = 1; c <= nl_max; c++) {
        const int need = n_inner * c + n_edge * (n_inner ? edge_chunks(c) : c);
        if (need > capm && c > 1) break;
        nl = c;
    }
    const int ne = n_inner ? edge_chunks(nl) : nl;
    struct T { double key; int4 t; };
    std::vector<T> ts;
    auto add = [&](int tj, int i_s, int i_e, int kind) {
        const int t0 = tj * step - sh;
        const bool src = p.src_on && p.src_i >= i_s - K && p.src_i < i_e + K && p.src_j >= t0 && p.src_j < t0 + 128;
        if (kind == 0 && src) kind = 1;
        ts.push_back({(i_s + i_e) * 0.5 / nx + tj * 1e-9, make_int4(tj, i_s, i_e, kind)});
    };
    for (int tj = 0; tj < tiles_j; tj++) {
        if (segs) {
            add(tj, 0, R, 2);
            add(tj, nx - R, nx, 2);
        }
        const int n = col_kind[tj] ? ne : nl;
        for (int q = 0; q < n; q++) {
            const int i_s = mid0 + (int)((long long)q * nmid / n), i_e = mid0 + (int)((long long)(q + 1) * nmid / n);
            if (i_s < i_e) add(tj, i_s, i_e, segs ? col_kind[tj] : 2);
        }
    }
    std::sort(ts.begin(), ts.end(), [](const T &x, const T &y) { return x.key < y.key; });
    std::vector<int4> out(ts.size());
    for (size_t i = 0; i < ts.size(); i++) out[i] = ts[i].t;
    return out;
}

// Task list of (depth K, minimum rows L) for this scene, built once and kept on the device.
static wg_status skew_tasks(wg_scene *s, int K, int L, const int4 **tasks, int *ntasks)
{
    if (K < 0 || K > WG_SKEW_MAX_K) { set_error("skewed depth %d outside 0..%d", K, WG_SKEW_MAX_K); return WG_ERR_INVALID; }
    SkewPlanCache &c = s->skew[K];
    if (!c.dev || c.min_rows != L) {
        const int cap = skew_call(s->dp, nullptr, s->coef, K, nullptr, 0, s->st);
        const std::vector<int4> v = skew_plan(s->dp, K, L, cap);
        if (c.dev) cudaFree(c.dev);
        c.dev = nullptr;
        WG_CUDA(cudaMalloc(&c.dev, v.size() * sizeof(int4)));
        WG_CUDA(cudaMemcpy(c.dev, v.data(), v.size() * sizeof(int4), cudaMemcpyHostToDevice));
        c.n = (int)v.size();
        c.min_rows = L;
    }
    *tasks = c.dev;
    *ntasks = c.n;
    return WG_OK;
}

// ---------------------------------------------------------------------------
// Skewed passes over a batch of scenes (mask coefficients, FP32).  Persistent warps take
// tasks from a ticket counter: table entry, first column of the tile (shifted tiling),
// rows i_s | i_e << 16, kind.  The scene's parameters are staged in the warp's shared
// memory.  Pass q of a frame reads pair (pair ^ q) of the scene (with the
// scene's cur on the first pass, 0 after) and writes the other pair.  Oscillating values
// and source increments are computed inline at update time + toff + level.
// ---------------------------------------------------------------------------
static_assert(sizeof(DevParams) % 4 == 0, "DevParams is copied as 32-bit words");

template <int K>
__global__ void __launch_bounds__(128, 4) k_batch_skew(const SlotDev *__restrict__ tab, const SlotDyn *__restrict__ dyn,
                                                       const int4 *__restrict__ tasks, const int *__restrict__ ntasks,
                                                       int *__restrict__ ticket, int q, int toff)
{
    constexpr int H = (K + 3) & ~3;
    using SL = SkewSlot<WG_COEF_MASK>;
    extern __shared__ float4 skew_smem[];
    __shared__ DevParams s_p[4];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float *ring = reinterpret_cast<float *>(skew_smem) + wid * SL::DEPTH * SL::SIZE;
    DevParams &p = s_p[wid];
    pdl_wait();  // launched by launch_pdl: the previous pass (or ghost refresh) has completed
    pdl_trigger();
    const int n = *ntasks;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(ticket, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= n) break;  // warp-uniform
        const int4 w = tasks[t];
        // the scene's parameters are staged in the warp's shared memory; the pass
        // arguments are built by every lane (the same values)
        const SlotDev &sd = tab[w.x];
        __syncwarp();  // every lane is done with the previous task's parameters
        {
            const int *src = reinterpret_cast<const int *>(&sd.p);
            int *dst = reinterpret_cast<int *>(&p);
            for (int k = lane; k < (int)(sizeof(DevParams) / 4); k += 32) dst[k] = src[k];
        }
        __syncwarp();
        const SlotDyn dy = dyn[sd.slot];
        const int pin = dy.pair ^ (q & 1), pout = pin ^ 1;
        TbArgs a;
        a.phi = (const float *)sd.f[2 * pin];
        a.psi = (const float *)sd.f[2 * pin + 1];
        a.phi_out = (float *)sd.f[2 * pout];
        a.psi_out = (float *)sd.f[2 * pout + 1];
        a.act = sd.act;
        a.tcc = a.tc = nullptr;
        a.c2 = sd.cf[CF_C2];
        a.c2b = sd.cf[CF_C2B];
        a.gam = sd.cf[CF_GAM];
        a.gamb = sd.cf[CF_GAMB];
        a.kappa = sd.cf[CF_KAPPA];
        a.ks = sd.cf[CF_KS];
        a.kt = sd.cf[CF_KT];
        a.gs = sd.cf[CF_GS];
        a.gt = sd.cf[CF_GT];
        a.vmax = sd.cf[CF_VMAX];
        a.courant = sd.cf[CF_COURANT];
        a.courantb = sd.cf[CF_COURANTB];
        a.t0 = dy.time + toff;
        a.osc = nullptr;
        a.src = nullptr;
        a.err = nullptr;
        const int i_s = w.z & 0xFFFF, i_e = (int)((unsigned)w.z >> 16);
        const int gjs = w.y, gj0 = gjs + 4 * lane;
        // one call site per strip form, so that inner, edge and periodic tiles share a loop
        const bool wrap = w.w == 3;  // periodic, ghost layout: a halo on both sides of every tile
        const int lo = wrap ? max(gjs + H, 0) : (gjs <= 0 ? 0 : gjs + H);
        const int hi = wrap ? min(gjs + 128 - H, sd.p.ny) : (gjs + 128 >= sd.p.ny ? sd.p.ny : gjs + 128 - H);
        if (w.w == 2) skew_strip<WG_COEF_MASK, K, false, true, true>(p, a, i_s, i_e, gj0, lane, ring, nullptr, true, lo, hi);
        else skew_strip<WG_COEF_MASK, K, false, false, true>(p, a, i_s, i_e, gj0, lane, ring, nullptr, w.w == 1, lo, hi, wrap);
    }
}

// dynamic shared memory of k_batch_skew: 4 warps x row ring
template <int K>
constexpr size_t batch_skew_smem()
{
    return 4 * SkewSlot<WG_COEF_MASK>::DEPTH * SkewSlot<WG_COEF_MASK>::SIZE * sizeof(float);
}

template <int K>
static int batch_skew_cap_k()
{
    constexpr size_t smem = batch_skew_smem<K>();
    static int per_sm = 0;
    if (!per_sm) {
        cudaFuncSetAttribute(k_batch_skew<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_skew<K>, 128, smem);
        per_sm = nb > 0 ? nb : 1;
    }
    return per_sm * sm_count() * 4;
}

int batch_skew_tiles(const DevParams &p, int K)
{
    const int step = 128 - 2 * ((K + 3) & ~3);
    if (p.b_cond == WG_BC_PERIODIC) return (p.ny + step - 1) / step;  // halo on both sides of every tile
    return 1 + std::max(0, (p.ny - 128 + step - 1) / step);
}

int batch_skew_capacity(int K)
{
    switch (K) {
    case 2: return batch_skew_cap_k<2>();
    case 3: return batch_skew_cap_k<3>();
    case 4: return batch_skew_cap_k<4>();
    case 5: return batch_skew_cap_k<5>();
    case 6: return batch_skew_cap_k<6>();
    default: return 0;
    }
}

void launch_batch_skew(int K, const SlotDev *tab, const SlotDyn *dyn, const int4 *tasks, const int *ntasks, int *ticket,
                       int q, int toff, cudaStream_t st)
{
    const int blocks = std::max(1, batch_skew_capacity(K) / 4);
    const dim3 g(blocks), b(128);
    switch (K) {
    case 2: launch_pdl(k_batch_skew<2>, g, b, batch_skew_smem<2>(), st, tab, dyn, tasks, ntasks, ticket, q, toff); break;
    case 3: launch_pdl(k_batch_skew<3>, g, b, batch_skew_smem<3>(), st, tab, dyn, tasks, ntasks, ticket, q, toff); break;
    case 4: launch_pdl(k_batch_skew<4>, g, b, batch_skew_smem<4>(), st, tab, dyn, tasks, ntasks, ticket, q, toff); break;
    case 5: launch_pdl(k_batch_skew<5>, g, b, batch_skew_smem<5>(), st, tab, dyn, tasks, ntasks, ticket, q, toff); break;
    case 6: launch_pdl(k_batch_skew<6>, g, b, batch_skew_smem<6>(), st, tab, dyn, tasks, ntasks, ticket, q, toff); break;
    default: break;
    }
}

bool batch_wrap_ok(const wg_params &p, int prec)
{
    // nx + 2 ghost-row bands within a grid dimension of the mask's ghost kernel (65535)
    return prec == WG_FP32 && p.b_cond == WG_BC_PERIODIC && !p.bc_neumann && !p.src_on && !p.oscillate_left &&
           !p.oscillate_topbot && p.ny >= 8 && p.nx >= 2 && p.nx + 2 * BATCH_GHOST_ROWS <= 0xFFFF;
}

bool batch_skew_ok(const wg_params &p, int prec)
{
    if (batch_wrap_ok(p, prec)) return true;
    return prec == WG_FP32 && (p.b_cond == WG_BC_DIRICHLET || p.b_cond == WG_BC_ABSORBING) && !p.bc_neumann &&
           p.ny >= 8 && p.nx >= 2 && p.nx <= 0xFFFF;
}

void batch_skew_plan(const DevParams &p, int entry, int K, int rows, std::vector<int4> &tasks, std::vector<float> &cost)
{
    const int H = (K + 3) & ~3, step = 128 - 2 * H, F = 2 * K + 1;
    if (p.b_cond == WG_BC_PERIODIC) {  // ghost layout: every tile inner (kind 3), rows in chunks of rows..2 rows
        const int tiles_j = (p.ny + step - 1) / step, nl = std::max(1, p.nx / std::max(rows, 1));
        for (int tj = 0; tj < tiles_j; tj++)
            for (int q = 0; q < nl; q++) {
                const int i_s = (int)((long long)q * p.nx / nl), i_e = (int)((long long)(q + 1) * p.nx / nl);
                if (i_s >= i_e) continue;
                tasks.push_back(make_int4(entry, tj * step - H, (int)((unsigned)i_s | ((unsigned)i_e << 16)), 3));
                cost.push_back((float)(i_e - i_s + F));
            }
        return;
    }
    const std::vector<int4> v = skew_plan(p, K, rows, 1 << 30, true);  // inner chunks of rows..2 rows rows
    for (const int4 &t : v) {
        tasks.push_back(make_int4(entry, t.x * step, (int)((unsigned)t.y | ((unsigned)t.z << 16)), t.w));
        cost.push_back((float)((t.z - t.y + F) * (t.w ? SKEW_EDGE_COST : 1.0)));
    }
}

static int tb_halo(int K) { return (K + 3) & ~3; }

static bool tb_shape_ok(int K, int L, int W)
{
    return K >= 2 && K <= 8 && (W == 128 || W == 256) && L >= 16 && L <= 64 && (L % 2 == 0) && L - 2 * K >= 8 &&
           W - 2 * tb_halo(K) >= 32 && tb_layout(WG_COEF_TABLE, L, W).bytes <= 200 * 1024;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)f;
    });
    return fn;
}

// 2-D map over a pitched array of 4-byte elements: dims {cols, rows}, row stride bytes
static bool make_map(CUtensorMap *m, const void *base, bool is_float, uint64_t cols, uint64_t rows, uint64_t stride,
                     uint32_t box_cols, uint32_t box_rows)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {cols, rows};
    cuuint64_t strides[1] = {stride};
    cuuint32_t box[2] = {box_cols, box_rows};
    cuuint32_t es[2] = {1, 1};
    return fn(m, is_float ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void *>(base),
              dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct TbMaps {
    CUtensorMap phi, psi, tcc, act;
};

static bool tb_maps(wg_scene *s, const TbArgs &a, int L, int W, TbMaps *m)
{
    const uint64_t stride = (uint64_t)s->pitch * 4;
    bool ok = make_map(&m->phi, a.phi, true, s->prm.ny, s->prm.nx, stride, W, L) &&
              make_map(&m->psi, a.psi, true, s->prm.ny, s->prm.nx, stride, W, L) &&
              make_map(&m->act, s->act, false, s->dp.wpitch, s->prm.nx, (uint64_t)s->dp.wpitch * 4, TB_AW, L);
    if (ok && s->coef == WG_COEF_TABLE) ok = make_map(&m->tcc, a.tcc, true, s->prm.ny, s->prm.nx, stride, W, L);
    else m->tcc = m->phi;
    return ok;
}

static bool launch_tb(wg_scene *s, const TbArgs &a, int K, int L, int W)
{
    if (!tb_shape_ok(K, L, W)) return false;
    const int Kh = tb_halo(K);
    TbMaps m;
    if (!tb_maps(s, a, L, W, &m)) {
        set_error("cuTensorMapEncodeTiled failed");
        return false;
    }
    const DevParams &p = s->dp;
    dim3 grd((p.ny + (W - 2 * Kh) - 1) / (W - 2 * Kh), (p.nx + (L - 2 * K) - 1) / (L - 2 * K));
    const size_t sm = tb_layout(s->coef, L, W).bytes;
    static std::once_flag attr_once;  // raise the dynamic shared-memory limit once per process
    std::call_once(attr_once, [] {
        cudaFuncSetAttribute(k_step_tb<WG_COEF_TABLE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_step_tb<WG_COEF_MASK>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    });
    if (s->coef == WG_COEF_TABLE)
        k_step_tb<WG_COEF_TABLE><<<grd, W, sm, s->st>>>(p, a, m.phi, m.psi, m.tcc, m.act, K, Kh, L);
    else
        k_step_tb<WG_COEF_MASK><<<grd, W, sm, s->st>>>(p, a, m.phi, m.psi, m.tcc, m.act, K, Kh, L);
    return true;
}

static bool tb_depth_ok(int k) { return k >= 2 && k <= 8; }

bool tb_supported(const wg_scene *s)
{
    return s->prec == WG_FP32 && (s->prm.b_cond == WG_BC_DIRICHLET || s->prm.b_cond == WG_BC_ABSORBING) &&
           s->nrec == 0 && !s->has_ghosts && (s->coef == WG_COEF_MASK || s->tg == nullptr);
}

static wg_status ensure_tb_buffers(wg_scene *s)
{
    const size_t fb = (size_t)s->prm.nx * s->pitch * s->esz;
    for (int k = 0; k < 2; k++)
        if (!s->g[k]) {
            WG_CUDA(cudaMalloc(&s->g[k], fb));
            WG_CUDA(cudaMemsetAsync(s->g[k], 0, fb, s->st));
        }
    return WG_OK;
}

wg_status tb_prepare(wg_scene *s, int n)
{
    if (!s->prm.oscillate_left && !s->prm.src_on) return WG_OK;
    const size_t need = (size_t)n * (s->prm.oscillate_left ? s->prm.ny : 1);
    if (need > s->bv_cap) {
        if (s->bv_osc) cudaFree(s->bv_osc);
        if (s->bv_src) cudaFree(s->bv_src);
        s->bv_osc = nullptr;
        s->bv_src = nullptr;
        s->bv_cap = 0;
        WG_CUDA(cudaMalloc(&s->bv_osc, need * sizeof(float)));
        WG_CUDA(cudaMalloc(&s->bv_src, need * sizeof(double)));
        s->bv_cap = need;
    }
    s->bv_t0 = s->time;
    const int threads = 256, blocks = (int)((need + threads - 1) / threads);
    launch_pdl(k_boundary_values, dim3(blocks), dim3(threads), 0, s->st, s->dp, s->time, n, s->bv_osc, s->bv_src);
    s->launches++;
    WG_CUDA(cudaGetLastError());
    return WG_OK;
}

static TbArgs tb_args(wg_scene *s)
{
    TbArgs a;
    a.phi = (const float *)s->f[s->cur];
    a.psi = (const float *)s->f[1 - s->cur];
    a.phi_out = (float *)s->g[0];
    a.psi_out = (float *)s->g[1];
    a.act = s->act;
    a.tcc = (const float *)s->tcc;
    a.tc = (const float *)s->tc;
    a.c2 = (float)s->dp.c2;
    a.c2b = (float)s->dp.c2b;
    a.gam = (float)s->dp.gam;
    a.gamb = (float)s->dp.gamb;
    a.kappa = (float)s->dp.kappa;
    a.ks = (float)s->dp.kappa_sides;
    a.kt = (float)s->dp.kappa_topbot;
    a.gs = (float)s->dp.gamma_sides;
    a.gt = (float)s->dp.gamma_topbot;
    a.vmax = (float)s->dp.vmax;
    a.courant = (float)s->dp.courant;
    a.courantb = (float)s->dp.courantb;
    a.t0 = s->time;
    const long long off = s->time - s->bv_t0;
    a.osc = s->bv_osc ? s->bv_osc + off * s->prm.ny : nullptr;
    a.src = s->bv_src ? s->bv_src + off : nullptr;
    a.err = s->dflag;
    return a;
}

template <>
wg_status tb_pass<float>(wg_scene *s, int k)
{
    wg_status st = ensure_tb_buffers(s);
    if (st) return st;
    if (!tb_depth_ok(k)) { set_error("temporal block depth %d outside 2..8", k); return WG_ERR_INVALID; }
    const int W = s->tile_j > 0 ? s->tile_j : 256, L = s->tile_i > 0 ? s->tile_i : 32;
    TbArgs a = tb_args(s);
    if (W == 1) {  // time-skewed streaming strips of L rows
        if (!skew_shape_ok(s->dp, k, L)) {
            set_error("unsupported skewed strip (depth %d of 2..6, %d rows of 8..4096, ny >= 8)", k, L);
            return WG_ERR_INVALID;
        }
        const int4 *tasks = nullptr;
        int ntasks = 0;
        if ((st = skew_tasks(s, k, L, &tasks, &ntasks))) return st;
        skew_call(s->dp, &a, s->coef, k, tasks, ntasks, s->st);
    } else if (clear_error(), !launch_tb(s, a, k, L, W)) {
        if (wg_last_error()[0] == 0) set_error("unsupported temporal block (depth %d, tile %d x %d)", k, L, W);
        return WG_ERR_INVALID;
    }
    s->launches++;
    // the pass's outputs become the scene's fields; the inputs become the next outputs
    std::swap(s->f[s->cur], s->g[0]);
    std::swap(s->f[1 - s->cur], s->g[1]);
    s->time += k;
    return WG_OK;
}

template <>
wg_status tb_pass<double>(wg_scene *, int)
{
    set_error("temporal blocking is FP32 only");
    return WG_ERR_STATE;
}

int tb_pass_depth(int k, int remaining)
{
    // largest compiled depth <= min(k, remaining); 0 = use single updates
    const int m = std::min(std::min(k, remaining), 8);
    return m >= 2 ? m : 0;
}

// ---------------------------------------------------------------------------
// Autotuner: temporal-block depth and tile width per size class, measured once per
// (size class, coefficient mode) with CUDA events on a copy of the scene's state.
// ---------------------------------------------------------------------------
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, int>, std::tuple<int, int, int>> g_tune;

static std::tuple<int, int, int, int> size_class(const wg_scene *s)
{
    auto lg = [](int v) { int c = 0; while ((1 << (c + 1)) <= v) c++; return c; };
    return {lg(s->prm.nx), lg(s->prm.ny), s->coef, s->prm.b_cond};
}

void autotune_scene(wg_scene *s)
{
    if (!tb_supported(s)) {
        s->tb_k = 1;
        s->tile_i = s->tile_j = 0;
        return;
    }
    const auto key = size_class(s);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            std::tie(s->tb_k, s->tile_i, s->tile_j) = it->second;
            return;
        }
    }
    // save the state, time the candidates, restore the state
    const size_t fb = (size_t)s->prm.nx * s->pitch * s->esz;
    void *save[2] = {nullptr, nullptr};
    bool ok = ensure_tb_buffers(s) == WG_OK;
    for (int k = 0; k < 2 && ok; k++) ok = cudaMalloc(&save[k], fb) == cudaSuccess;
    int best_k = 1, best_l = 0, best_w = 0;
    if (ok) {
        cudaMemcpyAsync(save[0], s->f[0], fb, cudaMemcpyDeviceToDevice, s->st);
        cudaMemcpyAsync(save[1], s->f[1], fb, cudaMemcpyDeviceToDevice, s->st);
        const long long t_save = s->time;
        const int cur_save = s->cur;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        const int updates = 120;  // a multiple of every depth 2..6; long enough for stable timings
        float best = 1e30f;
        struct Cand { int k, l, w; };
        const Cand cands[] = {{1, 0, 0},    {2, 16, 256}, {3, 16, 256}, {4, 16, 256}, {4, 24, 256},
                              {6, 32, 256}, {4, 32, 128}, {2, 16, 1},   {3, 16, 1},   {4, 16, 1},
                              {5, 16, 1},   {6, 16, 1},   {4, 48, 1}};
        for (const Cand &c : cands) {
            s->tb_k = c.k;
            s->tile_i = c.l;
            s->tile_j = c.w;
            float ms_best = 1e30f;
            for (int rep = 0; rep < 3; rep++) {
                cudaEventRecord(e0, s->st);
                const wg_status st = scene_step_impl<float>(s, updates);
                cudaEventRecord(e1, s->st);
                if (st != WG_OK) {  // a shape this scene does not take
                    cudaEventSynchronize(e1);
                    clear_error();
                    ms_best = 1e30f;
                    break;
                }
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0) ms_best = std::min(ms_best, ms);
            }
            if (ms_best < best * 0.99f) {  // a later candidate must be faster by more than the noise
                best = ms_best;
                best_k = c.k;
                best_l = c.l;
                best_w = c.w;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        s->cur = cur_save;
        cudaMemcpyAsync(s->f[0], save[0], fb, cudaMemcpyDeviceToDevice, s->st);
        cudaMemcpyAsync(s->f[1], save[1], fb, cudaMemcpyDeviceToDevice, s->st);
        cudaStreamSynchronize(s->st);
        s->time = t_save;
    }
    for (void *p : save)
        if (p) cudaFree(p);
    cudaGetLastError();
    s->tb_k = best_k;
    s->tile_i = best_l;
    s->tile_j = best_w;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = {best_k, best_l, best_w};
}

}  // namespace wg
