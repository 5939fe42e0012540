// wg_batch.cu — many scenes of uneven sizes advanced together.
//
// Single updates: every active scene is cut into work items of BT_ROWS rows x (64
// threads x V) columns; a frame of n updates is n launches of one persistent kernel
// (k_batch_step, sized to fill every SM) whose CTAs take (scene, item) pairs from a
// device-side atomic counter, plus one kernel that advances each scene's step counter.
// The whole frame is recorded once as a CUDA graph and replayed; the scene table, the
// work counts and the per-scene time and buffer parity live in device memory, so
// admitting or removing scenes changes data, not the graph.
//
// The per-cell arithmetic is the single-scene kernels' (k_step_bulk / fast_edge), so a
// scene advanced in a batch is bit-identical to the same scene advanced alone.  FP64
// scenes update in place (the new level overwrites psi); FP32 scenes (phi and the
// velocity) write each update into their other pair of fields.
//
// FP32 scenes with mirror ("Dirichlet"), absorbing or periodic boundaries (periodic ones
// in the ghost layout of wg_batch.h) take skewed passes instead (k_batch_skew, wg_tb.cu):
// a frame of n updates is a few passes of 2..6 updates
// each, at the depth class tuned for the scene's size class, writing between two buffer
// pairs.  Each depth class runs as its own branch of the frame's graph, beside the chain
// of single updates of the other scenes.  The skewed cells are the single-update cells
// bit for bit, so a batch gives the same fields with and without skewed passes.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>
#include "wg_internal.h"
#include "wg_scene.h"
#include "wg_cells.cuh"
#include "wg_batch.h"

namespace wg {

// A boundary-line cell (reference rules) plus the point source; out of line so that
// the tile loop below stays small.  Its arguments are plain pointers and values: the
// rule's argument block is built here, in registers of this call, not passed by address
// (an address taken across the call would put the block in local memory).
// FP64 fields: phi and psi (y = the cell's psi); returns the new value.
// FP32 fields: phi and the velocity vel; returns the new phi and velocity.
template <class T>
__device__ __forceinline__ FastArgs<T> batch_args(const float *cf, const T *phi, const T *psi, const uint32_t *act,
                                                  const uint32_t *nz)
{
    FastArgs<T> a;
    a.phi = phi;
    a.psi = psi;
    a.out = nullptr;
    a.vout = nullptr;
    a.act = act;
    a.nz = nz;
    a.tcc = a.tc = a.tg = nullptr;
    a.c2f = cf[CF_C2];  // rounded on the host (a conversion here would run on the FP64 pipe)
    a.c2bf = cf[CF_C2B];
    a.gamf = cf[CF_GAM];
    a.gambf = cf[CF_GAMB];
    a.kappaf = cf[CF_KAPPA];
    a.courantf = cf[CF_COURANT];
    a.courantbf = cf[CF_COURANTB];
    a.ksf = cf[CF_KS];
    a.ktf = cf[CF_KT];
    a.gsf = cf[CF_GS];
    a.gtf = cf[CF_GT];
    a.vmaxf = cf[CF_VMAX];
    a.has_ghosts = 0;
    a.do_source = 1;
    return a;
}
__device__ __noinline__ double batch_edge(const DevParams &p, const float *cf, const double *phi, const double *psi,
                                          const uint32_t *act, const uint32_t *nz, int i, int j, long long time,
                                          double y)
{
    const FastArgs<double> a = batch_args<double>(cf, phi, psi, act, nz);
    double v = fast_edge<double, WG_COEF_MASK>(p, a, i, j, time, y);
    if (p.src_on && i == p.src_i && j == p.src_j) v = A_(v, point_source(p, time));
    return v;
}
__device__ __noinline__ XV batch_edge_v(const DevParams &p, const float *cf, const float *phi, const float *vel,
                                        const uint32_t *act, const uint32_t *nz, int i, int j, long long time)
{
    const FastArgs<float> a = batch_args<float>(cf, phi, vel, act, nz);
    XV r = fast_edge_v<WG_COEF_MASK>(p, a, i, j, time);
    if (p.src_on && i == p.src_i && j == p.src_j) r = source32(r, point_source(p, time));
    return r;
}

// The scene values the bulk update reads, held in registers for a work item (the
// descriptor lives in global memory, which the tile's stores could alias); the
// coefficients in the field precision only.
template <class T>
struct TileCoef {
    int nx, ny, pitch, wpitch, twospeeds, floor_clamp;
    T c2, c2b, gam, gamb, kappa;
};

// One work item.  FP64 (in place): phi, and psi = out, overwritten by the new level.
// FP32: phi and the velocity vin; the new phi and velocity go to out and vout.
// Z (FP64 scenes): upd64's flags for KAPPA = 0 and GAMMA = GAMMAB = 0, the bulk update
// without those zero terms (values unchanged).
template <class T, int Z = 0>
__device__ __forceinline__ void batch_tile(const DevParams &p, const float *cf, const T *__restrict__ phi,
                                           const T *__restrict__ vin, T *__restrict__ out, T *__restrict__ vout,
                                           const uint32_t *__restrict__ act, const uint32_t *__restrict__ nz, int i0,
                                           int jt, long long time)
{
    constexpr int V = Vec<T>::n;
    constexpr bool F32 = sizeof(T) == 4;
    TileCoef<T> k;
    k.nx = p.nx;
    k.ny = p.ny;
    k.pitch = p.pitch;
    k.wpitch = p.wpitch;
    k.twospeeds = p.twospeeds;
    k.floor_clamp = p.floor_clamp;
    if constexpr (F32) {
        k.c2 = cf[CF_C2];
        k.c2b = cf[CF_C2B];
        k.gam = cf[CF_GAM];
        k.gamb = cf[CF_GAMB];
        k.kappa = cf[CF_KAPPA];
    } else {
        k.c2 = p.c2;
        k.c2b = p.c2b;
        k.gam = p.gam;
        k.gamb = p.gamb;
        k.kappa = p.kappa;
    }
    const float vmaxf = cf[CF_VMAX];
    const int j0 = (jt * BT_THREADS + (int)threadIdx.x) * V;
    // interior rows: the bulk rule (boundary columns and padding take the unwritten-cell
    // rule for now)
    for (int rr = threadIdx.y; rr < BT_ROWS; rr += blockDim.y) {
        const int i = i0 + rr;
        if (i >= k.nx - 1 || i == 0 || j0 >= k.pitch) continue;
        const size_t row = (size_t)i * k.pitch;
        T c[V], y[V], n[V], s[V];
        vload(phi + row + j0, c);
        vload(vin + row + j0, y);
        vload(phi + row + k.pitch + j0, n);
        vload(phi + row - k.pitch + j0, s);
        const T wl = (j0 > 0) ? phi[row + j0 - 1] : (T)0;
        const T er = (j0 + V < k.pitch) ? phi[row + j0 + V] : (T)0;
        const uint32_t word = act[(size_t)i * k.wpitch + (j0 >> 5)] >> (j0 & 31);
        T o[V], ov[V];
#pragma unroll
        for (int q = 0; q < V; q++) {
            const int j = j0 + q;
            const bool ac = (word >> q) & 1u;
            const bool upd = j >= 1 && j < k.ny - 1 && (k.twospeeds || ac);
            const T x = c[q];
            const T w = (q == 0) ? wl : c[q - 1];
            const T e = (q == V - 1) ? er : c[q + 1];
            if constexpr (!F32) {
                double v = y[q];
                if (upd) {
                    const double delta = L4_(A_(A_(A_(n[q], s[q]), e), w), x);
                    v = upd64<Z>(x, y[q], ac ? k.c2 : k.c2b, delta, k.kappa, ac ? k.gam : k.gamb);
                    if (k.floor_clamp && ac) v = floor_clamp(p, v);
                }
                o[q] = (T)v;
            } else {
                XV r = keep32(x, y[q]);
                if (upd) {
                    const float delta = ((n[q] - x) + (s[q] - x)) + ((e - x) + (w - x));
                    r = upd32(x, y[q], ac ? k.c2 : k.c2b, delta, k.kappa, ac ? k.gam : k.gamb);
                    if (k.floor_clamp && ac) r = clamp32(x, r, vmaxf);
                }
                o[q] = r.x;
                ov[q] = r.v;
            }
        }
        vstore(out + row + j0, o);
        if constexpr (F32) vstore(vout + row + j0, ov);
    }
    // then the boundary lines and the point source, by the threads that stored those
    // cells above (each reads phi and its own cell's psi or velocity)
    const bool col0 = j0 == 0, colr = k.ny - 1 >= j0 && k.ny - 1 < j0 + V;
    const bool srcj = p.src_on && p.src_j >= j0 && p.src_j < j0 + V && p.src_j > 0 && p.src_j < k.ny - 1;
    auto edge = [&](size_t row, int i, int j) {
        if constexpr (F32) {
            const XV r = batch_edge_v(p, cf, phi, vin, act, nz, i, j, time);
            out[row + j] = r.x;
            vout[row + j] = r.v;
        } else {
            out[row + j] = batch_edge(p, cf, phi, out, act, nz, i, j, time, out[row + j]);
        }
    };
    for (int rr = threadIdx.y; rr < BT_ROWS; rr += blockDim.y) {
        const int i = i0 + rr;
        if (i >= k.nx || j0 >= k.pitch) continue;
        const size_t row = (size_t)i * k.pitch;
        if (i == 0 || i == k.nx - 1) {
            for (int q = 0; q < V; q++) {
                const int j = j0 + q;
                if (j >= k.ny) break;
                edge(row, i, j);
            }
            continue;
        }
        if (col0) edge(row, i, 0);
        if (colr) edge(row, i, k.ny - 1);
        if (srcj && i == p.src_i) {
            const double add = point_source(p, time);
            out[row + p.src_j] = (T)A_((double)out[row + p.src_j], add);
            if constexpr (F32) vout[row + p.src_j] = (T)A_((double)vout[row + p.src_j], add);
        }
    }
}

// Persistent blocks take work items (BT_ROWS rows x one column tile of one scene) from
// a device counter.  Each item's scene entry, first row, column tile and slot come from
// one int4 of the item table built with the scene table.  The ticket of the following
// item is taken while this one runs, and read after it, so its latency is hidden.
// all = 0: only the items of scenes without skewed passes (the first plain_tiles).
template <class T>
__global__ void __launch_bounds__(256, 4) k_batch_step(const BatchHdr *__restrict__ hdr, const SlotDev *__restrict__ tab,
                                                    const int4 *__restrict__ items, SlotDyn *__restrict__ dyn,
                                                    int *__restrict__ counter, int u, int all)
{
    __shared__ int s_next[2];
    pdl_wait();  // launched by launch_pdl: the previous update has completed
    pdl_trigger();
    const int total = all ? hdr->total_tiles : hdr->plain_tiles;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if (tid == 0) s_next[0] = atomicAdd(counter + u, 1);
    __syncthreads();
    for (int buf = 0;; buf ^= 1) {
        const int it = s_next[buf];
        if (it >= total) break;
        int next = 0;
        if (tid == 0) next = atomicAdd(counter + u, 1);
        const int4 w = items[it];
        const SlotDev &sd = tab[w.x];
        const SlotDyn d = dyn[w.w];
        const T *in, *vin;
        T *out, *vout;
        if constexpr (sizeof(T) == 4) {  // pair (pair ^ u) -> the other pair
            const int pin = d.pair ^ (u & 1);
            in = (const T *)sd.f[2 * pin];
            vin = (const T *)sd.f[2 * pin + 1];
            out = (T *)sd.f[2 * (pin ^ 1)];
            vout = (T *)sd.f[2 * (pin ^ 1) + 1];
        } else {  // in place within pair 0
            const int phase = (d.cur + u) & 1;
            in = (const T *)sd.f[phase];
            out = (T *)sd.f[1 - phase];
            vin = out;
            vout = nullptr;
        }
        int z = 0;  // block-uniform
        if constexpr (sizeof(T) == 8)
            z = (sd.p.kappa == 0.0 ? Z_KAPPA : 0) | (sd.p.gam == 0.0 && sd.p.gamb == 0.0 ? Z_GAMMA : 0);
        if (z == (Z_KAPPA | Z_GAMMA))
            batch_tile<T, Z_KAPPA | Z_GAMMA>(sd.p, sd.cf, in, vin, out, vout, sd.act, sd.nz, w.y, w.z, d.time + u + 1);
        else if (z == Z_KAPPA)
            batch_tile<T, Z_KAPPA>(sd.p, sd.cf, in, vin, out, vout, sd.act, sd.nz, w.y, w.z, d.time + u + 1);
        else
            batch_tile<T>(sd.p, sd.cf, in, vin, out, vout, sd.act, sd.nz, w.y, w.z, d.time + u + 1);
        if (tid == 0) s_next[buf ^ 1] = next;
        __syncthreads();  // the next ticket is visible; s_next[buf] is free again
    }
}

// Ghost cells of the input pair of pass q for the wrapped scenes of depth class K (K < 0:
// every wrapped scene, the current pair): each ghost cell of both fields takes the value of
// the real cell it wraps to.  Ghost cells are written and real cells read, so blocks need
// no ordering.  Block (x, y): table entry x, a share y of its ghost cells.
__global__ void k_batch_ghosts(const BatchHdr *__restrict__ hdr, const SlotDev *__restrict__ tab,
                               const SlotDyn *__restrict__ dyn, int K, int q)
{
    const int e = blockIdx.x;
    if (e >= hdr->nactive) return;
    const SlotDev &sd = tab[e];
    if (!sd.wrap || (K >= 0 && sd.skew_k != K)) return;
    const SlotDyn dy = dyn[sd.slot];
    const int pin = K < 0 ? dy.pair : dy.pair ^ (q & 1);
    float *f0 = (float *)sd.f[2 * pin], *f1 = (float *)sd.f[2 * pin + 1];
    const int nx = sd.p.nx, ny = sd.p.ny, pitch = sd.p.pitch;
    constexpr int GC = BATCH_GHOST_COLS, GR = BATCH_GHOST_ROWS;
    const int wide = ny + 2 * GC, ncol = 2 * GC * nx, total = ncol + 2 * GR * wide;
    for (int t = blockIdx.y * blockDim.x + threadIdx.x; t < total; t += gridDim.y * blockDim.x) {
        int i, j;
        if (t < ncol) {  // the ghost columns of the real rows
            i = t / (2 * GC);
            const int g = t - i * 2 * GC;
            j = g < GC ? g - GC : ny + g - GC;
        } else {  // the ghost rows, over the extended width
            const int u = t - ncol, rg = u / wide;
            j = u - rg * wide - GC;
            i = rg < GR ? rg - GR : nx + rg - GR;
        }
        const int si = ((i % nx) + nx) % nx, sj = ((j % ny) + ny) % ny;
        const long long d = (long long)i * pitch + j, s = (long long)si * pitch + sj;
        f0[d] = f0[s];
        f1[d] = f1[s];
    }
}

// The ghost words and rows of a wrapped scene's active plane: one thread per word of rows
// -BATCH_GHOST_ROWS..nx+BATCH_GHOST_ROWS-1, words -1..(ny+BATCH_GHOST_COLS-1)/32; a bit of a
// real cell keeps its value, a bit of a ghost cell takes the bit of the cell it wraps to.
__global__ void k_act_ghosts(uint32_t *act, int wpitch, int nx, int ny)
{
    constexpr int GC = BATCH_GHOST_COLS, GR = BATCH_GHOST_ROWS;
    const int w = (int)(blockIdx.x * blockDim.x + threadIdx.x) - 1;
    const int i = (int)blockIdx.y - GR;
    if (w > (ny + GC - 1) / 32 || i >= nx + GR) return;
    const bool real_row = i >= 0 && i < nx;
    if (real_row && w >= 0 && 32 * w + 31 < ny) return;  // all real cells
    const long long base = (long long)i * wpitch + w;
    uint32_t v = 0;
    for (int bit = 0; bit < 32; bit++) {
        const int j = 32 * w + bit;
        uint32_t x;
        if (real_row && j >= 0 && j < ny) {
            x = (act[base] >> bit) & 1u;
        } else if (j >= -GC && j < ny + GC) {
            const int si = ((i % nx) + nx) % nx, sj = ((j % ny) + ny) % ny;
            x = (act[(long long)si * wpitch + (sj >> 5)] >> (sj & 31)) & 1u;
        } else {
            x = 0;
        }
        v |= x << bit;
    }
    act[base] = v;
}

// skewed: the frame ran the skewed passes of the scenes with a depth class.  pairs: FP32
// scenes, whose single updates also alternate between the pairs.
__global__ void k_batch_advance(const BatchHdr *__restrict__ hdr, const SlotDev *__restrict__ tab,
                                SlotDyn *__restrict__ dyn, int n, int skewed, int pairs)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= hdr->nactive) return;
    SlotDyn &d = dyn[tab[k].slot];
    d.time += n;
    const int P = skewed ? batch_passes(n, tab[k].skew_k) : 0;
    if (P > 0) d.pair ^= P & 1;
    else if (pairs) d.pair ^= n & 1;
    else d.cur = (d.cur + n) & 1;
}

}  // namespace wg

using namespace wg;

namespace wg {

static void batch_drop_graphs(wg_batch *b);

BatchLayout batch_layout(const wg_params &p, int prec)
{
    BatchLayout L;
    const int esz = prec == WG_FP32 ? 4 : 8;
    if (batch_wrap_ok(p, prec)) {  // ghost columns, ghost rows, one ghost mask word per row
        L.pitch = pitch_for(p.ny + 2 * BATCH_GHOST_COLS + 64, esz);
        const size_t rows = (size_t)p.nx + 2 * BATCH_GHOST_ROWS, wpitch = (L.pitch + 31) / 32;
        L.field_bytes = rows * L.pitch * esz;
        L.mask_bytes = rows * wpitch * 4;
        L.field_off = (size_t)BATCH_GHOST_ROWS * L.pitch + BATCH_GHOST_COLS;
        L.mask_off = (size_t)BATCH_GHOST_ROWS * wpitch + 1;
    } else {
        L.pitch = pitch_for(p.ny, esz);
        const size_t wpitch = (L.pitch + 31) / 32;
        L.field_bytes = (size_t)p.nx * L.pitch * esz;
        L.mask_bytes = (size_t)p.nx * wpitch * 4;
        L.field_off = L.mask_off = 0;
    }
    return L;
}

static int entry_skew_k(const wg_batch *b, const BatchSlotHost &h)
{
    if (!h.skew || b->skew_mode == 0) return 0;
    return b->skew_mode > 0 ? b->skew_mode : b->class_k[h.cls];
}

// Tasks of the pass depth d for the scenes of depth class K (table entries), largest first
// so that the ticket order balances the warps.  Row chunks: the rows tuned for the scene's
// size class, or (untuned, fixed depth) sized from the whole list's work, about two tasks
// per resident warp (at least 32 rows), so that no single chunk outlasts the rest of the
// pass; the short top and bottom segments fill the end.  force_rows > 0 overrides both.
static void build_skew_tasks(const wg_batch *b, const std::vector<const BatchSlotHost *> &hs,
                             const std::vector<int> &entries, int d, std::vector<int4> &out, int force_rows = 0)
{
    const int F = 2 * d + 1;
    double rows = 0.0;
    for (const BatchSlotHost *h : hs) rows += (double)batch_skew_tiles(h->dp, d) * (h->prm.nx + 3 * F);
    const int cap = std::max(1, batch_skew_capacity(d));
    const int chunk = std::max(32, std::min(4096, (int)(rows / (2.0 * cap))));
    std::vector<int4> t;
    std::vector<float> cost;
    for (size_t k = 0; k < hs.size(); k++) {
        const int tuned = b->skew_mode < 0 ? b->class_rows[hs[k]->cls] : 0;
        batch_skew_plan(hs[k]->dp, entries[k], d, force_rows > 0 ? force_rows : (tuned > 0 ? tuned : chunk), t, cost);
    }
    std::vector<int> ord(t.size());
    for (size_t k = 0; k < ord.size(); k++) ord[k] = (int)k;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return cost[x] > cost[y]; });
    out.resize(t.size());
    for (size_t k = 0; k < ord.size(); k++) out[k] = t[ord[k]];
}

// (re)build the task list of (depth class K, pass depth d) from the current table
static wg_status build_list(wg_batch *b, int K, int d, const std::vector<int> &tab_slot)
{
    auto it = b->lists.find({K, d});
    if (it == b->lists.end()) {
        if ((int)b->lists.size() >= b->skew_n_cap - 1) { set_error("too many skewed task lists"); return WG_ERR_STATE; }
        BatchSkewList L;
        L.index = (int)b->lists.size();
        it = b->lists.emplace(std::make_pair(K, d), L).first;
    }
    BatchSkewList &L = it->second;
    std::vector<const BatchSlotHost *> hs;
    std::vector<int> entries;
    for (size_t e = 0; e < tab_slot.size(); e++) {
        const BatchSlotHost &h = b->slots[tab_slot[e]];
        if (entry_skew_k(b, h) == K) {
            hs.push_back(&h);
            entries.push_back((int)e);
        }
    }
    std::vector<int4> tasks;
    build_skew_tasks(b, hs, entries, d, tasks);
    if ((int)tasks.size() > L.cap) {
        if (L.dev) cudaFree(L.dev);
        L.dev = nullptr;
        const int cap = std::max(1024, (int)tasks.size() * 2);
        WG_CUDA(cudaMalloc(&L.dev, sizeof(int4) * cap));
        L.cap = cap;
        batch_drop_graphs(b);  // the graphs hold the list pointer
    }
    L.n = (int)tasks.size();
    if (L.n) WG_CUDA(cudaMemcpyAsync(L.dev, tasks.data(), sizeof(int4) * L.n, cudaMemcpyHostToDevice, b->st));
    WG_CUDA(cudaMemcpyAsync(b->d_skew_n + L.index, &L.n, sizeof(int), cudaMemcpyHostToDevice, b->st));
    WG_CUDA(cudaStreamSynchronize(b->st));  // the host vectors above go out of scope
    return WG_OK;
}

wg_status batch_refresh_table(wg_batch *b)
{
    constexpr int Vf = 4, Vd = 2;
    const int V = (b->prec == WG_FP32) ? Vf : Vd;
    std::vector<SlotDev> tab;
    std::vector<int> tab_slot;
    std::vector<int4> items;
    int base = 0, plain = 0, nskew = 0, nwrap = 0;
    long long cells = 0;
    unsigned sig = 0;
    // scenes without skewed passes first: their items are the first plain_tiles
    for (int pass = 0; pass < 2; pass++) {
        for (int k = 0; k < (int)b->slots.size(); k++) {
            const BatchSlotHost &h = b->slots[k];
            if (!h.used) continue;
            const int sk = entry_skew_k(b, h);
            if ((sk > 0) != (pass == 1)) continue;
            SlotDev d;
            memset(&d, 0, sizeof d);
            d.p = h.dp;
            for (int q = 0; q < 4; q++) d.f[q] = h.f[q];
            d.act = h.act;
            d.nz = h.nz;
            d.slot = k;
            {
                const double c[12] = {h.dp.c2, h.dp.c2b, h.dp.gam, h.dp.gamb, h.dp.kappa, h.dp.kappa_sides,
                                      h.dp.kappa_topbot, h.dp.gamma_sides, h.dp.gamma_topbot, h.dp.vmax,
                                      h.dp.courant, h.dp.courantb};
                for (int q = 0; q < 12; q++) d.cf[q] = (float)c[q];
            }
            d.skew_k = sk;
            d.wrap = h.wrap ? 1 : 0;
            d.tiles_j = (h.dp.pitch / V + BT_THREADS - 1) / BT_THREADS;
            const int tiles_i = (h.prm.nx + BT_ROWS - 1) / BT_ROWS;
            d.ntiles = tiles_i * d.tiles_j;
            d.tile_base = base;
            base += d.ntiles;
            for (int ti = 0; ti < tiles_i; ti++)
                for (int tj = 0; tj < d.tiles_j; tj++) items.push_back(make_int4((int)tab.size(), ti * BT_ROWS, tj, k));
            cells += (long long)h.prm.nx * h.prm.ny;
            if (sk > 0) {
                sig |= 1u << sk;
                nskew++;
                if (h.wrap) nwrap++;
            } else {
                plain = base;
            }
            tab.push_back(d);
            tab_slot.push_back(k);
        }
    }
    if (plain > 0) sig |= 1u;
    if (nwrap > 0) sig |= 1u << 8;  // ghost refreshes in the branches
    if ((int)tab.size() > b->tab_cap) {
        if (b->d_tab) cudaFree(b->d_tab);
        b->d_tab = nullptr;
        const int cap = std::max(64, (int)tab.size() * 2);
        WG_CUDA(cudaMalloc(&b->d_tab, sizeof(SlotDev) * cap));
        b->tab_cap = cap;
        batch_drop_graphs(b);  // the graphs hold the table pointer and size the advance launch by it
    }
    if ((int)items.size() > b->items_cap) {
        if (b->d_items) cudaFree(b->d_items);
        b->d_items = nullptr;
        const int cap = std::max(1024, (int)items.size() * 2);
        WG_CUDA(cudaMalloc(&b->d_items, sizeof(int4) * cap));
        b->items_cap = cap;
        batch_drop_graphs(b);  // the graphs hold the item-table pointer
    }
    if (sig != b->graph_sig) {  // another set of branches: the graphs are recorded again
        batch_drop_graphs(b);
        b->graph_sig = sig;
    }
    if (!tab.empty()) {
        WG_CUDA(cudaMemcpyAsync(b->d_tab, tab.data(), sizeof(SlotDev) * tab.size(), cudaMemcpyHostToDevice, b->st));
        WG_CUDA(cudaMemcpyAsync(b->d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, b->st));
    }
    BatchHdr h{(int)tab.size(), base, plain, 0};
    WG_CUDA(cudaMemcpyAsync(b->d_hdr, &h, sizeof h, cudaMemcpyHostToDevice, b->st));
    WG_CUDA(cudaStreamSynchronize(b->st));
    b->nactive = (int)tab.size();
    b->total_cells = cells;
    b->plain_tiles = plain;
    b->skew_scenes = nskew;
    b->wrap_scenes = nwrap;
    b->tab_slot = tab_slot;
    // the task lists in use follow the new table
    std::vector<std::pair<int, int>> keys;
    for (auto &kv : b->lists) keys.push_back(kv.first);
    for (auto &key : keys) {
        wg_status st = build_list(b, key.first, key.second, tab_slot);
        if (st) return st;
    }
    return WG_OK;
}

static void batch_drop_graphs(wg_batch *b)
{
    for (auto &g : b->graphs) cudaGraphExecDestroy(g.second);
    b->graphs.clear();
}

// depth classes present in the table (bits 2..6 of graph_sig)
static std::vector<int> batch_groups(const wg_batch *b)
{
    std::vector<int> g;
    for (int K = 2; K <= WG_SKEW_MAX_K; K++)
        if (b->graph_sig & (1u << K)) g.push_back(K);
    return g;
}

// Everything a frame of n updates needs before it is recorded: counters, tickets, the
// task lists of its passes, the branches' streams and events, the kernels' attributes.
static wg_status batch_prepare_frame(wg_batch *b, int n, bool skewed)
{
    if (n > b->counter_cap) {
        if (b->d_counter) cudaFree(b->d_counter);
        b->d_counter = nullptr;
        WG_CUDA(cudaMalloc(&b->d_counter, sizeof(int) * n));
        b->counter_cap = n;
        batch_drop_graphs(b);
    }
    if (!skewed) return WG_OK;
    int tickets = 0;
    for (int K : batch_groups(b)) {
        const int P = batch_passes(n, K);
        tickets += P;
        for (int q = 0; q < P; q++) {
            const int d = batch_pass_depth(n, P, q);
            batch_skew_capacity(d);  // sets the kernel's shared-memory attribute outside the capture
            if (!b->lists.count({K, d})) {
                wg_status st = build_list(b, K, d, b->tab_slot);
                if (st) return st;
            }
        }
    }
    if (tickets > b->ticket_cap) {
        if (b->d_ticket) cudaFree(b->d_ticket);
        b->d_ticket = nullptr;
        const int cap = std::max(64, tickets * 2);
        WG_CUDA(cudaMalloc(&b->d_ticket, sizeof(int) * cap));
        b->ticket_cap = cap;
        batch_drop_graphs(b);
    }
    for (int K : batch_groups(b)) {
        if (!b->side[K]) WG_CUDA(cudaStreamCreateWithFlags(&b->side[K], cudaStreamNonBlocking));
        if (!b->ev_join[K]) WG_CUDA(cudaEventCreateWithFlags(&b->ev_join[K], cudaEventDisableTiming));
    }
    if (!b->ev_fork) WG_CUDA(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
    return WG_OK;
}

template <class T>
static void batch_enqueue_frame(wg_batch *b, int n, bool skewed)
{
    cudaMemsetAsync(b->d_counter, 0, sizeof(int) * n, b->st);
    std::vector<int> groups;
    if (skewed) {
        groups = batch_groups(b);
        int tickets = 0;
        for (int K : groups) tickets += batch_passes(n, K);
        cudaMemsetAsync(b->d_ticket, 0, sizeof(int) * tickets, b->st);
        cudaEventRecord(b->ev_fork, b->st);
        int ti = 0;
        for (int K : groups) {  // one branch per depth class
            cudaStream_t ss = b->side[K];
            cudaStreamWaitEvent(ss, b->ev_fork, 0);
            const int P = batch_passes(n, K);
            int toff = 0;
            for (int q = 0; q < P; q++) {
                const int d = batch_pass_depth(n, P, q);
                const BatchSkewList &L = b->lists.at({K, d});
                if (b->graph_sig & (1u << 8))  // the wrapped scenes' ghosts of this pass's input pair
                    k_batch_ghosts<<<dim3(std::max(b->tab_cap, 1), 8), 256, 0, ss>>>(b->d_hdr, b->d_tab, b->d_dyn, K, q);
                launch_batch_skew(d, b->d_tab, b->d_dyn, L.dev, b->d_skew_n + L.index, b->d_ticket + ti++, q, toff, ss);
                toff += d;
            }
            cudaEventRecord(b->ev_join[K], ss);
        }
    }
    if (!skewed || (b->graph_sig & 1u)) {  // the chain of single updates
        dim3 blk(BT_THREADS, 4);
        for (int u = 0; u < n; u++)
            launch_pdl(k_batch_step<T>, dim3(b->persistent_blocks), blk, 0, b->st, (const BatchHdr *)b->d_hdr,
                       (const SlotDev *)b->d_tab, (const int4 *)b->d_items, b->d_dyn, b->d_counter, u, skewed ? 0 : 1);
    }
    for (int K : groups) cudaStreamWaitEvent(b->st, b->ev_join[K], 0);
    const int cap = std::max(b->tab_cap, 1);
    k_batch_advance<<<(cap + 255) / 256, 256, 0, b->st>>>(b->d_hdr, b->d_tab, b->d_dyn, n, skewed ? 1 : 0,
                                                          sizeof(T) == 4 ? 1 : 0);
}

// Depth and row chunk per size class, in two stages: depths 2..4 with the list-wide
// chunk, then chunks of 32, 64, 128 and 256 rows at the best depth.  Each candidate
// times one skewed pass over the class's scenes (reading their current fields, writing
// the other pair, so the state does not change), best of five after one untimed pass;
// the fastest per update is kept.  Seven candidates per class keep the tuning frame of a
// server tick short.
// Tuned classes are kept for the process, keyed by device, size class and the kinds of
// scene in the class (their boundary conditions, the ghost layout, two speeds): a later
// batch or server whose class holds the same kinds takes that depth and chunk without
// timing them again, so a serving tick pays the tuning of a size class at most once per
// process.  (Keyed by size class alone, the sweep's absorbing scenes took the depth tuned
// for the uneven batch's mirror and periodic ones: 309 against 351 Gcell/s.)
struct TuneCacheEntry {
    int k = 0, rows = 0;
    double ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, unsigned>, TuneCacheEntry> g_tune_cache;  // (device, class, kinds)

static unsigned class_kinds(const wg_batch *b, int c)
{
    unsigned sig = 0;
    for (size_t e = 0; e < b->tab_slot.size(); e++) {
        const BatchSlotHost &h = b->slots[b->tab_slot[e]];
        if (!(h.skew && h.cls == c)) continue;
        sig |= 1u << (h.prm.b_cond & 7);
        if (h.wrap) sig |= 1u << 8;
        if (h.prm.twospeeds) sig |= 1u << 9;
        if (h.prm.oscillate_left || h.prm.oscillate_topbot) sig |= 1u << 10;
        if (h.prm.src_on) sig |= 1u << 11;
    }
    return sig;
}

static wg_status batch_autotune(wg_batch *b)
{
    bool tuned = false, ghosts = false;
    int devno = 0;
    WG_CUDA(cudaGetDevice(&devno));
    for (int c = 0; c < BATCH_CLASSES; c++) {
        if (b->class_k[c]) continue;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            const unsigned kinds = class_kinds(b, c);
            if (!kinds) continue;  // no scene of this class takes skewed passes
            auto it = g_tune_cache.find(std::make_tuple(devno, c, kinds));
            if (it != g_tune_cache.end()) {
                if (b->tune_ms.empty()) b->tune_ms.assign(BATCH_CLASSES * 8, 0.0);
                b->class_k[c] = it->second.k;
                b->class_rows[c] = it->second.rows;
                for (int K = 0; K < 8; K++) b->tune_ms[c * 8 + K] = it->second.ms[K];
                tuned = true;
                continue;
            }
        }
        std::vector<const BatchSlotHost *> hs;
        std::vector<int> entries;
        for (size_t e = 0; e < b->tab_slot.size(); e++) {
            const BatchSlotHost &h = b->slots[b->tab_slot[e]];
            if (h.skew && h.cls == c) {
                hs.push_back(&h);
                entries.push_back((int)e);
            }
        }
        if (hs.empty()) continue;
        if (b->tune_ms.empty()) b->tune_ms.assign(BATCH_CLASSES * 8, 0.0);
        if (!ghosts) {  // the wrapped scenes' ghosts of their current pair, read by the timed passes
            k_batch_ghosts<<<dim3(std::max(b->nactive, 1), 8), 256, 0, b->st>>>(b->d_hdr, b->d_tab, b->d_dyn, -1, 0);
            b->launches++;
            ghosts = true;
        }
        cudaEvent_t ev[6];
        for (int q = 0; q < 6; q++) WG_CUDA(cudaEventCreate(&ev[q]));
        int best = 0, best_rows = 0;
        double best_ms = 1e30;
        int4 *dev = nullptr;
        cudaError_t err = cudaSuccess;
        static const int ROWS[] = {32, 64, 128, 256};
        // depths 2..4: at 5 and 6 the velocity rows push the pass past its 128 registers
        // (spills) and those depths measured slower on every size class tried
        const int ndepth = 3;
        for (int cand = 0; cand < ndepth + 4 && err == cudaSuccess; cand++) {
            const int K = cand < ndepth ? 2 + cand : best, R = cand < ndepth ? 0 : ROWS[cand - ndepth];
            std::vector<int4> tasks;
            build_skew_tasks(b, hs, entries, K, tasks, R);
            const int nt = (int)tasks.size();
            err = cudaMallocAsync((void **)&dev, sizeof(int4) * std::max(nt, 1), b->st);
            if (err == cudaSuccess && nt) err = cudaMemcpyAsync(dev, tasks.data(), sizeof(int4) * nt, cudaMemcpyHostToDevice, b->st);
            const int idx = b->skew_n_cap - 1;  // the count slot kept for tuning
            if (err == cudaSuccess) err = cudaMemcpyAsync(b->d_skew_n + idx, &nt, sizeof(int), cudaMemcpyHostToDevice, b->st);
            const int reps = 5;  // one untimed pass, then the best of five
            for (int r = 0; r <= reps && err == cudaSuccess; r++) {
                cudaMemsetAsync(b->d_tune_ticket + r, 0, sizeof(int), b->st);
                launch_batch_skew(K, b->d_tab, b->d_dyn, dev, b->d_skew_n + idx, b->d_tune_ticket + r, 0, 0, b->st);
                b->launches++;
                err = cudaGetLastError();
                if (err == cudaSuccess) err = cudaEventRecord(ev[r], b->st);
            }
            if (err == cudaSuccess) err = cudaEventSynchronize(ev[reps]);
            float ms = 1e30f;
            for (int r = 1; r <= reps && err == cudaSuccess; r++) {
                float t = 0.f;
                err = cudaEventElapsedTime(&t, ev[r - 1], ev[r]);
                ms = std::min(ms, t);
            }
            if (dev) cudaFreeAsync(dev, b->st);
            dev = nullptr;
            if (err == cudaSuccess) err = cudaStreamSynchronize(b->st);  // tasks outlives its copy
            const double per = ms / K;
            if (R == 0 || per < b->tune_ms[c * 8 + K]) b->tune_ms[c * 8 + K] = per;
            if (per < best_ms) {
                best_ms = per;
                best = K;
                best_rows = R;
            }
        }
        for (int q = 0; q < 6; q++) cudaEventDestroy(ev[q]);
        if (err != cudaSuccess) return cuda_fail(err, "batch autotune");
        b->class_k[c] = best;
        b->class_rows[c] = best_rows;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            TuneCacheEntry &ce = g_tune_cache[std::make_tuple(devno, c, class_kinds(b, c))];
            ce.k = best;
            ce.rows = best_rows;
            for (int K = 0; K < 8; K++) ce.ms[K] = b->tune_ms[c * 8 + K];
        }
        tuned = true;
    }
    if (tuned) return batch_refresh_table(b);
    return WG_OK;
}

}  // namespace wg

extern "C" {

wg_status wg_batch_create(int32_t precision, void *stream, wg_batch **out)
{
    if (!out) { set_error("NULL argument"); return WG_ERR_INVALID; }
    if (precision != WG_FP32 && precision != WG_FP64) { set_error("precision must be WG_FP32 or WG_FP64"); return WG_ERR_INVALID; }
    wg_batch *b = new wg_batch();
    b->prec = precision;
    b->esz = precision == WG_FP32 ? 4 : 8;
    cudaError_t e = cudaSuccess;
    if (stream) b->st = (cudaStream_t)stream;
    else {
        e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
        b->own_stream = true;
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->d_hdr, sizeof(BatchHdr));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_hdr, 0, sizeof(BatchHdr), b->st);
    int dev = 0, sms = 0, per = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = (precision == WG_FP32)
                ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_step<float>, BT_THREADS * 4, 0)
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_step<double>, BT_THREADS * 4, 0);
    if (e == cudaSuccess) e = cudaHostAlloc(&b->h_out, 16 * sizeof(double), cudaHostAllocDefault);
    b->skew_n_cap = 32;
    if (e == cudaSuccess) e = cudaMalloc(&b->d_skew_n, sizeof(int) * b->skew_n_cap);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_skew_n, 0, sizeof(int) * b->skew_n_cap, b->st);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_tune_ticket, sizeof(int) * 8);
    if (e != cudaSuccess) {
        wg_status r = cuda_fail(e, "wg_batch_create");
        wg_batch_destroy(b);
        return r;
    }
    b->persistent_blocks = std::max(1, sms * std::max(per, 1));
    *out = b;
    return WG_OK;
}

wg_status wg_batch_destroy(wg_batch *b)
{
    if (!b) return WG_OK;
    if (b->st) cudaStreamSynchronize(b->st);
    batch_drop_graphs(b);
    for (auto &h : b->slots) {
        if (!h.used) continue;
        void *ptrs[] = {h.mem[0], h.mem[1], h.mem[2], h.mem[3], h.act_mem, h.nz_mem, h.ebot, h.etop, h.eout};
        for (void *p : ptrs) if (p) cudaFree(p);
    }
    for (auto &kv : b->lists) if (kv.second.dev) cudaFree(kv.second.dev);
    void *ptrs[] = {b->d_tab, b->d_dyn, b->d_hdr, b->d_counter, b->d_items, b->d_skew_n, b->d_ticket, b->d_tune_ticket};
    for (void *p : ptrs) if (p) cudaFree(p);
    for (int k = 0; k < BATCH_GROUPS; k++) {
        if (b->side[k]) cudaStreamDestroy(b->side[k]);
        if (b->ev_join[k]) cudaEventDestroy(b->ev_join[k]);
    }
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->h_out) cudaFreeHost(b->h_out);
    if (b->own_stream && b->st) cudaStreamDestroy(b->st);
    delete b;
    return WG_OK;
}

wg_status wg_batch_add(wg_batch *b, const wg_params *p, const double *phi, const double *psi, const int16_t *xy,
                       int32_t *slot)
{
    if (!b || !p || !phi || !psi || !xy || !slot) { set_error("NULL argument"); return WG_ERR_INVALID; }
    wg_status st = validate_params(*p);
    if (st) return st;
    if (p->bc_neumann) { set_error("batches do not take Neumann records; use a scene"); return WG_ERR_INVALID; }
    const size_t n = (size_t)p->nx * p->ny;
    for (size_t c = 0; c < n; c++)
        if (xy[c] != 0 && xy[c] != 1) { set_error("batch masks take values 0/1"); return WG_ERR_INVALID; }
    int k = 0;
    while (k < (int)b->slots.size() && b->slots[k].used) k++;
    if (k == (int)b->slots.size()) b->slots.emplace_back();
    BatchSlotHost &h = b->slots[k];
    h = BatchSlotHost();
    h.prm = *p;
    h.skew = batch_skew_ok(*p, b->prec);
    h.wrap = batch_wrap_ok(*p, b->prec);
    const BatchLayout L = batch_layout(*p, b->prec);
    const int pitch = L.pitch;
    h.dp = make_dev_params(*p, pitch);
    {
        const double cells = (double)p->nx * p->ny;
        h.cls = std::min(BATCH_CLASSES - 1, std::max(0, (int)std::floor(std::log2(cells)) - 10));
    }
    const size_t fb = L.field_bytes, mb = L.mask_bytes;
    cudaError_t e = cudaSuccess;
    const int nf = b->prec == WG_FP32 ? 4 : 2;  // FP32: the second pair takes every update's output
    for (int q = 0; q < nf && e == cudaSuccess; q++) e = cudaMallocAsync(&h.mem[q], fb, b->st);
    for (int q = (h.wrap ? 0 : 2); q < nf && e == cudaSuccess; q++) e = cudaMemsetAsync(h.mem[q], 0, fb, b->st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&h.act_mem, mb, b->st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&h.nz_mem, mb, b->st);
    if (e == cudaSuccess && h.wrap) e = cudaMemsetAsync(h.act_mem, 0, mb, b->st);
    for (int q = 0; q < nf; q++) h.f[q] = h.mem[q] ? (char *)h.mem[q] + L.field_off * b->esz : nullptr;
    h.act = h.act_mem ? h.act_mem + L.mask_off : nullptr;
    h.nz = h.nz_mem ? h.nz_mem + L.mask_off : nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&h.ebot, p->nx * sizeof(double2), b->st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&h.etop, p->nx * sizeof(double2), b->st);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&h.eout, (p->nx + 8) * sizeof(double), b->st);
    void *stage = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync(&stage, 2 * n * sizeof(double), b->st);
    if (e != cudaSuccess) {
        void *ptrs[] = {h.mem[0], h.mem[1], h.mem[2], h.mem[3], h.act_mem, h.nz_mem, h.ebot, h.etop, h.eout, stage};
        for (void *q : ptrs) if (q) cudaFreeAsync(q, b->st);
        h = BatchSlotHost();
        return cuda_fail(e, "wg_batch_add");
    }
    h.bytes = nf * fb + 2 * mb;
    // mask planes, then the two fields (FP64 host values rounded on the device)
    WG_CUDA(cudaMemcpyAsync(stage, xy, n * sizeof(int16_t), cudaMemcpyHostToDevice, b->st));
    launch_pack_mask(p->nx, p->ny, h.dp.wpitch, (const int16_t *)stage, h.act, h.nz, b->st);
    if (h.wrap) {  // the mask's ghost words and rows, once (the mask does not change)
        const int words = (p->ny + BATCH_GHOST_COLS + 31) / 32 + 1, rows = p->nx + 2 * BATCH_GHOST_ROWS;
        k_act_ghosts<<<dim3((words + 63) / 64, rows), 64, 0, b->st>>>(h.act, h.dp.wpitch, p->nx, p->ny);
        b->launches++;
    }
    double *dstage = (double *)stage;
    WG_CUDA(cudaMemcpyAsync(dstage, phi, n * sizeof(double), cudaMemcpyHostToDevice, b->st));
    WG_CUDA(cudaMemcpyAsync(dstage + n, psi, n * sizeof(double), cudaMemcpyHostToDevice, b->st));
    if (b->prec == WG_FP32) {  // phi and the velocity phi - psi
        launch_state_in32<double>(p->nx, p->ny, pitch, dstage, dstage + n, (float *)h.f[0], (float *)h.f[1], b->st);
    } else {
        launch_convert_in<double>(p->nx, p->ny, pitch, dstage, (double *)h.f[0], b->st);
        launch_convert_in<double>(p->nx, p->ny, pitch, dstage + n, (double *)h.f[1], b->st);
    }
    WG_CUDA(cudaFreeAsync(stage, b->st));
    WG_CUDA(cudaGetLastError());
    // dynamic state: time 0, phi in f[0]
    if (k >= b->dyn_cap) {
        const int cap = std::max(64, 2 * (k + 1));
        SlotDyn *nd = nullptr;
        WG_CUDA(cudaMalloc(&nd, sizeof(SlotDyn) * cap));
        WG_CUDA(cudaMemsetAsync(nd, 0, sizeof(SlotDyn) * cap, b->st));
        if (b->d_dyn) {
            WG_CUDA(cudaMemcpyAsync(nd, b->d_dyn, sizeof(SlotDyn) * b->dyn_cap, cudaMemcpyDeviceToDevice, b->st));
            WG_CUDA(cudaStreamSynchronize(b->st));
            cudaFree(b->d_dyn);
        }
        b->d_dyn = nd;
        b->dyn_cap = cap;
        batch_drop_graphs(b);
    }
    SlotDyn zero{0, 0, 0};
    WG_CUDA(cudaMemcpyAsync(b->d_dyn + k, &zero, sizeof zero, cudaMemcpyHostToDevice, b->st));
    h.used = true;
    const int old_cap = b->tab_cap;
    if ((st = batch_refresh_table(b))) return st;
    if (b->tab_cap != old_cap) batch_drop_graphs(b);
    *slot = k;
    return WG_OK;
}

wg_status wg_batch_remove(wg_batch *b, int32_t slot)
{
    if (!b || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used) {
        set_error("unknown batch slot %d", slot);
        return WG_ERR_NOTFOUND;
    }
    BatchSlotHost &h = b->slots[slot];
    h.used = false;
    wg_status st = batch_refresh_table(b);  // the kernels stop seeing the slot first
    void *ptrs[] = {h.mem[0], h.mem[1], h.mem[2], h.mem[3], h.act_mem, h.nz_mem, h.ebot, h.etop, h.eout};
    for (void *p : ptrs) if (p) WG_CUDA(cudaFreeAsync(p, b->st));
    h = BatchSlotHost();
    return st;
}

wg_status wg_batch_step(wg_batch *b, int32_t nsteps)
{
    if (!b || nsteps < 0) { set_error("bad arguments"); return WG_ERR_INVALID; }
    if (nsteps == 0 || b->nactive == 0) return WG_OK;
    wg_status st;
    if (b->prec == WG_FP32 && b->skew_mode < 0 && nsteps >= 2 && (st = batch_autotune(b))) return st;
    const bool skewed = b->prec == WG_FP32 && nsteps >= 2 && b->skew_scenes > 0;
    if ((st = batch_prepare_frame(b, nsteps, skewed))) return st;
    auto it = b->graphs.find(nsteps);
    if (it == b->graphs.end()) {
        cudaGraph_t g;
        WG_CUDA(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
        if (b->prec == WG_FP32) batch_enqueue_frame<float>(b, nsteps, skewed);
        else batch_enqueue_frame<double>(b, nsteps, skewed);
        WG_CUDA(cudaStreamEndCapture(b->st, &g));
        cudaGraphExec_t ge;
        cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        it = b->graphs.emplace(nsteps, ge).first;
    }
    WG_CUDA(cudaGraphLaunch(it->second, b->st));
    long long n = 1;  // the advance kernel
    if (!skewed || (b->graph_sig & 1u)) n += nsteps;
    if (skewed)
        for (int K : batch_groups(b)) n += batch_passes(nsteps, K) * ((b->graph_sig & (1u << 8)) ? 2 : 1);
    b->launches += n;
    return WG_OK;
}

wg_status wg_batch_set_skew(wg_batch *b, int32_t mode)
{
    if (!b) { set_error("NULL batch"); return WG_ERR_INVALID; }
    if (!(mode == -1 || mode == 0 || (mode >= 2 && mode <= WG_SKEW_MAX_K))) {
        set_error("skewed depth %d: -1 (tuned per size class), 0 (off) or 2..%d", mode, WG_SKEW_MAX_K);
        return WG_ERR_INVALID;
    }
    WG_CUDA(cudaStreamSynchronize(b->st));
    b->skew_mode = mode;
    batch_drop_graphs(b);
    return batch_refresh_table(b);
}

wg_status wg_batch_skew_depths(wg_batch *b, int32_t *depths, int32_t *chunk_rows, double *ms_per_update)
{
    if (!b || !depths) { set_error("NULL argument"); return WG_ERR_INVALID; }
    for (int c = 0; c < BATCH_CLASSES; c++) {
        depths[c] = b->skew_mode >= 0 ? b->skew_mode : b->class_k[c];
        if (chunk_rows) chunk_rows[c] = b->skew_mode >= 0 ? 0 : b->class_rows[c];
        if (ms_per_update)
            for (int K = 0; K < 8; K++)
                ms_per_update[c * 8 + K] = b->tune_ms.empty() ? 0.0 : b->tune_ms[c * 8 + K];
    }
    return WG_OK;
}

wg_status wg_batch_download(wg_batch *b, int32_t slot, double *phi, double *psi)
{
    if (!b || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used) {
        set_error("unknown batch slot %d", slot);
        return WG_ERR_NOTFOUND;
    }
    BatchSlotHost &h = b->slots[slot];
    SlotDyn d;
    WG_CUDA(cudaMemcpyAsync(&d, b->d_dyn + slot, sizeof d, cudaMemcpyDeviceToHost, b->st));
    WG_CUDA(cudaStreamSynchronize(b->st));
    const size_t n = (size_t)h.prm.nx * h.prm.ny;
    double *stage = nullptr;
    WG_CUDA(cudaMallocAsync((void **)&stage, 2 * n * sizeof(double), b->st));
    if (b->prec == WG_FP32) {  // phi, and psi = phi - v
        launch_state_out32<double>(h.prm.nx, h.prm.ny, h.dp.pitch, (const float *)h.f[2 * d.pair],
                                   (const float *)h.f[2 * d.pair + 1], phi ? stage : nullptr, psi ? stage + n : nullptr,
                                   b->st);
    } else {
        if (phi) launch_convert_out<double>(h.prm.nx, h.prm.ny, h.dp.pitch, (const double *)h.f[d.cur], stage, b->st);
        if (psi) launch_convert_out<double>(h.prm.nx, h.prm.ny, h.dp.pitch, (const double *)h.f[1 - d.cur], stage + n, b->st);
    }
    if (phi) WG_CUDA(cudaMemcpyAsync(phi, stage, n * sizeof(double), cudaMemcpyDeviceToHost, b->st));
    if (psi) WG_CUDA(cudaMemcpyAsync(psi, stage + n, n * sizeof(double), cudaMemcpyDeviceToHost, b->st));
    WG_CUDA(cudaFreeAsync(stage, b->st));
    WG_CUDA(cudaStreamSynchronize(b->st));
    return WG_OK;
}

wg_status wg_batch_energy(wg_batch *b, int32_t slot, double *total)
{
    if (!b || !total || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used) {
        set_error("unknown batch slot %d", slot);
        return WG_ERR_NOTFOUND;
    }
    BatchSlotHost &h = b->slots[slot];
    SlotDyn d;
    WG_CUDA(cudaMemcpyAsync(&d, b->d_dyn + slot, sizeof d, cudaMemcpyDeviceToHost, b->st));
    WG_CUDA(cudaStreamSynchronize(b->st));
    // FP32: phi and the velocity of the current pair; FP64: phi and psi of pair 0
    const void *phi = h.f[2 * d.pair + d.cur], *psi = h.f[2 * d.pair + 1 - d.cur];
    if (b->prec == WG_FP32)
        launch_energy<float>(h.dp, (const float *)phi, (const float *)psi, nullptr, h.nz, h.ebot, h.etop, 0, 0, h.eout, b->st);
    else
        launch_energy<double>(h.dp, (const double *)phi, (const double *)psi, nullptr, h.nz, h.ebot, h.etop, 0, 0, h.eout, b->st);
    b->launches += 2;
    WG_CUDA(cudaGetLastError());
    WG_CUDA(cudaMemcpyAsync(b->h_out, h.eout, sizeof(double), cudaMemcpyDeviceToHost, b->st));
    WG_CUDA(cudaStreamSynchronize(b->st));
    *total = b->h_out[0];
    return WG_OK;
}

wg_status wg_batch_count(wg_batch *b, int32_t *n_active, int64_t *cells)
{
    if (!b) return WG_ERR_INVALID;
    if (n_active) *n_active = b->nactive;
    if (cells) *cells = b->total_cells;
    return WG_OK;
}

wg_status wg_batch_launch_count(wg_batch *b, int64_t *n)
{
    if (!b || !n) return WG_ERR_INVALID;
    *n = b->launches;
    return WG_OK;
}

}  // extern "C"
