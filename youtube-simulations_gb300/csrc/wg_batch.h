// wg_batch.h — batch engine objects shared by wg_batch.cu and wg_serve.cu.
#pragma once
#include <map>
#include <vector>
#include "wg_internal.h"
#include "wg_scene.h"

namespace wg {

constexpr int BT_ROWS = 32;      // rows of one work item
constexpr int BT_THREADS = 64;   // threads along j per tile row (x V cells)

struct __align__(16) SlotDev {   // one entry of the compact table of active scenes
    DevParams p;
    void *f[4];                  // pair 0: f[0], f[1]; pair 1 (FP32 scenes): f[2], f[3]
    uint32_t *act, *nz;
    int slot;                    // index into the per-slot dynamic state
    int tiles_j, tile_base, ntiles;
    int skew_k;                  // depth class of the scene's skewed passes; 0: single updates only
    int wrap;                    // periodic scene in the ghost layout (skewed passes read wrapped halos)
    int pad_[2];
    // the coefficients rounded to FP32 once on the host (a conversion from FP64 costs the
    // FP64 pipe on the device): c2, c2b, gam, gamb, kappa, kappa_sides, kappa_topbot,
    // gamma_sides, gamma_topbot, vmax, courant, courantb
    float cf[12];
};
enum { CF_C2, CF_C2B, CF_GAM, CF_GAMB, CF_KAPPA, CF_KS, CF_KT, CF_GS, CF_GT, CF_VMAX, CF_COURANT, CF_COURANTB };
struct SlotDyn {
    long long time;
    int cur;                     // FP64: phi = f[cur], psi = f[1 - cur]
    int pair;                    // FP32: phi = f[2 pair], velocity = f[2 pair + 1]
};
struct BatchHdr {
    int nactive, total_tiles;    // all work items
    int plain_tiles, pad_;       // items of the scenes without skewed passes (they come first)
};

constexpr int BATCH_CLASSES = 16;   // size classes: floor(log2(cells)) - 10, clamped to 0..15

// Ghost layout of a periodic scene taking skewed passes: every field row carries
// BATCH_GHOST_COLS copies of the opposite side's columns on each side, and the field
// BATCH_GHOST_ROWS copies of the opposite rows above row 0 and below row nx-1, so that a
// pass reads its wrapped halo as ordinary neighbours.  The scene's pointers address cell
// (0, 0); the ghosts sit at negative offsets and in the row padding.  Mask planes carry one
// ghost word on the left of every row and the same ghost rows.
constexpr int BATCH_GHOST_COLS = 8;   // the widest column halo of a pass (depth 5..6)
constexpr int BATCH_GHOST_ROWS = 7;   // the deepest row halo of a pass (depth 6 + 1)
constexpr int BATCH_GROUPS = WG_SKEW_MAX_K + 1;

// Skewed passes of a frame of n updates with depth class K: P passes of n/P or n/P+1
// updates (2..6 each); 0 when n < 2.
__host__ __device__ inline int batch_passes(int n, int K)
{
    if (K < 2 || n < 2) return 0;
    int P = (n + K - 1) / K;
    if (n < 2 * P) P = n / 2;
    return P;
}
__host__ __device__ inline int batch_pass_depth(int n, int P, int q) { return n / P + (q < n % P ? 1 : 0); }

// Skewed passes over many scenes (wg_tb.cu): persistent warps take tasks (table entry,
// first column of the 128-column tile, rows i_s | i_e << 16, kind) from a ticket counter;
// pass q of a frame reads the pair the previous pass wrote, toff updates after the frame start.
int batch_skew_capacity(int K);
int batch_skew_tiles(const DevParams &p, int K);  // column tiles of a scene (shifted tiling)
// tasks of one scene, inner row chunks of rows..2*rows rows
void batch_skew_plan(const DevParams &p, int entry, int K, int rows, std::vector<int4> &tasks, std::vector<float> &cost);
void launch_batch_skew(int K, const SlotDev *tab, const SlotDyn *dyn, const int4 *tasks, const int *ntasks, int *ticket,
                       int q, int toff, cudaStream_t st);
bool batch_skew_ok(const wg_params &p, int prec);
bool batch_wrap_ok(const wg_params &p, int prec);   // periodic scenes the skewed passes take (ghost layout)

wg_status batch_refresh_table(::wg_batch *b);

struct BatchLayout {            // device layout of one batch scene
    int pitch;                  // elements per field row
    size_t field_bytes, mask_bytes;  // one field, one mask plane
    size_t field_off, mask_off;      // cell (0, 0) within the allocation (elements, words)
};
BatchLayout batch_layout(const wg_params &p, int prec);

}  // namespace wg

struct BatchSlotHost {
    bool used = false;
    wg_params prm;
    wg::DevParams dp;
    void *f[4] = {nullptr, nullptr, nullptr, nullptr};  // f[2], f[3]: second pair of FP32 scenes
    void *mem[4] = {nullptr, nullptr, nullptr, nullptr};  // the allocations behind f (ghost layout: f is inside)
    uint32_t *act_mem = nullptr, *nz_mem = nullptr;
    uint32_t *act = nullptr, *nz = nullptr;
    double2 *ebot = nullptr, *etop = nullptr;
    double *eout = nullptr;
    size_t bytes = 0;
    bool skew = false;      // FP32 scene whose boundaries the skewed passes cover
    bool wrap = false;      // periodic, in the ghost layout
    int cls = 0;            // size class
};

struct BatchSkewList {      // tasks of one pass depth for one depth class
    int4 *dev = nullptr;
    int cap = 0, n = 0, index = 0;  // index: its count in d_skew_n
};

struct wg_batch {
    int prec = WG_FP32;
    size_t esz = 4;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    std::vector<BatchSlotHost> slots;
    wg::SlotDev *d_tab = nullptr;
    int tab_cap = 0;
    wg::SlotDyn *d_dyn = nullptr;
    int dyn_cap = 0;
    wg::BatchHdr *d_hdr = nullptr;
    int4 *d_items = nullptr;                // (table entry, first row, column tile, slot) per work item
    int items_cap = 0;
    int *d_counter = nullptr;
    int counter_cap = 0;
    int nactive = 0;
    long long total_cells = 0;
    long long launches = 0;
    int persistent_blocks = 0;
    std::map<int, cudaGraphExec_t> graphs;  // one per frame length
    double *h_out = nullptr;
    // skewed passes
    int skew_mode = -1;                                   // -1 autotuned per size class, 0 off, 2..6 fixed
    int class_k[wg::BATCH_CLASSES] = {0};                 // tuned depth per size class (0: not yet)
    int class_rows[wg::BATCH_CLASSES] = {0};              // tuned row chunk per size class (0: list-wide size)
    std::map<std::pair<int, int>, BatchSkewList> lists;   // (depth class, pass depth) -> tasks
    int *d_skew_n = nullptr, *d_ticket = nullptr;        // task counts; tickets of a frame's passes
    int skew_n_cap = 0, ticket_cap = 0;
    cudaStream_t side[wg::BATCH_GROUPS] = {};             // one branch per depth class in a frame
    cudaEvent_t ev_fork = nullptr, ev_join[wg::BATCH_GROUPS] = {};
    unsigned graph_sig = 0;                               // depth classes present (bit K), plain chain (bit 0)
    int plain_tiles = 0, skew_scenes = 0, wrap_scenes = 0;
    std::vector<int> tab_slot;                            // slot of each table entry
    int *d_tune_ticket = nullptr;                         // tickets of the autotuner's passes
    std::vector<double> tune_ms;                          // last autotune: ms per update, [class * 8 + K]
};
