// wg_batch.h — batch engine objects shared by wg_batch.cu and wg_serve.cu.
#pragma once
#include <map>
#include <vector>
#include "wg_internal.h"

namespace wg {

constexpr int BT_ROWS = 32;      // rows of one work item
constexpr int BT_THREADS = 64;   // threads along j per tile row (x V cells)

struct __align__(16) SlotDev {   // one entry of the compact table of active scenes
    DevParams p;
    void *f[2];                  // the two field buffers; dyn.cur says which holds phi
    uint32_t *act, *nz;
    int slot;                    // index into the per-slot dynamic state
    int tiles_j, tile_base, ntiles;
};
struct SlotDyn {
    long long time;
    int cur;
    int pad;
};
struct BatchHdr {
    int nactive, total_tiles;
};

wg_status batch_refresh_table(::wg_batch *b);

}  // namespace wg

struct BatchSlotHost {
    bool used = false;
    wg_params prm;
    wg::DevParams dp;
    void *f[2] = {nullptr, nullptr};
    uint32_t *act = nullptr, *nz = nullptr;
    double2 *ebot = nullptr, *etop = nullptr;
    double *eout = nullptr;
    size_t bytes = 0;
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
};

