// wg_scene.h — the native scene object and the temporal-blocking entry points.
#pragma once
#include <vector>
#include "wg_internal.h"

#define WG_TB_MAX_K 16
#define WG_SKEW_MAX_K 6  // deepest skewed pass

struct SkewPlanCache {
    int4 *dev = nullptr;  // (column tile, first row, end row, edge) per warp
    int n = 0, min_rows = 0;
};

struct wg_scene {
    wg_params prm;
    wg::DevParams dp;
    int prec = WG_FP64, coef = WG_COEF_MASK;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    size_t esz = 8;
    int pitch = 0;
    void *f[2] = {nullptr, nullptr};  // f[cur] = phi (level t), f[1-cur] = psi (FP64) or the velocity (FP32)
    void *g[2] = {nullptr, nullptr};  // FP32: the output pair of every update and blocked pass
    int cur = 0;
    uint32_t *act = nullptr, *nz = nullptr;
    int has_ghosts = 0;
    std::vector<int16_t> xy_host;
    void *tcc = nullptr, *tc = nullptr, *tg = nullptr;
    int4 *nidx = nullptr;
    double2 *nw = nullptr;
    int nrec = 0;                          // gather entries (flag bit 1: an inactive record)
    wg_neumann_bc *nrec_dev = nullptr;     // records built on the device (wg_scene_build_domain)
    int nrec_all = 0;
    long long time = 0, launches = 0;
    double2 *ebot = nullptr, *etop = nullptr;
    double *eout = nullptr, *hout = nullptr;
    unsigned long long *dcount = nullptr;
    int *dflag = nullptr;          // set by a kernel whose bounded wait gave up
    void *dstage = nullptr;
    size_t dstage_bytes = 0;
    void *hstage = nullptr;
    size_t hstage_bytes = 0;
    uint8_t *rgb = nullptr, *lut = nullptr;
    int2 *probe_cells = nullptr;             // SAVE_TIME_SERIES probes: cells, samples [update][probe]
    double *probe_buf = nullptr;
    int probe_n = 0, probe_cap = 0, probe_count = 0;
    double *facc = nullptr;                  // frame running sums (mean, average, total flux)
    size_t facc_n = 0;
    int facc_plot = -1, facc_size = 0;
    size_t rgb_bytes = 0;
    int tb_k = 0, tile_i = 0, tile_j = 0;
    SkewPlanCache skew[WG_SKEW_MAX_K + 1];  // task lists of the skewed kernel, by depth
    float *bv_osc = nullptr;   // oscillating values of the current step() call, [n][ny]
    double *bv_src = nullptr;  // point-source increments of the current step() call, [n]
    size_t bv_cap = 0;
    long long bv_t0 = 0;
    bool uploaded = false;
    bool has_mask = false;  // by wg_scene_upload or wg_scene_build_domain
};

namespace wg {
wg_status scene_alloc_dense_stage(wg_scene *s, size_t bytes);
size_t scene_device_bytes(const wg_params &p, int prec, int coef);
template <class T> wg_status scene_step_impl(wg_scene *s, int nsteps);
// temporal blocking (wg_tb.cu)
bool tb_supported(const wg_scene *s);
template <class T> wg_status tb_pass(wg_scene *s, int k);
int tb_pass_depth(int k, int remaining);
wg_status tb_prepare(wg_scene *s, int n);
wg_status scene_check_flag(wg_scene *s);
void autotune_scene(wg_scene *s);
void probe_record(wg_scene *s);  // wg_io.cu: phi at the probes after an update
}  // namespace wg
