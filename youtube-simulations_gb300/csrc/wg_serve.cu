// wg_serve.cu — the serving loop: scene requests admitted under an HBM budget into a
// running batch (continuous batching), one frame of steps_per_frame updates per tick
// for every resident scene (the batch's CUDA graph), their RGB8 frames rendered in one
// launch into a packed buffer and copied to pinned host memory, per-frame latency and
// time to first frame recorded, finished scenes retired and their memory returned.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <unordered_map>
#include <vector>
#include "wg_batch.h"
#include "wg_internal.h"

namespace wg {

struct FrameDev {                // one resident scene in the frame launch
    DevParams p;
    void *f[4];
    uint32_t *nz;
    int slot;                    // batch slot (its dynamic state says which buffer is phi)
    int w, h, row_base;
    unsigned long long out_off;
};

template <class T>
__global__ void k_server_frames(const FrameDev *__restrict__ tab, int ntab, const SlotDyn *__restrict__ dyn,
                                const uint8_t *__restrict__ lut, wg_frame_params fp, uint8_t *__restrict__ out)
{
    __shared__ int e;
    if (threadIdx.x == 0) {
        int lo = 0, hi = ntab - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tab[mid].row_base <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
        }
        e = lo;
    }
    __syncthreads();
    const FrameDev &d = tab[e];
    const int row = (int)blockIdx.x - d.row_base;
    if (row >= d.h) return;
    const SlotDyn dy = dyn[d.slot];
    const T *phi = (const T *)d.f[2 * dy.pair + dy.cur];
    const int j = row * fp.size;
    for (int col = threadIdx.x; col < d.w; col += blockDim.x) {
        const int i = col * fp.size;
        uint8_t *o = out + d.out_off + ((size_t)row * d.w + col) * 3;
        const int m = (d.nz[(size_t)i * d.p.wpitch + (j >> 5)] >> (j & 31)) & 1u;
        if (!(d.p.twospeeds || m)) {
            o[0] = o[1] = o[2] = 0;
            continue;
        }
        const double value = fp.vshift + fp.vscale * (double)phi[(size_t)i * d.p.pitch + j];
        const double amp = fp.color_range * tanh(fp.slope * value / fp.scale);
        int hue = (int)(256.0 * (0.5 * (1.0 + amp)));
        hue = hue > 255 ? 255 : (hue < 0 ? 0 : hue);
        double f = 1.0;
        if (fp.fade_in_obstacle) f *= pow((m ? d.p.c2 : d.p.c2b) / d.p.c2, 0.1);
        if (fp.fade) f *= fp.fade_value;
        for (int k = 0; k < 3; k++) {
            const int b = (int)((double)lut[hue * 3 + k] * f + 0.5);
            o[k] = (uint8_t)(b > 255 ? 255 : (b < 0 ? 0 : b));
        }
    }
}

static double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static double percentile(std::vector<double> v, double q)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = q * (double)(v.size() - 1);
    const size_t lo = (size_t)pos;
    const size_t hi = std::min(lo + 1, v.size() - 1);
    return v[lo] + (pos - (double)lo) * (v[hi] - v[lo]);
}

}  // namespace wg

using namespace wg;

struct ServeReq {
    int64_t id = 0;
    wg_params p;
    std::vector<double> phi, psi;
    std::vector<int16_t> xy;
    int frames = 0, keep = 0, state = WG_REQ_QUEUED, slot = -1, frames_done = 0, last_index = -1;
    int64_t frame_tick = -1;  // the tick that rendered last_index into the host buffer
    double t_submit = 0.0, t_first = -1.0;
    uint64_t bytes = 0;
    int w = 0, h = 0;
    unsigned long long frame_off = 0;
    std::vector<double> res_phi, res_psi;
};

struct wg_server {
    wg_server_config cfg;
    wg_batch *batch = nullptr;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    std::deque<int64_t> queue;
    std::unordered_map<int64_t, ServeReq> reqs;
    std::vector<int64_t> resident;
    int64_t next_id = 1;
    uint64_t used = 0, peak = 0;
    uint8_t *d_lut = nullptr, *d_frames = nullptr, *h_frames = nullptr;
    size_t frames_cap = 0, frames_bytes = 0;
    FrameDev *d_ftab = nullptr;
    int ftab_cap = 0, total_rows = 0;
    bool layout_dirty = false;  // retirements since the last layout
    std::vector<double> lat_ms, first_ms;
    int64_t submitted = 0, admitted = 0, completed = 0, frames = 0, ticks = 0;
    double cell_updates = 0.0, busy = 0.0;
};

static uint64_t request_bytes(const wg_server *s, const wg_params &p)
{
    const BatchLayout L = batch_layout(p, s->cfg.precision);  // the batch's own layout (ghost layout included)
    const size_t pairs = batch_skew_ok(p, s->cfg.precision) ? 2 : 1;  // skewed scenes keep a second pair
    const size_t fields = 2 * pairs * L.field_bytes, masks = 2 * L.mask_bytes;
    const size_t frame = (size_t)(p.nx / s->cfg.frame.size) * (p.ny / s->cfg.frame.size) * 3;
    return fields + masks + frame + (size_t)p.nx * 40 + 4096;
}

// rebuild the frame table and the packed frame buffer after admissions/retirements
static wg_status server_layout(wg_server *s)
{
    std::vector<FrameDev> tab;
    int rows = 0;
    unsigned long long off = 0;
    for (int64_t id : s->resident) {
        ServeReq &r = s->reqs[id];
        const BatchSlotHost &h = s->batch->slots[r.slot];
        FrameDev d;
        memset(&d, 0, sizeof d);
        d.p = h.dp;
        for (int q = 0; q < 4; q++) d.f[q] = h.f[q];
        d.nz = h.nz;
        d.slot = r.slot;
        d.w = r.w;
        d.h = r.h;
        d.row_base = rows;
        d.out_off = off;
        r.frame_off = off;
        rows += r.h;
        off += (unsigned long long)r.w * r.h * 3;
        tab.push_back(d);
    }
    if ((int)tab.size() > s->ftab_cap) {
        if (s->d_ftab) cudaFree(s->d_ftab);
        s->d_ftab = nullptr;
        const int cap = std::max(64, (int)tab.size() * 2);
        WG_CUDA(cudaMalloc(&s->d_ftab, sizeof(FrameDev) * cap));
        s->ftab_cap = cap;
    }
    if (!tab.empty()) WG_CUDA(cudaMemcpyAsync(s->d_ftab, tab.data(), sizeof(FrameDev) * tab.size(), cudaMemcpyHostToDevice, s->st));
    if (off > s->frames_cap) {
        if (s->d_frames) cudaFree(s->d_frames);
        if (s->h_frames) cudaFreeHost(s->h_frames);
        s->d_frames = s->h_frames = nullptr;
        const size_t cap = (size_t)off * 3 / 2 + 4096;
        WG_CUDA(cudaMalloc(&s->d_frames, cap));
        WG_CUDA(cudaHostAlloc(&s->h_frames, cap, cudaHostAllocDefault));
        s->frames_cap = cap;
    }
    s->frames_bytes = off;
    s->total_rows = rows;
    return WG_OK;
}

extern "C" {

wg_status wg_server_create(const wg_server_config *cfg, void *stream, wg_server **out)
{
    if (!cfg || !out) { set_error("NULL argument"); return WG_ERR_INVALID; }
    if (cfg->frame.plot != WG_P_AMPLITUDE) { set_error("server frames are P_AMPLITUDE frames"); return WG_ERR_INVALID; }
    if (cfg->steps_per_frame < 1 || cfg->max_scenes < 1 || cfg->frame.size < 1 || !(cfg->frame.scale != 0.0)) {
        set_error("bad server configuration");
        return WG_ERR_INVALID;
    }
    wg_server *s = new wg_server();
    s->cfg = *cfg;
    if (stream) s->st = (cudaStream_t)stream;
    else {
        cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete s; return cuda_fail(e, "cudaStreamCreate"); }
        s->own_stream = true;
    }
    wg_status st = wg_batch_create(cfg->precision, s->st, &s->batch);
    if (st) { wg_server_destroy(s); return st; }
    cudaError_t e = cudaMalloc(&s->d_lut, 768);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_lut, cfg->lut, 768, cudaMemcpyHostToDevice, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) { wg_server_destroy(s); return cuda_fail(e, "wg_server_create"); }
    *out = s;
    return WG_OK;
}

wg_status wg_server_destroy(wg_server *s)
{
    if (!s) return WG_OK;
    if (s->st) cudaStreamSynchronize(s->st);
    if (s->batch) wg_batch_destroy(s->batch);
    if (s->d_lut) cudaFree(s->d_lut);
    if (s->d_frames) cudaFree(s->d_frames);
    if (s->h_frames) cudaFreeHost(s->h_frames);
    if (s->d_ftab) cudaFree(s->d_ftab);
    if (s->own_stream && s->st) cudaStreamDestroy(s->st);
    delete s;
    return WG_OK;
}

wg_status wg_server_submit(wg_server *s, const wg_params *p, const double *phi, const double *psi, const int16_t *xy,
                           int32_t frames, int32_t keep_result, int64_t *request_id)
{
    if (!s || !p || !phi || !psi || !xy || !request_id || frames < 1) { set_error("bad arguments"); return WG_ERR_INVALID; }
    wg_status st = validate_params(*p);
    if (st) return st;
    if (p->nx < s->cfg.frame.size || p->ny < s->cfg.frame.size) { set_error("grid smaller than the frame downsampling"); return WG_ERR_INVALID; }
    ServeReq r;
    r.id = s->next_id++;
    r.p = *p;
    const size_t n = (size_t)p->nx * p->ny;
    r.phi.assign(phi, phi + n);
    r.psi.assign(psi, psi + n);
    r.xy.assign(xy, xy + n);
    r.frames = frames;
    r.keep = keep_result;
    r.t_submit = now_s();
    r.bytes = request_bytes(s, *p);
    r.w = p->nx / s->cfg.frame.size;
    r.h = p->ny / s->cfg.frame.size;
    if (r.bytes > s->cfg.hbm_budget) { set_error("request needs %llu bytes, more than the whole budget", (unsigned long long)r.bytes); return WG_ERR_BUDGET; }
    *request_id = r.id;
    s->queue.push_back(r.id);
    s->reqs.emplace(r.id, std::move(r));
    s->submitted++;
    return WG_OK;
}

wg_status wg_server_tick(wg_server *s, int32_t *frames_out)
{
    if (!s) { set_error("NULL server"); return WG_ERR_INVALID; }
    const double t0 = now_s();
    wg_status st;
    // 1. admission, first come first served, while the budget and the slots allow
    bool changed = false;
    while (!s->queue.empty() && (int)s->resident.size() < s->cfg.max_scenes) {
        ServeReq &r = s->reqs[s->queue.front()];
        if (s->used + r.bytes > s->cfg.hbm_budget) break;
        int32_t slot = -1;
        if ((st = wg_batch_add(s->batch, &r.p, r.phi.data(), r.psi.data(), r.xy.data(), &slot))) return st;
        r.slot = slot;
        r.state = WG_REQ_RESIDENT;
        r.phi.clear(); r.phi.shrink_to_fit();
        r.psi.clear(); r.psi.shrink_to_fit();
        r.xy.clear(); r.xy.shrink_to_fit();
        s->used += r.bytes;
        s->peak = std::max(s->peak, s->used);
        s->resident.push_back(r.id);
        s->queue.pop_front();
        s->admitted++;
        changed = true;
    }
    // the frame table is rebuilt before this tick's frame launch whenever scenes were
    // admitted now or retired at the end of the previous tick
    if ((changed || s->layout_dirty) && (st = server_layout(s))) return st;
    s->layout_dirty = false;
    if (s->resident.empty()) {
        if (frames_out) *frames_out = 0;
        return WG_OK;
    }
    // 2. one frame for every resident scene (one graph launch)
    const double t_step = now_s();
    if ((st = wg_batch_step(s->batch, s->cfg.steps_per_frame))) return st;
    // 3. all frames in one launch, one copy to pinned host memory
    if (s->cfg.precision == WG_FP32)
        k_server_frames<float><<<s->total_rows, 128, 0, s->st>>>(s->d_ftab, (int)s->resident.size(), s->batch->d_dyn, s->d_lut, s->cfg.frame, s->d_frames);
    else
        k_server_frames<double><<<s->total_rows, 128, 0, s->st>>>(s->d_ftab, (int)s->resident.size(), s->batch->d_dyn, s->d_lut, s->cfg.frame, s->d_frames);
    WG_CUDA(cudaGetLastError());
    s->batch->launches++;
    WG_CUDA(cudaMemcpyAsync(s->h_frames, s->d_frames, s->frames_bytes, cudaMemcpyDeviceToHost, s->st));
    WG_CUDA(cudaStreamSynchronize(s->st));
    const double t1 = now_s();
    const double lat = 1e3 * (t1 - t_step);
    // 4. bookkeeping; retire finished requests
    std::vector<int64_t> keep_resident;
    long long cells = 0;
    for (int64_t id : s->resident) {
        ServeReq &r = s->reqs[id];
        cells += (long long)r.p.nx * r.p.ny;
        r.frames_done++;
        r.last_index = r.frames_done - 1;
        r.frame_tick = s->ticks;
        s->lat_ms.push_back(lat);
        if (r.t_first < 0.0) {
            r.t_first = t1;
            s->first_ms.push_back(1e3 * (t1 - r.t_submit));
        }
        s->frames++;
        if (r.frames_done >= r.frames) {
            if (r.keep) {
                r.res_phi.resize((size_t)r.p.nx * r.p.ny);
                r.res_psi.resize((size_t)r.p.nx * r.p.ny);
                if ((st = wg_batch_download(s->batch, r.slot, r.res_phi.data(), r.res_psi.data()))) return st;
            }
            r.state = WG_REQ_DONE;
            s->completed++;
        } else {
            keep_resident.push_back(id);
        }
    }
    s->cell_updates += (double)cells * s->cfg.steps_per_frame;
    if (frames_out) *frames_out = (int32_t)s->resident.size();
    if (keep_resident.size() != s->resident.size()) {
        // the retired scenes' frames stay readable in the host buffer until the next
        // layout change; their device memory returns to the pool now
        for (int64_t id : s->resident) {
            ServeReq &r = s->reqs[id];
            if (r.state == WG_REQ_DONE && r.slot >= 0) {
                if ((st = wg_batch_remove(s->batch, r.slot))) return st;
                s->used -= r.bytes;
                r.slot = -1;
            }
        }
        s->resident.swap(keep_resident);
        s->layout_dirty = true;
    }
    s->ticks++;
    s->busy += now_s() - t0;
    return WG_OK;
}

wg_status wg_server_frame(wg_server *s, int64_t id, uint8_t *rgb, int32_t *frame_index, int32_t *width, int32_t *height)
{
    if (!s) return WG_ERR_INVALID;
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { set_error("unknown request %lld", (long long)id); return WG_ERR_NOTFOUND; }
    const ServeReq &r = it->second;
    if (r.last_index < 0) { set_error("request %lld has no frame yet", (long long)id); return WG_ERR_STATE; }
    if (r.frame_tick != s->ticks - 1) {  // a later tick has rendered over the host buffer
        set_error("the last frame of request %lld (tick %lld) was overwritten by tick %lld: read frames before the "
                  "next tick", (long long)id, (long long)r.frame_tick, (long long)(s->ticks - 1));
        return WG_ERR_STATE;
    }
    if (width) *width = r.w;
    if (height) *height = r.h;
    if (frame_index) *frame_index = r.last_index;
    if (rgb) memcpy(rgb, s->h_frames + r.frame_off, (size_t)r.w * r.h * 3);
    return WG_OK;
}

wg_status wg_server_result(wg_server *s, int64_t id, double *phi, double *psi)
{
    if (!s) return WG_ERR_INVALID;
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { set_error("unknown request %lld", (long long)id); return WG_ERR_NOTFOUND; }
    const ServeReq &r = it->second;
    if (r.state != WG_REQ_DONE || !r.keep) { set_error("request %lld has no kept result", (long long)id); return WG_ERR_STATE; }
    if (phi) memcpy(phi, r.res_phi.data(), r.res_phi.size() * sizeof(double));
    if (psi) memcpy(psi, r.res_psi.data(), r.res_psi.size() * sizeof(double));
    return WG_OK;
}

wg_status wg_server_request_state(wg_server *s, int64_t id, int32_t *state, int32_t *frames_done)
{
    if (!s) return WG_ERR_INVALID;
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { set_error("unknown request %lld", (long long)id); return WG_ERR_NOTFOUND; }
    if (state) *state = it->second.state;
    if (frames_done) *frames_done = it->second.frames_done;
    return WG_OK;
}

wg_status wg_server_get_stats(wg_server *s, wg_server_stats *o)
{
    if (!s || !o) return WG_ERR_INVALID;
    memset(o, 0, sizeof *o);
    o->submitted = s->submitted;
    o->admitted = s->admitted;
    o->completed = s->completed;
    o->queued = (int64_t)s->queue.size();
    o->resident = (int64_t)s->resident.size();
    o->frames = s->frames;
    o->ticks = s->ticks;
    o->cell_updates = s->cell_updates;
    o->busy_seconds = s->busy;
    o->frame_latency_p50_ms = percentile(s->lat_ms, 0.50);
    o->frame_latency_p99_ms = percentile(s->lat_ms, 0.99);
    o->frame_latency_max_ms = s->lat_ms.empty() ? 0.0 : *std::max_element(s->lat_ms.begin(), s->lat_ms.end());
    o->first_frame_p50_ms = percentile(s->first_ms, 0.50);
    o->first_frame_p99_ms = percentile(s->first_ms, 0.99);
    o->bytes_resident = s->used;
    o->bytes_peak = s->peak;
    return WG_OK;
}

wg_status wg_server_request_bytes(wg_server *s, const wg_params *p, uint64_t *bytes)
{
    if (!s || !p || !bytes) return WG_ERR_INVALID;
    *bytes = request_bytes(s, *p);
    return WG_OK;
}

}  // extern "C"
