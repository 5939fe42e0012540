// wg_serve.cu — the serving loop: scene requests admitted under an HBM budget into a
// running batch (continuous batching), one frame of steps_per_frame updates per tick
// for every resident scene (the batch's CUDA graph), their RGB8 frames rendered in one
// launch into a packed buffer and copied to pinned host memory, per-frame latency and
// time to first frame recorded, finished and cancelled scenes retired and their memory
// returned.  Two frame buffers (device and pinned host) alternate between ticks, each
// with its own frame table and events: a pipelined server enqueues tick t and only then
// waits for tick t-1, so the device never idles while the host does a tick's
// bookkeeping, and the copy of tick t-1's frames overlaps tick t's updates.
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

// Where a request's latest frame lies in host memory.
struct FrameLoc {
    int64_t tick = -1;
    int buf = 0;
    unsigned long long off = 0;
    int index = -1;
};

struct ServeReq {
    int64_t id = 0;
    wg_params p;
    std::vector<double> phi, psi;
    std::vector<int16_t> xy;
    int frames = 0, keep = 0, state = WG_REQ_QUEUED, slot = -1;
    int frames_enqueued = 0, frames_done = 0;
    bool cancel = false;                       // resident: leave the batch at the next tick
    unsigned long long off[2] = {0, 0};        // its frame's offset in each frame buffer
    FrameLoc last;                             // its latest frame in host memory
    double t_submit = 0.0, t_first = -1.0;
    uint64_t bytes = 0;
    int w = 0, h = 0;
    std::vector<double> res_phi, res_psi;
};

// One enqueued tick: its frame buffer, when the host enqueued it, who takes part.
struct TickRec {
    bool pending = false;
    int64_t tick = -1;
    double t_enqueue = 0.0;
    long long cells = 0;
    std::vector<int64_t> ids;
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
    uint8_t *d_lut = nullptr;
    // per frame buffer q: device and pinned host frames, frame table, layout state, events
    uint8_t *d_frames[2] = {nullptr, nullptr}, *h_frames[2] = {nullptr, nullptr};
    size_t frames_cap[2] = {0, 0}, frames_bytes[2] = {0, 0};
    FrameDev *d_ftab[2] = {nullptr, nullptr};
    int ftab_cap[2] = {0, 0}, total_rows[2] = {0, 0}, ntab[2] = {0, 0};
    bool layout_dirty[2] = {true, true};  // membership changed since buffer q's layout
    cudaEvent_t ev_start[2] = {nullptr, nullptr}, ev_done[2] = {nullptr, nullptr};
    TickRec rec[2];
    int64_t readable_tick = -1;           // the tick whose frames wg_server_frame returns
    std::vector<double> lat_ms, first_ms, dev_ms;
    int64_t submitted = 0, admitted = 0, completed = 0, cancelled = 0, frames = 0, ticks = 0;
    double cell_updates = 0.0, busy = 0.0;
};

static uint64_t request_bytes(const wg_server *s, const wg_params &p)
{
    const BatchLayout L = batch_layout(p, s->cfg.precision);  // the batch's own layout (ghost layout included)
    const size_t pairs = s->cfg.precision == WG_FP32 ? 2 : 1;  // FP32 scenes keep a second pair
    const size_t fields = 2 * pairs * L.field_bytes, masks = 2 * L.mask_bytes;
    const size_t frame = (size_t)(p.nx / s->cfg.frame.size) * (p.ny / s->cfg.frame.size) * 3;
    return fields + masks + frame + (size_t)p.nx * 40 + 4096;
}

// Frame table and packed frame buffer q for the current resident scenes.  Buffer q was
// last used by a tick that has completed, and its frames are no longer readable.
static wg_status server_layout(wg_server *s, int q)
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
        for (int k = 0; k < 4; k++) d.f[k] = h.f[k];
        d.nz = h.nz;
        d.slot = r.slot;
        d.w = r.w;
        d.h = r.h;
        d.row_base = rows;
        d.out_off = off;
        r.off[q] = off;
        rows += r.h;
        off += (unsigned long long)r.w * r.h * 3;
        tab.push_back(d);
    }
    if ((int)tab.size() > s->ftab_cap[q]) {
        if (s->d_ftab[q]) cudaFree(s->d_ftab[q]);
        s->d_ftab[q] = nullptr;
        const int cap = std::max(64, (int)tab.size() * 2);
        WG_CUDA(cudaMalloc(&s->d_ftab[q], sizeof(FrameDev) * cap));
        s->ftab_cap[q] = cap;
    }
    if (!tab.empty())
        WG_CUDA(cudaMemcpyAsync(s->d_ftab[q], tab.data(), sizeof(FrameDev) * tab.size(), cudaMemcpyHostToDevice, s->st));
    if (off > s->frames_cap[q]) {
        if (s->d_frames[q]) cudaFree(s->d_frames[q]);
        if (s->h_frames[q]) cudaFreeHost(s->h_frames[q]);
        s->d_frames[q] = s->h_frames[q] = nullptr;
        const size_t cap = (size_t)off * 3 / 2 + 4096;
        WG_CUDA(cudaMalloc(&s->d_frames[q], cap));
        WG_CUDA(cudaHostAlloc(&s->h_frames[q], cap, cudaHostAllocDefault));
        s->frames_cap[q] = cap;
    }
    // the table copy above reads `tab` from pageable memory: the copy is complete when
    // cudaMemcpyAsync returns for pageable sources
    s->frames_bytes[q] = off;
    s->total_rows[q] = rows;
    s->ntab[q] = (int)tab.size();
    s->layout_dirty[q] = false;
    return WG_OK;
}

// A request that has rendered all its frames, or was cancelled, leaves the batch: its
// final state is downloaded first when it was submitted with keep_result (stream order
// places the download after its last frame).
static wg_status server_retire(wg_server *s, ServeReq &r)
{
    wg_status st;
    if (r.slot < 0) return WG_OK;
    if (r.keep && !r.cancel) {
        r.res_phi.resize((size_t)r.p.nx * r.p.ny);
        r.res_psi.resize((size_t)r.p.nx * r.p.ny);
        if ((st = wg_batch_download(s->batch, r.slot, r.res_phi.data(), r.res_psi.data()))) return st;
    }
    if ((st = wg_batch_remove(s->batch, r.slot))) return st;
    s->used -= r.bytes;
    r.slot = -1;
    if (r.cancel) {
        r.state = WG_REQ_CANCELLED;
        s->cancelled++;
    } else if (r.frames_done >= r.frames) {
        r.state = WG_REQ_DONE;
        s->completed++;
    }
    s->layout_dirty[0] = s->layout_dirty[1] = true;
    return WG_OK;
}

static wg_status server_retire_finished(wg_server *s)
{
    std::vector<int64_t> keep;
    bool any = false;
    for (int64_t id : s->resident) {
        ServeReq &r = s->reqs[id];
        if (r.cancel || r.frames_enqueued >= r.frames) {
            wg_status st = server_retire(s, r);
            if (st) return st;
            any = true;
        } else {
            keep.push_back(id);
        }
    }
    if (any) s->resident.swap(keep);
    return WG_OK;
}

// Waits for the tick enqueued on buffer q and makes its frames readable.
static wg_status server_complete(wg_server *s, int q, int32_t *nframes)
{
    TickRec &t = s->rec[q];
    if (nframes) *nframes = 0;
    if (!t.pending) return WG_OK;
    WG_CUDA(cudaEventSynchronize(s->ev_done[q]));
    const double t_obs = now_s();
    float dev = 0.f;
    WG_CUDA(cudaEventElapsedTime(&dev, s->ev_start[q], s->ev_done[q]));
    s->dev_ms.push_back(dev);
    const double lat = 1e3 * (t_obs - t.t_enqueue);
    for (int64_t id : t.ids) {
        ServeReq &r = s->reqs[id];
        r.frames_done++;
        r.last.tick = t.tick;
        r.last.buf = q;
        r.last.off = r.off[q];
        r.last.index = r.frames_done - 1;
        s->lat_ms.push_back(lat);
        if (r.t_first < 0.0) {
            r.t_first = t_obs;
            s->first_ms.push_back(1e3 * (t_obs - r.t_submit));
        }
        s->frames++;
        if (r.frames_done >= r.frames && r.slot < 0 && r.state == WG_REQ_RESIDENT) {  // retired already
            r.state = WG_REQ_DONE;
            s->completed++;
        }
    }
    s->cell_updates += (double)t.cells * s->cfg.steps_per_frame;
    s->readable_tick = t.tick;
    if (nframes) *nframes = (int32_t)t.ids.size();
    t.pending = false;
    t.ids.clear();
    return WG_OK;
}

extern "C" {

wg_status wg_server_create(const wg_server_config *cfg, void *stream, wg_server **out)
{
    if (!cfg || !out) { set_error("NULL argument"); return WG_ERR_INVALID; }
    if (cfg->frame.plot != WG_P_AMPLITUDE) { set_error("server frames are P_AMPLITUDE frames"); return WG_ERR_INVALID; }
    if (cfg->steps_per_frame < 1 || cfg->max_scenes < 1 || cfg->frame.size < 1 || !(cfg->frame.scale != 0.0) ||
        cfg->pipeline < 0 || cfg->pipeline > 1) {
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
    for (int q = 0; q < 2 && e == cudaSuccess; q++) {
        e = cudaEventCreate(&s->ev_start[q]);
        if (e == cudaSuccess) e = cudaEventCreate(&s->ev_done[q]);
    }
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
    for (int q = 0; q < 2; q++) {
        if (s->d_frames[q]) cudaFree(s->d_frames[q]);
        if (s->h_frames[q]) cudaFreeHost(s->h_frames[q]);
        if (s->d_ftab[q]) cudaFree(s->d_ftab[q]);
        if (s->ev_start[q]) cudaEventDestroy(s->ev_start[q]);
        if (s->ev_done[q]) cudaEventDestroy(s->ev_done[q]);
    }
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
    if (frames_out) *frames_out = 0;
    const int q = (int)(s->ticks & 1), prev = q ^ 1;
    int32_t done_early = 0;
    // pipelined: the previous tick's frames, once its copy has landed, are taken before
    // this tick's retirement and admission work (downloads, uploads, table refreshes), so
    // that work does not add to their latency
    auto take_prev_if_ready = [&]() -> wg_status {
        if (!s->cfg.pipeline || !s->rec[prev].pending) return WG_OK;
        const cudaError_t e = cudaEventQuery(s->ev_done[prev]);
        if (e == cudaErrorNotReady) return WG_OK;
        if (e != cudaSuccess) return cuda_fail(e, "cudaEventQuery");
        int32_t n = 0;
        const wg_status r = server_complete(s, prev, &n);
        done_early += n;
        return r;
    };
    if ((st = take_prev_if_ready())) return st;
    // 1. finished and cancelled requests leave the batch (their last frames stay readable)
    if ((st = server_retire_finished(s))) return st;
    if ((st = take_prev_if_ready())) return st;
    // 2. admission, first come first served, while the budget and the slots allow
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
        s->layout_dirty[0] = s->layout_dirty[1] = true;
    }
    if ((st = take_prev_if_ready())) return st;
    int32_t done_prev = 0;
    if (!s->resident.empty()) {
        // 3. buffer q's frame table follows the membership (buffer q was last used two
        // ticks ago, and that tick has completed)
        if (s->layout_dirty[q] && (st = server_layout(s, q))) return st;
        // 4. one frame for every resident scene (one graph launch), all frames in one
        // launch, one copy to pinned host memory, bracketed by the buffer's events
        TickRec &t = s->rec[q];
        t.tick = s->ticks;
        t.t_enqueue = now_s();
        t.cells = 0;
        t.ids = s->resident;
        for (int64_t id : s->resident) {
            ServeReq &r = s->reqs[id];
            t.cells += (long long)r.p.nx * r.p.ny;
            r.frames_enqueued++;
        }
        WG_CUDA(cudaEventRecord(s->ev_start[q], s->st));
        if ((st = wg_batch_step(s->batch, s->cfg.steps_per_frame))) return st;
        if (s->cfg.precision == WG_FP32)
            k_server_frames<float><<<s->total_rows[q], 128, 0, s->st>>>(s->d_ftab[q], s->ntab[q], s->batch->d_dyn,
                                                                        s->d_lut, s->cfg.frame, s->d_frames[q]);
        else
            k_server_frames<double><<<s->total_rows[q], 128, 0, s->st>>>(s->d_ftab[q], s->ntab[q], s->batch->d_dyn,
                                                                         s->d_lut, s->cfg.frame, s->d_frames[q]);
        WG_CUDA(cudaGetLastError());
        s->batch->launches++;
        WG_CUDA(cudaMemcpyAsync(s->h_frames[q], s->d_frames[q], s->frames_bytes[q], cudaMemcpyDeviceToHost, s->st));
        WG_CUDA(cudaEventRecord(s->ev_done[q], s->st));
        t.pending = true;
        s->ticks++;
    }
    // 5. pipelined: the previous tick's frames (its work ran ahead of this tick's);
    // otherwise this tick's own frames, and the requests they finished leave now
    if (s->cfg.pipeline) {
        if ((st = server_complete(s, prev, &done_prev))) return st;
    } else {
        if ((st = server_complete(s, q, &done_prev))) return st;
        if ((st = server_retire_finished(s))) return st;
    }
    if (frames_out) *frames_out = done_prev + done_early;
    s->busy += now_s() - t0;
    return WG_OK;
}

wg_status wg_server_drain(wg_server *s, int32_t *frames_out)
{
    if (!s) { set_error("NULL server"); return WG_ERR_INVALID; }
    const double t0 = now_s();
    if (frames_out) *frames_out = 0;
    for (int q = 0; q < 2; q++)
        if (s->rec[q].pending) {
            wg_status st = server_complete(s, q, frames_out);
            if (st) return st;
        }
    s->busy += now_s() - t0;
    return WG_OK;
}

wg_status wg_server_cancel(wg_server *s, int64_t id)
{
    if (!s) { set_error("NULL server"); return WG_ERR_INVALID; }
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { set_error("unknown request %lld", (long long)id); return WG_ERR_NOTFOUND; }
    ServeReq &r = it->second;
    if (r.state == WG_REQ_QUEUED) {
        s->queue.erase(std::find(s->queue.begin(), s->queue.end(), id));
        r.state = WG_REQ_CANCELLED;
        r.phi.clear(); r.phi.shrink_to_fit();
        r.psi.clear(); r.psi.shrink_to_fit();
        r.xy.clear(); r.xy.shrink_to_fit();
        s->cancelled++;
        return WG_OK;
    }
    if (r.state == WG_REQ_RESIDENT && !r.cancel && r.slot >= 0) {
        r.cancel = true;  // leaves the batch at the next tick, before that tick's frame
        return WG_OK;
    }
    set_error("request %lld is finished or already cancelled", (long long)id);
    return WG_ERR_STATE;
}

wg_status wg_server_frame(wg_server *s, int64_t id, uint8_t *rgb, int32_t *frame_index, int32_t *width, int32_t *height)
{
    if (!s) return WG_ERR_INVALID;
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { set_error("unknown request %lld", (long long)id); return WG_ERR_NOTFOUND; }
    const ServeReq &r = it->second;
    if (r.last.index < 0) { set_error("request %lld has no frame yet", (long long)id); return WG_ERR_STATE; }
    if (r.last.tick != s->readable_tick) {  // newer frames have been made readable since
        set_error("the last frame of request %lld (tick %lld) is no longer in host memory (tick %lld is): read "
                  "frames before the next tick", (long long)id, (long long)r.last.tick, (long long)s->readable_tick);
        return WG_ERR_STATE;
    }
    if (width) *width = r.w;
    if (height) *height = r.h;
    if (frame_index) *frame_index = r.last.index;
    if (rgb) memcpy(rgb, s->h_frames[r.last.buf] + r.last.off, (size_t)r.w * r.h * 3);
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
    o->tick_device_p50_ms = percentile(s->dev_ms, 0.50);
    o->tick_device_p99_ms = percentile(s->dev_ms, 0.99);
    o->cancelled = s->cancelled;
    return WG_OK;
}

wg_status wg_server_request_bytes(wg_server *s, const wg_params *p, uint64_t *bytes)
{
    if (!s || !p || !bytes) return WG_ERR_INVALID;
    *bytes = request_bytes(s, *p);
    return WG_OK;
}

}  // extern "C"
