// wg_api.cu — the C ABI of include/wavegpu.h: errors, parameters, the drop-in
// surface (row-pointer fields of the reference) and the native scene handles.
//
// No CPU fallback: every step, energy and colour map runs on the GPU; the host only
// packs/unpacks rows and copies.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>
#include "wg_internal.h"

namespace wg {

static thread_local std::string g_err;

void set_error(const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
}

void clear_error() { g_err.clear(); }

wg_status cuda_fail(cudaError_t e, const char *what)
{
    set_error("CUDA error %s (%s) in %s", cudaGetErrorName(e), cudaGetErrorString(e), what);
    return (e == cudaErrorMemoryAllocation) ? WG_ERR_NOMEM : WG_ERR_CUDA;
}

int pitch_for(int ny, int elem_bytes)
{
    const int per = 512 / elem_bytes;  // rows padded to 512 bytes: whole 16-byte vectors per warp
    return ((ny + per - 1) / per) * per;
}

static int y_to_j(const wg_params &p, double y)
{
    double y1 = (y - p.ymin) / (p.ymax - p.ymin);
    return (int)(y1 * (double)p.ny);
}

DevParams make_dev_params(const wg_params &p, int pitch)
{
    DevParams d;
    memset(&d, 0, sizeof d);
    d.nx = p.nx;
    d.ny = p.ny;
    d.pitch = pitch;
    d.wpitch = (pitch + 31) / 32;
    d.b_cond = p.b_cond;
    d.twospeeds = p.twospeeds != 0;
    d.osc_left = p.oscillate_left != 0;
    d.osc_topbot = p.oscillate_topbot != 0;
    d.sched = p.oscillation_schedule;
    d.floor_clamp = p.floor_clamp != 0;
    d.beam = (p.oscillation_schedule == WG_OSC_BEAM_SINE || p.oscillation_schedule == WG_OSC_BEAM_SINE_DECREASING ||
              p.oscillation_schedule == WG_OSC_BEAM_SINE_TWOPERIODS || p.oscillation_schedule == WG_OSC_BEAM_SINE_CHIRP);
    if (d.osc_left && d.beam) {
        d.bc_jmax = y_to_j(p, p.oscil_ymid + p.oscil_ymax);
        d.bc_jmin = y_to_j(p, p.oscil_ymid - p.oscil_ymax);
    } else {
        d.bc_jmin = 0;
        d.bc_jmax = p.ny - 1;
    }
    d.osc_beam_jmax = y_to_j(p, p.oscil_ymax);
    d.osc_sine_jmax = y_to_j(p, p.oscil_ymid + p.oscil_ymax);
    d.osc_sine_jmin = y_to_j(p, p.oscil_ymid - p.oscil_ymax);
    d.src_on = p.src_on != 0;
    d.src_i = p.src_i;
    d.src_j = p.src_j;
    d.corner2_on = p.nx <= p.ny;
    // the reference's tb_shift, (int)((XMAX-XMIN)*NX/(XMAX-XMIN)), an integer: its row test
    // i < tb_shift is i < tb_ilim
    d.tb_ilim = p.oscillate_topbot ? (int)((p.xmax - p.xmin) * (double)p.nx / (p.xmax - p.xmin)) : 0;
    d.pad0_ = 0;
    d.kappa = p.kappa;
    d.kappa_sides = p.kappa_sides;
    d.kappa_topbot = p.kappa_topbot;
    d.gamma_sides = p.gamma_sides;
    d.gamma_topbot = p.gamma_topbot;
    d.vmax = p.vmax;
    d.c2 = p.courant * p.courant;
    d.c2b = p.courantb * p.courantb;
    d.gam = p.gamma;
    d.gamb = p.gammab;
    d.courant = p.courant;
    d.courantb = p.courantb;
    d.omega = p.omega;
    d.omega_b = p.omega_b;
    d.amplitude = p.amplitude;
    d.damping = p.damping;
    d.achirp = p.achirp;
    d.yshift = p.oscil_left_yshift;
    d.ivar = p.initial_variance;
    d.ishift = p.initial_shift;
    d.wpshift = p.wave_packet_shift;
    d.ymin = p.ymin;
    d.ymax = p.ymax;
    d.src_amp = p.src_amp;
    d.src_period = p.src_period;
    d.e_scale2 = p.e_scale * p.e_scale;
    d.ehalf_c2 = 0.5 * p.courant * p.courant;
    d.ehalf_c2b = 0.5 * p.courantb * p.courantb;
    return d;
}

wg_status validate_params(const wg_params &p)
{
    if (p.nx < 3 || p.ny < 3) { set_error("grid %d x %d: NX and NY must be >= 3", p.nx, p.ny); return WG_ERR_INVALID; }
    if ((long long)p.nx * p.ny > (1LL << 34)) { set_error("grid too large"); return WG_ERR_INVALID; }
    if (p.b_cond < 0 || p.b_cond > 3) { set_error("B_COND %d not supported (0..3)", p.b_cond); return WG_ERR_INVALID; }
    if (p.src_on && (p.src_i < 0 || p.src_i >= p.nx || p.src_j < 0 || p.src_j >= p.ny)) {
        set_error("point source (%d,%d) outside the grid", p.src_i, p.src_j);
        return WG_ERR_INVALID;
    }
    if (p.src_on && !(p.src_period != 0.0)) { set_error("point source period must be non-zero"); return WG_ERR_INVALID; }
    if (p.xmax == p.xmin || p.ymax == p.ymin) { set_error("empty box"); return WG_ERR_INVALID; }
    return WG_OK;
}

static wg_status validate_records(const wg_params &p, const wg_neumann_bc *r, int n)
{
    if (n < 0) { set_error("negative record count"); return WG_ERR_INVALID; }
    if (n > 0 && !r) { set_error("records pointer is NULL"); return WG_ERR_INVALID; }
    for (int q = 0; q < n; q++) {
        if (!r[q].active) continue;
        if (r[q].i < 1 || r[q].i > p.nx - 2 || r[q].j < 1 || r[q].j > p.ny - 2 || r[q].nbi1 < 0 ||
            r[q].nbi1 >= p.nx || r[q].nbj1 < 0 || r[q].nbj1 >= p.ny || r[q].nbi2 < 0 || r[q].nbi2 >= p.nx ||
            r[q].nbj2 < 0 || r[q].nbj2 >= p.ny) {
            set_error("Neumann record %d: cell (%d,%d) must lie in 1..NX-2 x 1..NY-2 with neighbours in the grid", q,
                      r[q].i, r[q].j);
            return WG_ERR_INVALID;
        }
    }
    return WG_OK;
}

// ---------------------------------------------------------------------------
// Drop-in state (the reference's globals: one configuration per process)
// ---------------------------------------------------------------------------
struct DropIn {
    bool configured = false;
    wg_params prm;
    DevParams dp;
    int pitch = 0;
    int mode = WG_DROPIN_STRICT;
    int rows_mode = WG_ROWS_AUTO;
    int pageable = -1;           // the device addresses pageable host memory (-1: not asked yet)
    long long time = 0;
    cudaStream_t st = nullptr;
    double *buf[3] = {nullptr, nullptr, nullptr};
    double **host_rows[3] = {nullptr, nullptr, nullptr};  // identity of each slot (resident)
    int16_t *xy = nullptr;
    double *tcc = nullptr, *tc = nullptr, *tg = nullptr;
    wg_neumann_bc *rec = nullptr;
    int rec_cap = 0, nrec = 0;
    const void *static_key[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    const void *rec_key = nullptr;
    int rec_key_n = -1;
    bool statics_valid = false, energy_statics_valid = false;
    void *hstage = nullptr;
    size_t hstage_bytes = 0;
    double2 *ebot = nullptr, *etop = nullptr;
    double *eout = nullptr;
    double *hout = nullptr;
    void release()
    {
        for (auto &b : buf) { if (b) cudaFree(b); b = nullptr; }
        if (xy) cudaFree(xy);
        if (tcc) cudaFree(tcc);
        if (tc) cudaFree(tc);
        if (tg) cudaFree(tg);
        if (rec) cudaFree(rec);
        if (ebot) cudaFree(ebot);
        if (etop) cudaFree(etop);
        if (eout) cudaFree(eout);
        if (hstage) cudaFreeHost(hstage);
        if (hout) cudaFreeHost(hout);
        xy = nullptr; tcc = tc = tg = nullptr; rec = nullptr; ebot = etop = nullptr; eout = nullptr;
        hstage = nullptr; hout = nullptr; hstage_bytes = 0; rec_cap = 0;
    }
};
static DropIn g_di;
static std::mutex g_di_mu;

static wg_status di_stage(size_t bytes)
{
    if (g_di.hstage_bytes >= bytes) return WG_OK;
    if (g_di.hstage) cudaFreeHost(g_di.hstage);
    g_di.hstage = nullptr;
    g_di.hstage_bytes = 0;
    WG_CUDA(cudaHostAlloc(&g_di.hstage, bytes, cudaHostAllocDefault));
    g_di.hstage_bytes = bytes;
    return WG_OK;
}

// Rows read and written in place by the device: one block per row, 16-byte accesses where
// the row and its byte count allow (a pitched row starts on 512 bytes), the padding zeroed.
// Only on devices that address pageable host memory with the host's page tables.
template <class E>
__global__ void k_rows_in(const E *const *__restrict__ rows, int nx, int ny, int pitch, E *__restrict__ dst)
{
    const int i = blockIdx.x;
    if (i >= nx) return;
    const E *r = rows[i];
    E *d = dst + (size_t)i * pitch;
    const size_t rb = (size_t)ny * sizeof(E);
    if (((uintptr_t)r & 15) == 0 && rb % 16 == 0) {
        const int4 *s4 = reinterpret_cast<const int4 *>(r);
        int4 *d4 = reinterpret_cast<int4 *>(d);
        for (size_t k = threadIdx.x; k < rb / 16; k += blockDim.x) d4[k] = s4[k];
    } else {
        for (int j = threadIdx.x; j < ny; j += blockDim.x) d[j] = r[j];
    }
    for (int j = ny + threadIdx.x; j < pitch; j += blockDim.x) d[j] = E(0);
}
__global__ void k_rows_out(double *const *__restrict__ rows, int nx, int ny, int pitch, const double *__restrict__ src)
{
    const int i = blockIdx.x;
    if (i >= nx) return;
    double *r = rows[i];
    const double *s = src + (size_t)i * pitch;
    const size_t rb = (size_t)ny * sizeof(double);
    if (((uintptr_t)r & 15) == 0 && rb % 16 == 0) {
        const int4 *s4 = reinterpret_cast<const int4 *>(s);
        int4 *d4 = reinterpret_cast<int4 *>(r);
        for (size_t k = threadIdx.x; k < rb / 16; k += blockDim.x) d4[k] = s4[k];
    } else {
        for (int j = threadIdx.x; j < ny; j += blockDim.x) r[j] = s[j];
    }
}

// the rows go in place: asked for, and the device addresses pageable host memory through
// the host's page tables
static bool di_in_place()
{
    if (g_di.rows_mode != WG_ROWS_AUTO) return false;
    if (g_di.pageable < 0) {
        int dev = 0, a = 0, b = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
            cudaGetLastError();
            a = b = 0;
        }
        g_di.pageable = (a == 1 && b == 1) ? 1 : 0;
    }
    return g_di.pageable == 1;
}

// rows (NX pointers to NY values) -> pitched device array, in place or through pinned staging
// Row copies between the caller's row arrays and the pinned stage, split over up to 8
// host threads (one thread copies at well under the host link's rate: 43 against 12.5 ms
// per strict evolve_wave on config 2; 16 threads and a second stage measured the same);
// serial where threads cannot be started.
template <class F>
static void par_rows(int nx, F f)
{
    const unsigned hw = std::thread::hardware_concurrency();
    const int T = (int)std::min(8u, std::max(1u, hw));
    if (T == 1 || nx < 256) {
        f(0, nx);
        return;
    }
    const int chunk = (nx + T - 1) / T;
    std::vector<std::thread> th;
    int done = chunk;  // rows [0, chunk) run on this thread
    try {
        for (int t = 1; t < T; t++) {
            const int a = t * chunk, b = std::min(nx, a + chunk);
            if (a >= b) break;
            th.emplace_back(f, a, b);
            done = b;
        }
    } catch (...) {
    }
    f(0, std::min(nx, chunk));
    for (auto &x : th) x.join();
    if (done < nx) f(done, nx);  // rows whose thread could not be started
}

template <class E>
static wg_status di_upload_rows(E **rows, E *dev)
{
    const int nx = g_di.prm.nx, ny = g_di.prm.ny, P = g_di.pitch;
    const size_t bytes = (size_t)nx * P * sizeof(E);
    wg_status s = di_stage(bytes);
    if (s) return s;
    for (int i = 0; i < nx; i++)
        if (!rows[i]) { set_error("row %d is NULL", i); return WG_ERR_INVALID; }
    if (di_in_place()) {
        // the kernel reads the caller's row table and rows; the call waits for it, so the
        // rows may change (or go) as soon as it returns
        k_rows_in<E><<<nx, 256, 0, g_di.st>>>(rows, nx, ny, P, dev);
        WG_CUDA(cudaGetLastError());
        WG_CUDA(cudaStreamSynchronize(g_di.st));
        return WG_OK;
    }
    WG_CUDA(cudaStreamSynchronize(g_di.st));  // staging may still feed an earlier copy
    E *h = (E *)g_di.hstage;
    par_rows(nx, [&](int a, int b) {
        for (int i = a; i < b; i++) {
            memcpy(h + (size_t)i * P, rows[i], sizeof(E) * ny);
            memset(h + (size_t)i * P + ny, 0, sizeof(E) * (P - ny));
        }
    });
    WG_CUDA(cudaMemcpyAsync(dev, h, bytes, cudaMemcpyHostToDevice, g_di.st));
    return WG_OK;
}

static wg_status di_download_rows(double *dev, double **rows)
{
    const int nx = g_di.prm.nx, ny = g_di.prm.ny, P = g_di.pitch;
    const size_t bytes = (size_t)nx * P * sizeof(double);
    if (di_in_place()) {
        for (int i = 0; i < nx; i++)
            if (!rows[i]) { set_error("row %d is NULL", i); return WG_ERR_INVALID; }
        k_rows_out<<<nx, 256, 0, g_di.st>>>(rows, nx, ny, P, dev);
        WG_CUDA(cudaGetLastError());
        WG_CUDA(cudaStreamSynchronize(g_di.st));
        return WG_OK;
    }
    wg_status s = di_stage(bytes);
    if (s) return s;
    WG_CUDA(cudaMemcpyAsync(g_di.hstage, dev, bytes, cudaMemcpyDeviceToHost, g_di.st));
    WG_CUDA(cudaStreamSynchronize(g_di.st));
    const double *h = (const double *)g_di.hstage;
    par_rows(nx, [&](int a, int b) {
        for (int i = a; i < b; i++) memcpy(rows[i], h + (size_t)i * P, sizeof(double) * ny);
    });
    return WG_OK;
}

static wg_status di_require()
{
    if (!g_di.configured) {
        set_error("drop-in not configured: call wg_dropin_configure (wavegpu_dropin.h does it from the macros)");
        return WG_ERR_STATE;
    }
    return WG_OK;
}

// mask and tables: uploaded on every call in strict mode, on a change of the row
// arrays' identity in resident mode
static wg_status di_statics(int16_t **xy, double **tcc, double **tc, double **tg, bool with_tables)
{
    const bool resident = g_di.mode == WG_DROPIN_RESIDENT;
    wg_status s;
    if (!xy) { set_error("xy_in is NULL"); return WG_ERR_INVALID; }
    if (!(resident && g_di.statics_valid && g_di.static_key[0] == xy)) {
        if ((s = di_upload_rows<int16_t>(xy, g_di.xy))) return s;
        g_di.static_key[0] = xy;
        g_di.statics_valid = true;
    }
    if (!with_tables) return WG_OK;
    if (!tcc || !tg) { set_error("tcc/tgamma tables are NULL"); return WG_ERR_INVALID; }
    const bool absorbing = g_di.prm.b_cond == WG_BC_ABSORBING || g_di.prm.b_cond == WG_BC_VPER_HABS;
    if (absorbing && !tc) { set_error("tc table is NULL with an absorbing boundary"); return WG_ERR_INVALID; }
    if (resident && g_di.energy_statics_valid && g_di.static_key[1] == tcc && g_di.static_key[2] == tc &&
        g_di.static_key[3] == tg)
        return WG_OK;
    if ((s = di_upload_rows<double>(tcc, g_di.tcc))) return s;
    if ((s = di_upload_rows<double>(tg, g_di.tg))) return s;
    if (absorbing && (s = di_upload_rows<double>(tc, g_di.tc))) return s;
    g_di.static_key[1] = tcc;
    g_di.static_key[2] = tc;
    g_di.static_key[3] = tg;
    g_di.energy_statics_valid = true;
    return WG_OK;
}

static wg_status di_records(const wg_neumann_bc *r, int n)
{
    if (!g_di.prm.bc_neumann) { g_di.nrec = 0; return WG_OK; }
    if (g_di.mode == WG_DROPIN_RESIDENT && r == g_di.rec_key && n == g_di.rec_key_n) return WG_OK;
    wg_status s = validate_records(g_di.prm, r, n);
    if (s) return s;
    if (n > g_di.rec_cap) {
        if (g_di.rec) cudaFree(g_di.rec);
        g_di.rec = nullptr;
        WG_CUDA(cudaMalloc(&g_di.rec, sizeof(wg_neumann_bc) * n));
        g_di.rec_cap = n;
    }
    if (n) WG_CUDA(cudaMemcpyAsync(g_di.rec, r, sizeof(wg_neumann_bc) * n, cudaMemcpyHostToDevice, g_di.st));
    WG_CUDA(cudaStreamSynchronize(g_di.st));
    g_di.nrec = n;
    g_di.rec_key = r;
    g_di.rec_key_n = n;
    return WG_OK;
}

// slot of a row-pointer array: fixed order in strict mode, identity in resident mode
static int di_slot(double **rows, int strict_slot, bool *fresh)
{
    *fresh = false;
    if (g_di.mode == WG_DROPIN_STRICT) {
        g_di.host_rows[strict_slot] = rows;
        *fresh = true;
        return strict_slot;
    }
    for (int k = 0; k < 3; k++)
        if (g_di.host_rows[k] == rows) return k;
    for (int k = 0; k < 3; k++)
        if (!g_di.host_rows[k]) {
            g_di.host_rows[k] = rows;
            *fresh = true;
            return k;
        }
    return -1;
}

static wg_status di_one_update(int in, int prev, int out)
{
    g_di.time++;
    const bool recs = g_di.prm.bc_neumann && g_di.nrec > 0;
    launch_step_exact(g_di.dp, g_di.buf[in], g_di.buf[prev], g_di.buf[out], g_di.xy, g_di.tcc, g_di.tc, g_di.tg,
                      g_di.time, recs ? 0 : 1, g_di.st);
    if (recs) {
        launch_neumann_exact(g_di.dp, g_di.buf[in], g_di.buf[out], g_di.xy, g_di.rec, g_di.nrec, g_di.st);
        if (g_di.prm.src_on) launch_point_source<double>(g_di.dp, g_di.buf[out], nullptr, g_di.time, g_di.st);
    }
    WG_CUDA(cudaGetLastError());
    return WG_OK;
}

}  // namespace wg

using namespace wg;

extern "C" {

int32_t wg_abi_version(void) { return 3; }

const char *wg_last_error(void) { return g_err.c_str(); }

const char *wg_status_string(wg_status s)
{
    switch (s) {
    case WG_OK: return "ok";
    case WG_ERR_INVALID: return "invalid argument";
    case WG_ERR_CUDA: return "CUDA error";
    case WG_ERR_NOMEM: return "out of memory";
    case WG_ERR_BUDGET: return "HBM budget exceeded";
    case WG_ERR_STATE: return "invalid state";
    case WG_ERR_TIMEOUT: return "timeout";
    case WG_ERR_NONFINITE: return "non-finite field values";
    case WG_ERR_NOTFOUND: return "not found";
    default: return "unknown status";
    }
}

void wg_params_default(wg_params *p, int32_t nx, int32_t ny)
{
    memset(p, 0, sizeof *p);
    p->nx = nx;
    p->ny = ny;
    p->b_cond = WG_BC_DIRICHLET;
    p->xmin = -2.0; p->xmax = 2.0; p->ymin = -1.125; p->ymax = 1.125;
    p->courant = 0.1; p->courantb = 0.05;
    p->kappa_sides = 5.0e-4; p->gamma_sides = 1.0e-4; p->gamma_topbot = 1.0e-7;
    p->omega = 0.005; p->omega_b = 0.01; p->amplitude = 1.0; p->achirp = 0.25;
    p->oscil_ymax = 1.2;
    p->initial_variance = 0.0003; p->initial_shift = 20.0; p->wave_packet_shift = 200.0;
    p->vmax = 2.5; p->e_scale = 300.0; p->src_period = 1.0;
}

wg_status wg_dropin_configure(const wg_params *p)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    if (!p) { set_error("params is NULL"); return WG_ERR_INVALID; }
    wg_status s = validate_params(*p);
    if (s) return s;
    const bool same_size = g_di.configured && g_di.prm.nx == p->nx && g_di.prm.ny == p->ny;
    if (!same_size) {
        g_di.release();
        g_di.configured = false;
        if (!g_di.st) WG_CUDA(cudaStreamCreateWithFlags(&g_di.st, cudaStreamNonBlocking));
        g_di.pitch = pitch_for(p->ny, 8);
        const size_t f = (size_t)p->nx * g_di.pitch;
        for (auto &b : g_di.buf) WG_CUDA(cudaMalloc(&b, f * sizeof(double)));
        WG_CUDA(cudaMalloc(&g_di.xy, f * sizeof(int16_t)));
        WG_CUDA(cudaMalloc(&g_di.tcc, f * sizeof(double)));
        WG_CUDA(cudaMalloc(&g_di.tc, f * sizeof(double)));
        WG_CUDA(cudaMalloc(&g_di.tg, f * sizeof(double)));
        WG_CUDA(cudaMemset(g_di.tc, 0, f * sizeof(double)));
        WG_CUDA(cudaMalloc(&g_di.ebot, p->nx * sizeof(double2)));
        WG_CUDA(cudaMalloc(&g_di.etop, p->nx * sizeof(double2)));
        WG_CUDA(cudaMalloc(&g_di.eout, (p->nx + 8) * sizeof(double)));
        WG_CUDA(cudaHostAlloc(&g_di.hout, (p->nx + 8) * sizeof(double), cudaHostAllocDefault));
    }
    g_di.prm = *p;
    g_di.dp = make_dev_params(*p, g_di.pitch);
    g_di.time = 0;
    g_di.statics_valid = false;
    g_di.energy_statics_valid = false;
    g_di.rec_key = nullptr;
    g_di.rec_key_n = -1;
    for (auto &h : g_di.host_rows) h = nullptr;
    g_di.configured = true;
    return WG_OK;
}

wg_status wg_dropin_set_mode(int32_t mode)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    if (mode != WG_DROPIN_STRICT && mode != WG_DROPIN_RESIDENT) { set_error("unknown mode %d", mode); return WG_ERR_INVALID; }
    g_di.mode = mode;
    for (auto &h : g_di.host_rows) h = nullptr;
    g_di.statics_valid = false;
    g_di.energy_statics_valid = false;
    g_di.rec_key = nullptr;
    return WG_OK;
}

wg_status wg_dropin_set_rows(int32_t rows_mode)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    if (rows_mode != WG_ROWS_AUTO && rows_mode != WG_ROWS_PACKED) {
        set_error("unknown rows mode %d", rows_mode);
        return WG_ERR_INVALID;
    }
    g_di.rows_mode = rows_mode;
    return WG_OK;
}

wg_status wg_dropin_sync(void)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    wg_status s = di_require();
    if (s) return s;
    for (int k = 0; k < 3; k++)
        if (g_di.host_rows[k] && (s = di_download_rows(g_di.buf[k], g_di.host_rows[k]))) return s;
    return WG_OK;
}

wg_status wg_dropin_add_circular_wave(double init_amp, double factor, double x, double y, double variance,
                                      double wavelength, double **phi, double **psi, int16_t **xy_in)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    wg_status s = di_require();
    if (s) return s;
    if (!phi || !psi || !xy_in) { set_error("NULL argument"); return WG_ERR_INVALID; }
    PulseArgs pa;
    if ((s = pulse_args(g_di.prm, g_di.pitch, g_di.dp.wpitch, init_amp, factor, x, y, variance, wavelength, &pa)))
        return s;
    if ((s = di_statics(xy_in, nullptr, nullptr, nullptr, false))) return s;
    bool fresh;
    const int k = di_slot(phi, 0, &fresh);
    if (k < 0) { set_error("too many field arrays"); return WG_ERR_STATE; }
    if (fresh && (s = di_upload_rows<double>(phi, g_di.buf[k]))) return s;
    launch_add_circular_wave<double>(pa, g_di.buf[k], nullptr, g_di.xy, nullptr, g_di.st);
    WG_CUDA(cudaGetLastError());
    if (g_di.mode == WG_DROPIN_STRICT) return di_download_rows(g_di.buf[k], phi);
    return WG_OK;
}

wg_status wg_dropin_cell(double **phi, int32_t i, int32_t j, double *out)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    wg_status s = di_require();
    if (s) return s;
    if (!phi || !out || i < 0 || j < 0 || i >= g_di.prm.nx || j >= g_di.prm.ny) { set_error("bad arguments"); return WG_ERR_INVALID; }
    if (g_di.mode == WG_DROPIN_RESIDENT)
        for (int k = 0; k < 3; k++)
            if (g_di.host_rows[k] == phi) {
                WG_CUDA(cudaMemcpyAsync(g_di.hout, g_di.buf[k] + (size_t)i * g_di.pitch + j, sizeof(double),
                                        cudaMemcpyDeviceToHost, g_di.st));
                WG_CUDA(cudaStreamSynchronize(g_di.st));
                *out = g_di.hout[0];
                return WG_OK;
            }
    if (!phi[i]) { set_error("row %d is NULL", i); return WG_ERR_INVALID; }
    *out = phi[i][j];
    return WG_OK;
}

wg_status wg_dropin_invalidate(void)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    for (auto &h : g_di.host_rows) h = nullptr;
    g_di.statics_valid = false;
    g_di.energy_statics_valid = false;
    g_di.rec_key = nullptr;
    return WG_OK;
}

wg_status wg_dropin_get_time(int64_t *t)
{
    if (!t) return WG_ERR_INVALID;
    *t = g_di.time;
    return WG_OK;
}

wg_status wg_dropin_set_time(int64_t t)
{
    g_di.time = t;
    return WG_OK;
}

wg_status wg_evolve_wave_half(double **phi_in, double **psi_in, double **phi_out, int16_t **xy_in, double **tcc,
                              double **tc, double **tgamma, const wg_neumann_bc *neumann_bc, int32_t n_neumann)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    wg_status s = di_require();
    if (s) return s;
    if (!phi_in || !psi_in || !phi_out) { set_error("field pointer is NULL"); return WG_ERR_INVALID; }
    if (phi_in == phi_out || psi_in == phi_out) { set_error("phi_out must differ from phi_in and psi_in"); return WG_ERR_INVALID; }
    if ((s = di_statics(xy_in, tcc, tc, tgamma, true))) return s;
    if ((s = di_records(neumann_bc, n_neumann))) return s;
    bool f0, f1, f2;
    const int a = di_slot(phi_in, 0, &f0), b = di_slot(psi_in, 1, &f1), c = di_slot(phi_out, 2, &f2);
    if (a < 0 || b < 0 || c < 0 || a == b || a == c || b == c) {
        set_error("more than three distinct field arrays in resident mode; call wg_dropin_invalidate first");
        return WG_ERR_STATE;
    }
    if (f0 && (s = di_upload_rows<double>(phi_in, g_di.buf[a]))) return s;
    if (f1 && (s = di_upload_rows<double>(psi_in, g_di.buf[b]))) return s;
    if (f2 && (s = di_upload_rows<double>(phi_out, g_di.buf[c]))) return s;
    if ((s = di_one_update(a, b, c))) return s;
    if (g_di.mode == WG_DROPIN_STRICT) return di_download_rows(g_di.buf[c], phi_out);
    return WG_OK;
}

wg_status wg_evolve_wave(double **phi, double **psi, double **tmp, int16_t **xy_in, double **tcc, double **tc,
                         double **tgamma, const wg_neumann_bc *neumann_bc, int32_t n_neumann)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    wg_status s = di_require();
    if (s) return s;
    if (!phi || !psi || !tmp || phi == psi || phi == tmp || psi == tmp) {
        set_error("phi, psi and tmp must be three distinct arrays");
        return WG_ERR_INVALID;
    }
    if ((s = di_statics(xy_in, tcc, tc, tgamma, true))) return s;
    if ((s = di_records(neumann_bc, n_neumann))) return s;
    bool f0, f1, f2;
    const int a = di_slot(phi, 0, &f0), b = di_slot(psi, 1, &f1), c = di_slot(tmp, 2, &f2);
    if (a < 0 || b < 0 || c < 0) {
        set_error("more than three distinct field arrays in resident mode; call wg_dropin_invalidate first");
        return WG_ERR_STATE;
    }
    if (f0 && (s = di_upload_rows<double>(phi, g_di.buf[a]))) return s;
    if (f1 && (s = di_upload_rows<double>(psi, g_di.buf[b]))) return s;
    if (f2 && (s = di_upload_rows<double>(tmp, g_di.buf[c]))) return s;
    // wave_billiard.c:623-627
    if ((s = di_one_update(a, b, c))) return s;
    if ((s = di_one_update(c, a, b))) return s;
    if ((s = di_one_update(b, c, a))) return s;
    if (g_di.mode == WG_DROPIN_STRICT) {
        if ((s = di_download_rows(g_di.buf[a], phi))) return s;
        if ((s = di_download_rows(g_di.buf[b], psi))) return s;
        if ((s = di_download_rows(g_di.buf[c], tmp))) return s;
    }
    return WG_OK;
}

static wg_status energy_variant_check()
{
    if (g_di.prm.oscillate_topbot) {
        set_error("wave_energy's OSCILLATE_TOPBOT branch reads outside its tables (wave_energy.c:799-800); not supported");
        return WG_ERR_INVALID;
    }
    if (g_di.prm.ny < 6) { set_error("wave_energy stepper needs NY >= 6"); return WG_ERR_INVALID; }
    return WG_OK;
}

static wg_status di_energy_update(int in, int prev, int out)
{
    g_di.time++;
    launch_step_exact_energy(g_di.dp, g_di.buf[in], g_di.buf[prev], g_di.buf[out], g_di.xy, g_di.time, g_di.st);
    WG_CUDA(cudaGetLastError());
    return WG_OK;
}

wg_status wg_evolve_wave_half_energy(double **phi_in, double **psi_in, double **phi_out, int16_t **xy_in)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    wg_status s = di_require();
    if (s || (s = energy_variant_check())) return s;
    if (!phi_in || !psi_in || !phi_out || phi_in == phi_out || psi_in == phi_out) {
        set_error("phi_out must be a third array");
        return WG_ERR_INVALID;
    }
    if ((s = di_statics(xy_in, nullptr, nullptr, nullptr, false))) return s;
    bool f0, f1, f2;
    const int a = di_slot(phi_in, 0, &f0), b = di_slot(psi_in, 1, &f1), c = di_slot(phi_out, 2, &f2);
    if (a < 0 || b < 0 || c < 0) { set_error("too many field arrays"); return WG_ERR_STATE; }
    if (f0 && (s = di_upload_rows<double>(phi_in, g_di.buf[a]))) return s;
    if (f1 && (s = di_upload_rows<double>(psi_in, g_di.buf[b]))) return s;
    if (f2 && (s = di_upload_rows<double>(phi_out, g_di.buf[c]))) return s;
    if ((s = di_energy_update(a, b, c))) return s;
    if (g_di.mode == WG_DROPIN_STRICT) return di_download_rows(g_di.buf[c], phi_out);
    return WG_OK;
}

wg_status wg_evolve_wave_energy(double **phi, double **psi, double **tmp, int16_t **xy_in)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    wg_status s = di_require();
    if (s || (s = energy_variant_check())) return s;
    if (!phi || !psi || !tmp || phi == psi || phi == tmp || psi == tmp) {
        set_error("phi, psi and tmp must be three distinct arrays");
        return WG_ERR_INVALID;
    }
    if ((s = di_statics(xy_in, nullptr, nullptr, nullptr, false))) return s;
    bool f0, f1, f2;
    const int a = di_slot(phi, 0, &f0), b = di_slot(psi, 1, &f1), c = di_slot(tmp, 2, &f2);
    if (a < 0 || b < 0 || c < 0) { set_error("too many field arrays"); return WG_ERR_STATE; }
    if (f0 && (s = di_upload_rows<double>(phi, g_di.buf[a]))) return s;
    if (f1 && (s = di_upload_rows<double>(psi, g_di.buf[b]))) return s;
    if (f2 && (s = di_upload_rows<double>(tmp, g_di.buf[c]))) return s;
    if ((s = di_energy_update(a, b, c)) || (s = di_energy_update(c, a, b)) || (s = di_energy_update(b, c, a))) return s;
    if (g_di.mode == WG_DROPIN_STRICT) {
        if ((s = di_download_rows(g_di.buf[a], phi)) || (s = di_download_rows(g_di.buf[b], psi)) ||
            (s = di_download_rows(g_di.buf[c], tmp)))
            return s;
    }
    return WG_OK;
}

// energy of the drop-in fields: upload phi/psi (strict) or use the resident copies
static wg_status di_energy_fields(double **phi, double **psi, int16_t **xy, int *a, int *b)
{
    wg_status s = di_require();
    if (s) return s;
    if (!phi || !psi || !xy) { set_error("NULL argument"); return WG_ERR_INVALID; }
    if ((s = di_statics(xy, nullptr, nullptr, nullptr, false))) return s;
    bool f0, f1;
    if (g_di.mode == WG_DROPIN_STRICT) {
        *a = 0; *b = 1;
        if ((s = di_upload_rows<double>(phi, g_di.buf[0])) || (s = di_upload_rows<double>(psi, g_di.buf[1]))) return s;
        return WG_OK;
    }
    *a = di_slot(phi, 0, &f0);
    *b = di_slot(psi, 1, &f1);
    if (*a < 0 || *b < 0) { set_error("too many field arrays"); return WG_ERR_STATE; }
    if (f0 && (s = di_upload_rows<double>(phi, g_di.buf[*a]))) return s;
    if (f1 && (s = di_upload_rows<double>(psi, g_di.buf[*b]))) return s;
    return WG_OK;
}

wg_status wg_compute_energy(double **phi, double **psi, int16_t **xy_in, int32_t i, int32_t j, double *out)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    int a, b;
    wg_status s = di_energy_fields(phi, psi, xy_in, &a, &b);
    if (s) return s;
    if (!out || i < 0 || j < 0 || i >= g_di.prm.nx || j >= g_di.prm.ny) { set_error("cell out of range"); return WG_ERR_INVALID; }
    launch_cell_energy(g_di.dp, g_di.buf[a], g_di.buf[b], g_di.xy, i, j, g_di.eout, g_di.st);
    WG_CUDA(cudaGetLastError());
    WG_CUDA(cudaMemcpyAsync(g_di.hout, g_di.eout, sizeof(double), cudaMemcpyDeviceToHost, g_di.st));
    WG_CUDA(cudaStreamSynchronize(g_di.st));
    *out = g_di.hout[0];
    return WG_OK;
}

static wg_status di_energy_all(double **phi, double **psi, int16_t **xy, int ileft, int iright)
{
    int a, b;
    wg_status s = di_energy_fields(phi, psi, xy, &a, &b);
    if (s) return s;
    launch_energy<double>(g_di.dp, g_di.buf[a], g_di.buf[b], g_di.xy, nullptr, g_di.ebot, g_di.etop, ileft, iright,
                          g_di.eout, g_di.st);
    WG_CUDA(cudaGetLastError());
    WG_CUDA(cudaMemcpyAsync(g_di.hout, g_di.eout, sizeof(double) * (g_di.prm.nx + 7), cudaMemcpyDeviceToHost, g_di.st));
    WG_CUDA(cudaStreamSynchronize(g_di.st));
    return WG_OK;
}

wg_status wg_compute_energy_x_all(double **phi, double **psi, int16_t **xy_in, double *out)
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    if (!out) { set_error("out is NULL"); return WG_ERR_INVALID; }
    wg_status s = di_energy_all(phi, psi, xy_in, 0, 0);
    if (s) return s;
    memcpy(out, g_di.hout + 7, sizeof(double) * g_di.prm.nx);
    return WG_OK;
}

wg_status wg_compute_energy_tblr(double **phi, double **psi, int16_t **xy_in, int32_t ileft, int32_t iright,
                                 double energies[6])
{
    std::lock_guard<std::mutex> lk(g_di_mu);
    if (!energies) { set_error("energies is NULL"); return WG_ERR_INVALID; }
    wg_status s = di_energy_all(phi, psi, xy_in, ileft, iright);
    if (s) return s;
    memcpy(energies, g_di.hout + 1, sizeof(double) * 6);
    return WG_OK;
}

}  // extern "C"
