// wg_scene.cu — native scene handles: fields resident in HBM in FP64 (phi, psi; in-place
// leapfrog, the new level overwriting psi) or FP32 (phi and the velocity phi - psi, each
// update writing the other pair of fields), 1-bit masks, optional coefficient tables,
// temporal blocking, energy diagnostics and colour-mapped frames.
#include <cuda.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "wg_internal.h"
#include "wg_scene.h"

using namespace wg;

namespace wg {

// Device address of host memory that kernels can read and write in place: page-locked
// memory mapped into the device's address space (cudaHostAlloc, cudaMallocHost or
// cudaHostRegister) whose allocation covers [p, p + bytes).  nullptr for pageable memory,
// or when the driver cannot tell the allocation's range.  The range comes from the
// driver's pointer attributes, reached through the runtime's entry-point query (the
// library does not link libcuda itself).
void *mapped_host(const void *p, size_t bytes)
{
    typedef CUresult (*PfnPtrAttr)(void *, CUpointer_attribute, CUdeviceptr);
    static PfnPtrAttr attr = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        cudaGetLastError();
        return (PfnPtrAttr)f;
    }();
    if (!p || !bytes || !attr) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    CUdeviceptr start = 0;
    size_t size = 0;
    if (attr(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, (CUdeviceptr)(uintptr_t)p) != CUDA_SUCCESS ||
        attr(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, (CUdeviceptr)(uintptr_t)p) != CUDA_SUCCESS)
        return nullptr;
    const uintptr_t b = (uintptr_t)p;
    if (b < (uintptr_t)start || b - (uintptr_t)start > size || bytes > size - (b - (uintptr_t)start)) return nullptr;
    // the last byte must be reachable at the same offset from the device address
    cudaPointerAttributes z;
    if (cudaPointerGetAttributes(&z, (const char *)p + bytes - 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (z.type != cudaMemoryTypeHost || (char *)z.devicePointer != (char *)a.devicePointer + bytes - 1) return nullptr;
    return a.devicePointer;
}

wg_status scene_alloc_dense_stage(wg_scene *s, size_t bytes)
{
    if (s->dstage_bytes >= bytes) return WG_OK;
    if (s->dstage) cudaFree(s->dstage);
    s->dstage = nullptr;
    s->dstage_bytes = 0;
    WG_CUDA(cudaMalloc(&s->dstage, bytes));
    s->dstage_bytes = bytes;
    return WG_OK;
}

size_t scene_device_bytes(const wg_params &p, int prec, int coef)
{
    const size_t esz = prec == WG_FP32 ? 4 : 8;
    const size_t pitch = pitch_for(p.ny, (int)esz), wp = (pitch + 31) / 32;
    size_t b = 2 * (size_t)p.nx * pitch * esz;          // phi, psi
    b += 2 * (size_t)p.nx * wp * 4;                     // act, nz planes
    if (coef == WG_COEF_TABLE) {
        b += (size_t)p.nx * pitch * esz;                // tcc
        if (p.b_cond == WG_BC_ABSORBING || p.b_cond == WG_BC_VPER_HABS) b += (size_t)p.nx * pitch * esz;  // tc
    }
    if (prec == WG_FP32) b += 2 * (size_t)p.nx * pitch * esz;  // FP32: the output pair of every update
    b += (size_t)p.nx * 2 * sizeof(double2) + (p.nx + 8) * sizeof(double) + 64;  // energy scratch
    return b;
}

// Upload a dense [nx][ny] FP64 host array into a pitched field of the scene precision.
static wg_status upload_f64(wg_scene *s, const double *h, void *dev)
{
    const size_t n = (size_t)s->prm.nx * s->prm.ny;
    wg_status st = scene_alloc_dense_stage(s, n * sizeof(double));
    if (st) return st;
    WG_CUDA(cudaMemcpyAsync(s->dstage, h, n * sizeof(double), cudaMemcpyHostToDevice, s->st));
    if (s->prec == WG_FP32) launch_convert_in<float>(s->prm.nx, s->prm.ny, s->pitch, (const double *)s->dstage, (float *)dev, s->st);
    else launch_convert_in<double>(s->prm.nx, s->prm.ny, s->pitch, (const double *)s->dstage, (double *)dev, s->st);
    WG_CUDA(cudaGetLastError());
    WG_CUDA(cudaStreamSynchronize(s->st));  // the host array may be freed after return
    return WG_OK;
}

static wg_status flag_copy(wg_scene *s);
static wg_status flag_result(wg_scene *s);

// FP32 scene state from host (phi, psi) rows of H (double or float), phi and the velocity
// phi - psi formed on the device.  Page-locked mapped rows are read in place by the
// forming kernel, at the host link's rate (a copy engine reaches the same rate, and a
// staged copy adds a pass over HBM); other rows are staged contiguously first.  sync: wait
// for the reads (the host arrays may then be freed or changed).
template <class H>
static wg_status upload_state32(wg_scene *s, const H *phi, const H *psi, bool sync)
{
    const size_t n = (size_t)s->prm.nx * s->prm.ny, bytes = n * sizeof(H);
    const H *mphi = (const H *)mapped_host(phi, bytes), *mpsi = (const H *)mapped_host(psi, bytes);
    if (mphi && mpsi) {
        launch_state_in32<H>(s->prm.nx, s->prm.ny, s->pitch, mphi, mpsi, (float *)s->f[s->cur],
                             (float *)s->f[1 - s->cur], s->st);
    } else {
        wg_status st = scene_alloc_dense_stage(s, 2 * bytes);
        if (st) return st;
        H *stage = (H *)s->dstage;
        WG_CUDA(cudaMemcpyAsync(stage, phi, bytes, cudaMemcpyHostToDevice, s->st));
        WG_CUDA(cudaMemcpyAsync(stage + n, psi, bytes, cudaMemcpyHostToDevice, s->st));
        launch_state_in32<H>(s->prm.nx, s->prm.ny, s->pitch, stage, stage + n, (float *)s->f[s->cur],
                             (float *)s->f[1 - s->cur], s->st);
    }
    s->launches++;
    WG_CUDA(cudaGetLastError());
    if (sync) WG_CUDA(cudaStreamSynchronize(s->st));
    return WG_OK;
}

// FP32 scene state to host (phi, psi) rows of H; either pointer may be NULL.  Page-locked
// mapped rows are written in place by the forming kernel; other rows through a stage.
template <class H>
static wg_status download_state32(wg_scene *s, H *phi, H *psi)
{
    const size_t n = (size_t)s->prm.nx * s->prm.ny, bytes = n * sizeof(H);
    wg_status st;
    H *mphi = phi ? (H *)mapped_host(phi, bytes) : nullptr, *mpsi = psi ? (H *)mapped_host(psi, bytes) : nullptr;
    if ((!phi || mphi) && (!psi || mpsi)) {
        launch_state_out32<H>(s->prm.nx, s->prm.ny, s->pitch, (const float *)s->f[s->cur],
                              (const float *)s->f[1 - s->cur], mphi, mpsi, s->st);
        s->launches++;
        WG_CUDA(cudaGetLastError());
    } else {
        if ((st = scene_alloc_dense_stage(s, 2 * bytes))) return st;
        H *stage = (H *)s->dstage;
        launch_state_out32<H>(s->prm.nx, s->prm.ny, s->pitch, (const float *)s->f[s->cur],
                              (const float *)s->f[1 - s->cur], phi ? stage : nullptr, psi ? stage + n : nullptr, s->st);
        s->launches++;
        WG_CUDA(cudaGetLastError());
        if (phi) WG_CUDA(cudaMemcpyAsync(phi, stage, bytes, cudaMemcpyDeviceToHost, s->st));
        if (psi) WG_CUDA(cudaMemcpyAsync(psi, stage + n, bytes, cudaMemcpyDeviceToHost, s->st));
    }
    if ((st = flag_copy(s))) return st;
    WG_CUDA(cudaStreamSynchronize(s->st));
    return flag_result(s);
}

static wg_status download_f64(wg_scene *s, const void *dev, double *h)
{
    const size_t n = (size_t)s->prm.nx * s->prm.ny;
    wg_status st = scene_alloc_dense_stage(s, n * sizeof(double));
    if (st) return st;
    if (s->prec == WG_FP32) launch_convert_out<float>(s->prm.nx, s->prm.ny, s->pitch, (const float *)dev, (double *)s->dstage, s->st);
    else launch_convert_out<double>(s->prm.nx, s->prm.ny, s->pitch, (const double *)dev, (double *)s->dstage, s->st);
    WG_CUDA(cudaGetLastError());
    WG_CUDA(cudaMemcpyAsync(h, s->dstage, n * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    WG_CUDA(cudaStreamSynchronize(s->st));
    return WG_OK;
}

template <class T>
static FastArgs<T> fast_args(wg_scene *s, int do_source)
{
    FastArgs<T> a;
    a.phi = (const T *)s->f[s->cur];
    a.psi = (const T *)s->f[1 - s->cur];
    const bool pair = sizeof(T) == 4;  // FP32: the new phi and velocity go to the other pair
    a.out = (T *)(pair ? s->g[0] : s->f[1 - s->cur]);
    a.vout = pair ? (T *)s->g[1] : nullptr;
    a.act = s->act;
    a.nz = s->nz;
    a.tcc = (const T *)s->tcc;
    a.tc = (const T *)s->tc;
    a.tg = (const T *)s->tg;
    a.c2f = (float)s->dp.c2;
    a.c2bf = (float)s->dp.c2b;
    a.gamf = (float)s->dp.gam;
    a.gambf = (float)s->dp.gamb;
    a.kappaf = (float)s->dp.kappa;
    a.courantf = (float)s->dp.courant;
    a.courantbf = (float)s->dp.courantb;
    a.ksf = (float)s->dp.kappa_sides;
    a.ktf = (float)s->dp.kappa_topbot;
    a.gsf = (float)s->dp.gamma_sides;
    a.gtf = (float)s->dp.gamma_topbot;
    a.vmaxf = (float)s->dp.vmax;
    a.has_ghosts = s->has_ghosts;
    a.do_source = do_source;
    return a;
}

// One update of the single-step form (k_step_bulk + k_step_edge, Neumann gather, source).
template <class T>
static wg_status single_update(wg_scene *s)
{
    s->time++;
    const bool recs = s->nrec > 0;
    FastArgs<T> a = fast_args<T>(s, recs ? 0 : 1);
    launch_step_fast<T>(s->dp, a, s->coef, s->time, s->st);  // k_step_bulk + k_step_edge
    s->launches += 2;
    if (recs) {
        launch_neumann_fast<T>(s->dp, a.phi, a.out, a.vout, s->nidx, s->nw, s->nrec, s->st);
        s->launches++;
        if (s->prm.src_on) {
            launch_point_source<T>(s->dp, a.out, a.vout, s->time, s->st);
            s->launches++;
        }
    }
    if (sizeof(T) == 4) {  // the output pair becomes the scene's state
        std::swap(s->f[s->cur], s->g[0]);
        std::swap(s->f[1 - s->cur], s->g[1]);
    } else {
        s->cur = 1 - s->cur;
    }
    return WG_OK;
}

template <class T>
wg_status scene_step_impl(wg_scene *s, int nsteps)
{
    if (s->probe_n && s->probe_count + nsteps > s->probe_cap) {
        set_error("probe buffer full: %d of %d updates recorded; read them first", s->probe_count, s->probe_cap);
        return WG_ERR_STATE;
    }
    const int k = s->tb_k;
    const bool tb = k > 1 && tb_supported(s) && !s->probe_n;  // probes sample every update
    if (tb) {
        wg_status st = tb_prepare(s, nsteps);
        if (st) return st;
    }
    while (nsteps > 0) {
        const int d = tb ? tb_pass_depth(k, nsteps) : 0;
        if (d >= 2) {
            wg_status st = tb_pass<T>(s, d);
            if (st) return st;
            nsteps -= d;
        } else {
            wg_status st = single_update<T>(s);
            if (st) return st;
            probe_record(s);
            nsteps--;
        }
    }
    WG_CUDA(cudaGetLastError());
    return WG_OK;
}
template wg_status scene_step_impl<float>(wg_scene *, int);

// The flag a kernel sets when one of its bounded waits gave up: copied into the last slot
// of the pinned report buffer in stream order (flag_copy), read after the caller's
// synchronisation (flag_result), so a download or a sync pays one synchronisation.
static int *flag_slot(wg_scene *s) { return reinterpret_cast<int *>(s->hout + s->prm.nx + 7); }
static wg_status flag_copy(wg_scene *s)
{
    WG_CUDA(cudaMemcpyAsync(flag_slot(s), s->dflag, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    return WG_OK;
}
static wg_status flag_result(wg_scene *s)
{
    if (*flag_slot(s)) {
        *flag_slot(s) = 0;
        WG_CUDA(cudaMemsetAsync(s->dflag, 0, sizeof(int), s->st));
        set_error("a tile load did not complete within its bounded wait; the last step is invalid");
        return WG_ERR_TIMEOUT;
    }
    return WG_OK;
}

// Synchronises the scene's stream and reads (and clears) the flag, one synchronisation.
wg_status scene_check_flag(wg_scene *s)
{
    if (wg_status st = flag_copy(s)) return st;
    WG_CUDA(cudaStreamSynchronize(s->st));
    return flag_result(s);
}
template wg_status scene_step_impl<double>(wg_scene *, int);

}  // namespace wg

extern "C" {

wg_status wg_scene_bytes(const wg_params *p, int32_t precision, int32_t coef_mode, size_t *bytes)
{
    if (!p || !bytes) { set_error("NULL argument"); return WG_ERR_INVALID; }
    *bytes = scene_device_bytes(*p, precision, coef_mode);
    return WG_OK;
}

wg_status wg_scene_create(const wg_params *p, int32_t precision, int32_t coef_mode, void *stream, wg_scene **out)
{
    if (!p || !out) { set_error("NULL argument"); return WG_ERR_INVALID; }
    *out = nullptr;
    wg_status st = validate_params(*p);
    if (st) return st;
    if (precision != WG_FP32 && precision != WG_FP64) { set_error("precision must be WG_FP32 or WG_FP64"); return WG_ERR_INVALID; }
    if (coef_mode != WG_COEF_MASK && coef_mode != WG_COEF_TABLE) { set_error("unknown coefficient mode"); return WG_ERR_INVALID; }
    wg_scene *s = new wg_scene();
    s->prm = *p;
    s->prec = precision;
    s->coef = coef_mode;
    s->esz = precision == WG_FP32 ? 4 : 8;
    s->pitch = pitch_for(p->ny, (int)s->esz);
    s->dp = make_dev_params(*p, s->pitch);
    if (stream) s->st = (cudaStream_t)stream;
    else {
        cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete s; return cuda_fail(e, "cudaStreamCreate"); }
        s->own_stream = true;
    }
    const size_t fb = (size_t)p->nx * s->pitch * s->esz, mb = (size_t)p->nx * s->dp.wpitch * 4;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 2 && e == cudaSuccess; k++) {
        e = cudaMalloc(&s->f[k], fb);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->f[k], 0, fb, s->st);
        if (e == cudaSuccess && precision == WG_FP32) e = cudaMalloc(&s->g[k], fb);
        if (e == cudaSuccess && precision == WG_FP32) e = cudaMemsetAsync(s->g[k], 0, fb, s->st);
    }
    if (e == cudaSuccess) e = cudaMalloc(&s->act, mb);
    if (e == cudaSuccess) e = cudaMalloc(&s->nz, mb);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->act, 0, mb, s->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->nz, 0, mb, s->st);
    if (e == cudaSuccess && coef_mode == WG_COEF_TABLE) {
        e = cudaMalloc(&s->tcc, fb);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->tcc, 0, fb, s->st);
        if (e == cudaSuccess && (p->b_cond == WG_BC_ABSORBING || p->b_cond == WG_BC_VPER_HABS)) {
            e = cudaMalloc(&s->tc, fb);
            if (e == cudaSuccess) e = cudaMemsetAsync(s->tc, 0, fb, s->st);
        }
    }
    if (e == cudaSuccess) e = cudaMalloc(&s->ebot, p->nx * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&s->etop, p->nx * sizeof(double2));
    if (e == cudaSuccess) e = cudaMalloc(&s->eout, (p->nx + 8) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->dcount, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&s->dflag, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(s->dflag, 0, sizeof(int), s->st);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->hout, (p->nx + 8) * sizeof(double), cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) {
        wg_status r = cuda_fail(e, "wg_scene_create");
        wg_scene_destroy(s);
        return r;
    }
    s->tb_k = 0;  // autotuned at first step
    *out = s;
    return WG_OK;
}

wg_status wg_scene_destroy(wg_scene *s)
{
    if (!s) return WG_OK;
    if (s->st) cudaStreamSynchronize(s->st);
    for (auto &f : s->f) if (f) cudaFree(f);
    for (auto &g : s->g) if (g) cudaFree(g);
    void *dev[] = {s->act, s->nz, s->tcc, s->tc, s->tg, s->nidx, s->nw, s->ebot, s->etop, s->eout, s->dcount,
                   s->dstage, s->rgb, s->lut, s->bv_osc, s->bv_src, s->dflag, s->facc, s->probe_cells, s->probe_buf,
                   s->nrec_dev};
    for (void *d : dev) if (d) cudaFree(d);
    for (auto &c : s->skew) if (c.dev) cudaFree(c.dev);
    if (s->hout) cudaFreeHost(s->hout);
    if (s->hstage) cudaFreeHost(s->hstage);
    if (s->own_stream && s->st) cudaStreamDestroy(s->st);
    delete s;
    return WG_OK;
}

wg_status wg_scene_upload(wg_scene *s, const double *phi, const double *psi, const int16_t *xy, const double *tcc,
                          const double *tc, const double *tgamma)
{
    if (!s || !phi || !psi || !xy) { set_error("NULL argument"); return WG_ERR_INVALID; }
    const int nx = s->prm.nx, ny = s->prm.ny;
    const size_t n = (size_t)nx * ny;
    // mask: validate and pack into the two bit planes
    int has_neg = 0;
    for (size_t c = 0; c < n; c++) {
        if (xy[c] < 0) has_neg = 1;
        if (s->coef == WG_COEF_MASK && xy[c] != 0 && xy[c] != 1) {
            set_error("mask value %d at cell %zu: WG_COEF_MASK takes masks of 0/1 (use WG_COEF_TABLE)", (int)xy[c], c);
            return WG_ERR_INVALID;
        }
    }
    s->has_ghosts = has_neg;
    s->xy_host.assign(xy, xy + n);
    wg_status st = scene_alloc_dense_stage(s, n * sizeof(double));
    if (st) return st;
    WG_CUDA(cudaMemcpyAsync(s->dstage, xy, n * sizeof(int16_t), cudaMemcpyHostToDevice, s->st));
    launch_pack_mask(nx, ny, s->dp.wpitch, (const int16_t *)s->dstage, s->act, s->nz, s->st);
    WG_CUDA(cudaGetLastError());
    WG_CUDA(cudaStreamSynchronize(s->st));
    if (s->coef == WG_COEF_TABLE) {
        if (!tcc || !tgamma) { set_error("WG_COEF_TABLE needs tcc and tgamma"); return WG_ERR_INVALID; }
        if (s->tc && !tc) { set_error("tc table needed with an absorbing boundary"); return WG_ERR_INVALID; }
        if ((st = upload_f64(s, tcc, s->tcc))) return st;
        if (s->tc && (st = upload_f64(s, tc, s->tc))) return st;
        // tgamma: a scalar when it is the same on every cell the stepper writes
        bool uniform = true;
        double g0 = 0.0;
        bool have = false;
        for (int i = 0; i < nx && uniform; i++)
            for (int j = 0; j < ny; j++) {
                const size_t c = (size_t)i * ny + j;
                const bool edge = (i == 0 || i == nx - 1 || j == 0 || j == ny - 1);
                const bool used = s->prm.twospeeds || (edge ? xy[c] != 0 : xy[c] > 0);
                if (!used) continue;
                if (!have) { g0 = tgamma[c]; have = true; }
                else if (tgamma[c] != g0) { uniform = false; break; }
            }
        if (s->tg) { cudaFree(s->tg); s->tg = nullptr; }
        if (uniform) {
            s->dp.gam = g0;
            s->dp.gamb = g0;
        } else {
            WG_CUDA(cudaMalloc(&s->tg, (size_t)nx * s->pitch * s->esz));
            if ((st = upload_f64(s, tgamma, s->tg))) return st;
        }
    }
    s->cur = 0;
    if (s->prec == WG_FP32) {
        if ((st = upload_state32<double>(s, phi, psi, true))) return st;
    } else {
        if ((st = upload_f64(s, phi, s->f[0]))) return st;
        if ((st = upload_f64(s, psi, s->f[1]))) return st;
    }
    s->time = 0;
    s->uploaded = true;
    s->has_mask = true;
    return WG_OK;
}

wg_status wg_scene_upload_state(wg_scene *s, const void *phi, const void *psi, int32_t host_precision)
{
    if (!s || !phi || !psi) { set_error("NULL argument"); return WG_ERR_INVALID; }
    const int nx = s->prm.nx, ny = s->prm.ny;
    void *dst[2] = {s->f[s->cur], s->f[1 - s->cur]};
    const void *src[2] = {phi, psi};
    if (!s->has_mask) { set_error("upload or build the mask first"); return WG_ERR_STATE; }
    if (host_precision != WG_FP32 && host_precision != WG_FP64) { set_error("unknown host precision"); return WG_ERR_INVALID; }
    s->uploaded = true;
    if (s->prec == WG_FP32) {  // stream-ordered for FP32 host rows, as for same-precision copies below
        if (host_precision == WG_FP32) return upload_state32<float>(s, (const float *)phi, (const float *)psi, false);
        return upload_state32<double>(s, (const double *)phi, (const double *)psi, true);
    }
    if (host_precision == s->prec) {
        // contiguous copies (faster over the host link than row-pitched ones) into the dense
        // stage, then a repack into the pitched fields on the device
        const size_t bytes = (size_t)nx * ny * s->esz;
        if (wg_status st = scene_alloc_dense_stage(s, 2 * bytes)) return st;
        char *stage = (char *)s->dstage;
        for (int k = 0; k < 2; k++) {
            WG_CUDA(cudaMemcpyAsync(stage + k * bytes, src[k], bytes, cudaMemcpyHostToDevice, s->st));
            if (s->prec == WG_FP32)
                launch_repack_in<float>(nx, ny, s->pitch, (const float *)(stage + k * bytes), (float *)dst[k], s->st);
            else
                launch_repack_in<double>(nx, ny, s->pitch, (const double *)(stage + k * bytes), (double *)dst[k], s->st);
            s->launches++;
        }
        WG_CUDA(cudaGetLastError());
        return WG_OK;  // stream-ordered; the host buffers must stay valid until the next sync
    }
    if (host_precision == WG_FP64) {
        for (int k = 0; k < 2; k++) {
            wg_status st = upload_f64(s, (const double *)src[k], dst[k]);
            if (st) return st;
        }
        return WG_OK;
    }
    set_error("FP32 host state for an FP64 scene: upload FP64 values");
    return WG_ERR_INVALID;
}

wg_status wg_scene_download(wg_scene *s, void *phi, void *psi, int32_t host_precision)
{
    if (!s) { set_error("NULL scene"); return WG_ERR_INVALID; }
    const int nx = s->prm.nx, ny = s->prm.ny;
    if (s->prec == WG_FP32) {
        wg_status st;
        if (host_precision == WG_FP32) st = download_state32<float>(s, (float *)phi, (float *)psi);
        else if (host_precision == WG_FP64) st = download_state32<double>(s, (double *)phi, (double *)psi);
        else { set_error("download precision must be FP64 or the scene's"); return WG_ERR_INVALID; }
        return st;
    }
    const void *src[2] = {s->f[s->cur], s->f[1 - s->cur]};
    void *dst[2] = {phi, psi};
    for (int k = 0; k < 2; k++) {
        if (!dst[k]) continue;
        if (host_precision == s->prec) {
            WG_CUDA(cudaMemcpy2DAsync(dst[k], ny * s->esz, src[k], s->pitch * s->esz, ny * s->esz, nx,
                                      cudaMemcpyDeviceToHost, s->st));
        } else if (host_precision == WG_FP64) {
            wg_status st = download_f64(s, src[k], (double *)dst[k]);
            if (st) return st;
        } else {
            set_error("download precision must be FP64 or the scene's");
            return WG_ERR_INVALID;
        }
    }
    return scene_check_flag(s);  // one synchronisation for the copies and the flag
}

wg_status wg_scene_set_neumann(wg_scene *s, const wg_neumann_bc *r, int32_t n)
{
    if (!s) { set_error("NULL scene"); return WG_ERR_INVALID; }
    if (!s->prm.bc_neumann) { s->nrec = 0; return WG_OK; }
    if (n < 0 || (n > 0 && !r)) { set_error("bad records"); return WG_ERR_INVALID; }
    if (s->xy_host.empty()) { set_error("upload the mask before the Neumann records"); return WG_ERR_STATE; }
    std::vector<int4> idx;
    std::vector<double2> w;
    const int nx = s->prm.nx, ny = s->prm.ny, P = s->pitch;
    for (int q = 0; q < n; q++) {
        if (!r[q].active) continue;
        if (r[q].i < 1 || r[q].i > nx - 2 || r[q].j < 1 || r[q].j > ny - 2 || r[q].nbi1 < 0 || r[q].nbi1 >= nx ||
            r[q].nbj1 < 0 || r[q].nbj1 >= ny || r[q].nbi2 < 0 || r[q].nbi2 >= nx || r[q].nbj2 < 0 || r[q].nbj2 >= ny) {
            set_error("Neumann record %d outside 1..NX-2 x 1..NY-2", q);
            return WG_ERR_INVALID;
        }
        const int nzc = s->xy_host[(size_t)r[q].i * ny + r[q].j] != 0;
        idx.push_back(make_int4(r[q].i * P + r[q].j, r[q].nbi1 * P + r[q].nbj1, r[q].nbi2 * P + r[q].nbj2, nzc));
        w.push_back(make_double2(r[q].nx, r[q].ny));
    }
    if (s->nidx) cudaFree(s->nidx);
    if (s->nw) cudaFree(s->nw);
    if (s->nrec_dev) cudaFree(s->nrec_dev);
    s->nidx = nullptr;
    s->nw = nullptr;
    s->nrec_dev = nullptr;
    s->nrec_all = n;
    s->nrec = (int)idx.size();
    if (s->nrec) {
        WG_CUDA(cudaMalloc(&s->nidx, sizeof(int4) * idx.size()));
        WG_CUDA(cudaMalloc(&s->nw, sizeof(double2) * w.size()));
        WG_CUDA(cudaMemcpyAsync(s->nidx, idx.data(), sizeof(int4) * idx.size(), cudaMemcpyHostToDevice, s->st));
        WG_CUDA(cudaMemcpyAsync(s->nw, w.data(), sizeof(double2) * w.size(), cudaMemcpyHostToDevice, s->st));
        WG_CUDA(cudaStreamSynchronize(s->st));
    }
    return WG_OK;
}

wg_status wg_scene_step(wg_scene *s, int32_t nsteps)
{
    if (!s) { set_error("NULL scene"); return WG_ERR_INVALID; }
    if (!s->uploaded) { set_error("upload the scene before stepping"); return WG_ERR_STATE; }
    if (nsteps < 0) { set_error("negative step count"); return WG_ERR_INVALID; }
    if (s->tb_k == 0) autotune_scene(s);
    return s->prec == WG_FP32 ? scene_step_impl<float>(s, nsteps) : scene_step_impl<double>(s, nsteps);
}

wg_status wg_scene_energy(wg_scene *s, double *total, double *columns, int32_t ileft, int32_t iright, double *boxes)
{
    if (!s) { set_error("NULL scene"); return WG_ERR_INVALID; }
    const void *phi = s->f[s->cur], *psi = s->f[1 - s->cur];
    if (s->prec == WG_FP32)
        launch_energy<float>(s->dp, (const float *)phi, (const float *)psi, nullptr, s->nz, s->ebot, s->etop, ileft,
                             iright, s->eout, s->st);
    else
        launch_energy<double>(s->dp, (const double *)phi, (const double *)psi, nullptr, s->nz, s->ebot, s->etop, ileft,
                              iright, s->eout, s->st);
    s->launches += 2;
    WG_CUDA(cudaGetLastError());
    const size_t nout = columns ? (size_t)s->prm.nx + 7 : 7;
    WG_CUDA(cudaMemcpyAsync(s->hout, s->eout, nout * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    // the bounded-wait flag rides in the last slot of the same pinned buffer: one sync
    int *hflag = reinterpret_cast<int *>(s->hout + s->prm.nx + 7);
    WG_CUDA(cudaMemcpyAsync(hflag, s->dflag, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    WG_CUDA(cudaStreamSynchronize(s->st));
    if (*hflag) {
        WG_CUDA(cudaMemsetAsync(s->dflag, 0, sizeof(int), s->st));
        set_error("a tile load did not complete within its bounded wait; the last step is invalid");
        return WG_ERR_TIMEOUT;
    }
    if (total) *total = s->hout[0];
    if (boxes) memcpy(boxes, s->hout + 1, 6 * sizeof(double));
    if (columns) memcpy(columns, s->hout + 7, s->prm.nx * sizeof(double));
    return WG_OK;
}

wg_status wg_scene_get_time(wg_scene *s, int64_t *t)
{
    if (!s || !t) return WG_ERR_INVALID;
    *t = s->time;
    return WG_OK;
}

wg_status wg_scene_set_time(wg_scene *s, int64_t t)
{
    if (!s) return WG_ERR_INVALID;
    s->time = t;
    return WG_OK;
}

wg_status wg_scene_sync(wg_scene *s)
{
    if (!s) return WG_ERR_INVALID;
    WG_CUDA(cudaStreamSynchronize(s->st));
    return scene_check_flag(s);
}

wg_status wg_scene_set_blocking(wg_scene *s, int32_t k, int32_t tile_i, int32_t tile_j)
{
    if (!s || k < 0 || k > WG_TB_MAX_K) { set_error("temporal block depth must be 0..%d", WG_TB_MAX_K); return WG_ERR_INVALID; }
    if (tile_j != 0 && tile_j != 1 && tile_j != 128 && tile_j != 256) {
        set_error("tile width must be 1 (skewed strips), 128 or 256");
        return WG_ERR_INVALID;
    }
    if (tile_j == 1 && (tile_i < 8 || tile_i > 4096 || k > 6)) { set_error("skewed strips: 8..4096 rows, depth <= 6"); return WG_ERR_INVALID; }
    if (tile_j > 1 && tile_i != 0 && (tile_i < 16 || tile_i > 64 || tile_i - 2 * k < 8)) {
        set_error("tile height must be 16..64 with at least 8 core rows");
        return WG_ERR_INVALID;
    }
    s->tb_k = k;                 // 0: autotuned at the next step
    s->tile_i = k > 1 ? (tile_i ? tile_i : 32) : 0;
    s->tile_j = k > 1 ? (tile_j ? tile_j : 256) : 0;
    return WG_OK;
}

wg_status wg_scene_get_blocking(wg_scene *s, int32_t *k, int32_t *tile_i, int32_t *tile_j)
{
    if (!s) return WG_ERR_INVALID;
    if (s->tb_k == 0 && s->uploaded) autotune_scene(s);
    if (k) *k = s->tb_k;
    if (tile_i) *tile_i = s->tile_i;
    if (tile_j) *tile_j = s->tile_j;
    return WG_OK;
}

wg_status wg_scene_launch_count(wg_scene *s, int64_t *n)
{
    if (!s || !n) return WG_ERR_INVALID;
    *n = s->launches;
    return WG_OK;
}

wg_status wg_scene_check_finite(wg_scene *s, int64_t *bad)
{
    if (!s || !bad) return WG_ERR_INVALID;
    WG_CUDA(cudaMemsetAsync(s->dcount, 0, sizeof(unsigned long long), s->st));
    if (s->prec == WG_FP32) launch_count_nonfinite<float>(s->prm.nx, s->prm.ny, s->pitch, (const float *)s->f[s->cur], s->dcount, s->st);
    else launch_count_nonfinite<double>(s->prm.nx, s->prm.ny, s->pitch, (const double *)s->f[s->cur], s->dcount, s->st);
    s->launches++;
    WG_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    WG_CUDA(cudaMemcpyAsync(&h, s->dcount, sizeof h, cudaMemcpyDeviceToHost, s->st));
    WG_CUDA(cudaStreamSynchronize(s->st));
    *bad = (int64_t)h;
    return WG_OK;
}

}  // extern "C"
