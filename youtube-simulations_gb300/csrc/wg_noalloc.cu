// wg_noalloc.cu — energy diagnostics that allocate nothing.
//
// For callers that cannot allocate device memory when they need the diagnostics
// (their device memory is all taken by their own arena, or they must not call
// cudaMalloc while serving).  The caller passes the fields and the output in device
// memory; the per-column partial sums live in a fixed file-scope device array.
//
// Notes for users:
//  * The scratch holds WG_NOALLOC_MAX_NX columns; a larger nx is refused.
//  * The first call in a CUDA context (with that device current) looks up the array's
//    address with cudaGetSymbolAddress; make that first call before any stream capture.
//    A new context on the device (e.g. after cudaDeviceReset) takes a new lookup.
//  * Every call uses the same array, which keeps the last call's contents.  Nothing in
//    it has to start at zero: each call writes every column's partials before reading
//    them.  Calls that overlap on the GPU (different streams, unordered) race on it.
#include <cuda.h>
#include <mutex>
#include "wg_internal.h"

namespace wg {

static __device__ __align__(256) double2 g_energy_scratch[2 * WG_NOALLOC_MAX_NX];

// The array's device address belongs to the module loaded into one CUDA context; a new
// context on the same device (after cudaDeviceReset, or a context the caller made)
// loads the module again and the array can move.  So the address is cached per
// context, keyed by the context's unique id (cuCtxGetId), and looked up again for a
// context not seen before.  The driver calls are reached through the runtime's
// entry-point query, so the library does not link libcuda itself.
typedef CUresult (*PfnCtxGetCurrent)(CUcontext *);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long *);

struct ScratchSlot {
    unsigned long long ctx_id;
    double2 *addr;
};
static std::mutex g_scratch_mu;
static ScratchSlot g_scratch_slots[64];
static int g_scratch_n = 0, g_scratch_next = 0;
static PfnCtxGetCurrent g_ctx_current = nullptr;
static PfnCtxGetId g_ctx_id = nullptr;

static wg_status driver_entry_points()
{
    if (g_ctx_current && g_ctx_id) return WG_OK;
    void *a = nullptr, *b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa);
    if (e != cudaSuccess || qa != cudaDriverEntryPointSuccess || !a)
        return e != cudaSuccess ? cuda_fail(e, "cudaGetDriverEntryPointByVersion(cuCtxGetCurrent)")
                                : (set_error("cuCtxGetCurrent is not available from the driver"), WG_ERR_CUDA);
    e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb);
    if (e != cudaSuccess || qb != cudaDriverEntryPointSuccess || !b)
        return e != cudaSuccess ? cuda_fail(e, "cudaGetDriverEntryPointByVersion(cuCtxGetId)")
                                : (set_error("cuCtxGetId is not available from the driver"), WG_ERR_CUDA);
    g_ctx_current = (PfnCtxGetCurrent)a;
    g_ctx_id = (PfnCtxGetId)b;
    return WG_OK;
}

// Id of the current context, or 0 when the thread has none yet.
static wg_status current_ctx_id(unsigned long long *id)
{
    CUcontext ctx = nullptr;
    *id = 0;
    CUresult r = g_ctx_current(&ctx);
    if (r != CUDA_SUCCESS) { set_error("cuCtxGetCurrent failed (%d)", (int)r); return WG_ERR_CUDA; }
    if (!ctx) return WG_OK;
    r = g_ctx_id(ctx, id);
    if (r != CUDA_SUCCESS) { set_error("cuCtxGetId failed (%d)", (int)r); return WG_ERR_CUDA; }
    return WG_OK;
}

// Address of the scratch array in the current context (looked up once per context).
static wg_status scratch_in_current_context(double2 **out)
{
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    wg_status st = driver_entry_points();
    if (st) return st;
    unsigned long long id = 0;
    if ((st = current_ctx_id(&id))) return st;
    for (int k = 0; id && k < g_scratch_n; k++)
        if (g_scratch_slots[k].ctx_id == id) { *out = g_scratch_slots[k].addr; return WG_OK; }
    // a context not seen before (or none yet: the lookup makes the device's primary
    // context current, as any runtime call does)
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_energy_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_energy_scratch)");
    if ((st = current_ctx_id(&id))) return st;
    if (!id) { set_error("no current CUDA context after the scratch lookup"); return WG_ERR_CUDA; }
    ScratchSlot &slot = g_scratch_slots[g_scratch_next];
    slot.ctx_id = id;
    slot.addr = (double2 *)ptr;
    g_scratch_next = (g_scratch_next + 1) % 64;
    if (g_scratch_n < 64) g_scratch_n++;
    *out = (double2 *)ptr;
    return WG_OK;
}

}  // namespace wg

using namespace wg;

extern "C" wg_status wg_compute_energy_device_noalloc(const wg_params *p, const double *phi, const double *psi,
                                                      const int16_t *xy, int32_t pitch, int32_t ileft,
                                                      int32_t iright, double *out, void *stream)
{
    if (!p || !phi || !psi || !xy || !out) { set_error("NULL argument"); return WG_ERR_INVALID; }
    wg_status st = validate_params(*p);
    if (st) return st;
    if (p->nx > WG_NOALLOC_MAX_NX) {
        set_error("nx = %d exceeds the fixed scratch of this entry point (at most %d columns)", p->nx,
                  WG_NOALLOC_MAX_NX);
        return WG_ERR_INVALID;
    }
    if (pitch < p->ny) { set_error("pitch %d is smaller than ny %d", pitch, p->ny); return WG_ERR_INVALID; }
    if (ileft < 0 || iright < ileft || iright > p->nx) { set_error("box limits out of range"); return WG_ERR_INVALID; }
    double2 *scratch = nullptr;
    if ((st = scratch_in_current_context(&scratch))) return st;
    const DevParams dp = make_dev_params(*p, pitch);
    launch_energy<double>(dp, phi, psi, xy, nullptr, scratch, scratch + WG_NOALLOC_MAX_NX, ileft, iright, out,
                          (cudaStream_t)stream);
    WG_CUDA(cudaGetLastError());
    return WG_OK;
}
