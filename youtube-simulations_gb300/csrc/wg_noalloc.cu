// wg_noalloc.cu — energy diagnostics that allocate nothing.
//
// For callers that cannot allocate device memory when they need the diagnostics
// (their device memory is all taken by their own arena, or they must not call
// cudaMalloc while serving).  The caller passes the fields and the output in device
// memory; the per-column partial sums live in a fixed file-scope device array.
//
// Notes for users:
//  * The scratch holds WG_NOALLOC_MAX_NX columns; a larger nx is refused.
//  * The first call on a device (with that device current) looks up the array's
//    address with cudaGetSymbolAddress; make that first call before any stream capture.
//  * Every call uses the same array, which keeps the last call's contents.  Nothing in
//    it has to start at zero: each call writes every column's partials before reading
//    them.  Calls that overlap on the GPU (different streams, unordered) race on it.
#include <mutex>
#include "wg_internal.h"

namespace wg {

static __device__ __align__(256) double2 g_energy_scratch[2 * WG_NOALLOC_MAX_NX];

static std::mutex g_scratch_mu;
static double2 *g_scratch_addr[128] = {};  // per device ordinal

// Address of the scratch array on the current device (looked up once per device).
static wg_status scratch_on_current_device(double2 **out)
{
    int dev = 0;
    WG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) { set_error("device ordinal %d out of range", dev); return WG_ERR_INVALID; }
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_energy_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_energy_scratch)");
        g_scratch_addr[dev] = (double2 *)ptr;
    }
    *out = g_scratch_addr[dev];
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
    if ((st = scratch_on_current_device(&scratch))) return st;
    const DevParams dp = make_dev_params(*p, pitch);
    launch_energy<double>(dp, phi, psi, xy, nullptr, scratch, scratch + WG_NOALLOC_MAX_NX, ileft, iright, out,
                          (cudaStream_t)stream);
    WG_CUDA(cudaGetLastError());
    return WG_OK;
}
