// wg_internal.h — declarations shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include "../../include/wavegpu.h"
#include "wg_device.cuh"

namespace wg {

// FP64 fields: phi (level t), psi (level t-1, read at the cell itself only) and out
// (level t+1, == psi: in place).  FP32 fields: phi and the velocity v = phi - psi in psi;
// the update writes the new phi to out and the new velocity to vout (another pair).
template <class T>
struct FastArgs {
    const T *phi;
    const T *psi;
    T *out;
    T *vout;             // FP32 only
    const uint32_t *act; // "active" plane: bulk xy > 0, boundary lines xy != 0
    const uint32_t *nz;  // "nonzero" plane: xy != 0
    const T *tcc, *tc, *tg;  // WG_COEF_TABLE tables (tg may be null: uniform)
    float c2f, c2bf, gamf, gambf, kappaf;
    // the boundary rules' coefficients in FP32, rounded on the host (a conversion from
    // FP64 on the device runs on this GPU's slow FP64 pipe)
    float courantf, courantbf, ksf, ktf, gsf, gtf, vmaxf;
    int has_ghosts;      // the mask has cells < 0 (Neumann ghosts)
    int do_source;       // add the point source in this kernel
};

// Programmatic dependent launch.  A kernel launched by launch_pdl may start while the
// previous kernel in its stream is finishing; it calls pdl_wait() before its first access to
// memory that kernel reads or writes (the wait returns once that kernel has completed and
// its writes are visible), then pdl_trigger() to let the next such kernel launch early.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
template <class... KArgs, class... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args &&>(args)...);
}

// error state (thread-local message)
void set_error(const char *fmt, ...);
void clear_error();
wg_status cuda_fail(cudaError_t e, const char *what);
#define WG_CUDA(call)                                       \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// device address of mapped page-locked host memory covering [p, p + bytes), else nullptr
// (wg_scene.cu)
void *mapped_host(const void *p, size_t bytes);

DevParams make_dev_params(const wg_params &p, int pitch);
wg_status validate_params(const wg_params &p);
int pitch_for(int ny, int elem_bytes);

// launchers (wg_kernels.cu)
void launch_step_exact(const DevParams &p, const double *phi, const double *psi, double *out, const int16_t *xy,
                       const double *tcc, const double *tc, const double *tg, long long time, int do_source,
                       cudaStream_t st);
void launch_step_exact_energy(const DevParams &p, const double *phi, const double *psi, double *out,
                              const int16_t *xy, long long time, cudaStream_t st);
void launch_neumann_exact(const DevParams &p, const double *phi, double *out, const int16_t *xy,
                          const wg_neumann_bc *rec, int n, cudaStream_t st);
template <class T> void launch_point_source(const DevParams &p, T *out, T *vout, long long time, cudaStream_t st);
template <class T> void launch_step_fast(const DevParams &p, const FastArgs<T> &a, int coef_mode, long long time,
                                         cudaStream_t st);
template <class T> void launch_neumann_fast(const DevParams &p, const T *phi, T *out, T *vout, const int4 *idx,
                                            const double2 *w, int n, cudaStream_t st);
template <class T> void launch_energy(const DevParams &p, const T *phi, const T *psi, const int16_t *xy,
                                      const uint32_t *nz, double2 *bot, double2 *top, int ileft, int iright,
                                      double *out, cudaStream_t st);
template <class T> void launch_count_nonfinite(int nx, int ny, int pitch, const T *a, unsigned long long *count,
                                               cudaStream_t st);
void launch_pack_mask(int nx, int ny, int wpitch, const int16_t *xy, uint32_t *act, uint32_t *nz, cudaStream_t st);
template <class T> void launch_convert_in(int nx, int ny, int pitch, const double *src, T *dst, cudaStream_t st);
template <class T> void launch_convert_out(int nx, int ny, int pitch, const T *src, double *dst, cudaStream_t st);
template <class T> void launch_repack_in(int nx, int ny, int pitch, const T *src, T *dst, cudaStream_t st);
// FP32 state (phi, velocity) from and to host (phi, psi) rows of H = double or float
template <class H> void launch_state_in32(int nx, int ny, int pitch, const H *phi, const H *psi, float *x, float *v,
                                          cudaStream_t st);
template <class H> void launch_state_out32(int nx, int ny, int pitch, const float *x, const float *v, H *phi, H *psi,
                                           cudaStream_t st);

// add_circular_wave (wg_pulse.cu): the grid geometry, the pulse and the box of cells to visit
struct PulseArgs {
    int nx, ny, pitch, wpitch, twospeeds;
    int i0, ni, j0, nj;
    double init_amp, factor, x, y, variance, wavelength;
    double xmin, xspan, ymin, yspan;
};
wg_status pulse_args(const wg_params &p, int pitch, int wpitch, double init_amp, double factor, double x, double y,
                     double variance, double wavelength, PulseArgs *a);
// xy (int16 mask, nonzero test) or, when xy is NULL, nz (the "nonzero" bit plane); vel
// (FP32 fields, else NULL): the velocity, which takes the same increment
template <class T> void launch_add_circular_wave(const PulseArgs &a, T *phi, T *vel, const int16_t *xy,
                                                 const uint32_t *nz, cudaStream_t st);
void launch_cell_energy(const DevParams &p, const double *phi, const double *psi, const int16_t *xy, int i, int j,
                        double *out, cudaStream_t st);

}  // namespace wg
