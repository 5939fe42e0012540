// wg_pulse.cu — add_circular_wave (wave_common.c:337-351) on the device.
//
// phi += INITIAL_AMP*factor*exp(-r^2/INITIAL_VARIANCE)*cos(-r/INITIAL_WAVELENGTH) on the
// cells whose mask is nonzero (every cell with TWOSPEEDS), r the distance of the cell
// (ij_to_xy, sub_wave.c:469-476) from (x, y); psi is not touched, so an FP32 scene's
// velocity phi - psi takes the same increment.  The FP64 arithmetic runs in the
// reference's order without contraction; exp and cos are CUDA's.
//
// Only a box around (x, y) is visited.  Outside it, r^2 > 760 variance, where
// exp(-r^2/variance) is 0 in double precision (it underflows below about -745.1), so the
// reference adds an exact zero there.
#include <cmath>
#include "wg_internal.h"
#include "wg_scene.h"

namespace wg {

template <class T, int MASK>
__global__ void __launch_bounds__(128) k_add_circular_wave(PulseArgs a, T *__restrict__ phi, T *__restrict__ vel,
                                                           const int16_t *__restrict__ xy,
                                                           const uint32_t *__restrict__ nz)
{
    const int j = a.j0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int i = a.i0 + (int)blockIdx.y;
    if (j >= a.j0 + a.nj) return;
    bool m;
    if (MASK == 0) m = xy[(size_t)i * a.pitch + j] != 0;
    else m = (nz[(size_t)i * a.wpitch + (j >> 5)] >> (j & 31)) & 1u;
    if (!(m || a.twospeeds)) return;
    const double xi = A_(a.xmin, D_(M_((double)i, a.xspan), (double)a.nx));
    const double yj = A_(a.ymin, D_(M_((double)j, a.yspan), (double)a.ny));
    const double dx = S_(xi, a.x), dy = S_(yj, a.y);
    const double d2 = A_(M_(dx, dx), M_(dy, dy));
    const double v = M_(M_(M_(a.init_amp, a.factor), exp(D_(-d2, a.variance))), cos(D_(-sqrt(d2), a.wavelength)));
    T &c = phi[(size_t)i * a.pitch + j];
    c = (T)A_((double)c, v);
    if (vel) {
        T &u = vel[(size_t)i * a.pitch + j];
        u = (T)A_((double)u, v);
    }
}

wg_status pulse_args(const wg_params &p, int pitch, int wpitch, double init_amp, double factor, double x, double y,
                     double variance, double wavelength, PulseArgs *a)
{
    if (!(variance > 0.0) || !std::isfinite(variance)) {
        set_error("add_circular_wave: the variance must be positive and finite");
        return WG_ERR_INVALID;
    }
    if (!std::isfinite(x) || !std::isfinite(y)) { set_error("add_circular_wave: the centre must be finite"); return WG_ERR_INVALID; }
    PulseArgs r{};
    r.nx = p.nx;
    r.ny = p.ny;
    r.pitch = pitch;
    r.wpitch = wpitch;
    r.twospeeds = p.twospeeds;
    r.init_amp = init_amp;
    r.factor = factor;
    r.x = x;
    r.y = y;
    r.variance = variance;
    r.wavelength = wavelength;
    r.xmin = p.xmin;
    r.xspan = p.xmax - p.xmin;
    r.ymin = p.ymin;
    r.yspan = p.ymax - p.ymin;
    // support box (r <= R), widened by two cells on each side
    const double R = std::sqrt(760.0 * variance);
    const double sx = (double)p.nx / r.xspan, sy = (double)p.ny / r.yspan;
    double i0 = std::floor((x - R - p.xmin) * sx) - 2.0, i1 = std::ceil((x + R - p.xmin) * sx) + 3.0;
    double j0 = std::floor((y - R - p.ymin) * sy) - 2.0, j1 = std::ceil((y + R - p.ymin) * sy) + 3.0;
    i0 = std::fmax(i0, 0.0);
    j0 = std::fmax(j0, 0.0);
    i1 = std::fmin(i1, (double)p.nx);
    j1 = std::fmin(j1, (double)p.ny);
    r.i0 = (int)i0;
    r.j0 = (int)j0;
    r.ni = i1 > i0 ? (int)(i1 - i0) : 0;
    r.nj = j1 > j0 ? (int)(j1 - j0) : 0;
    *a = r;
    return WG_OK;
}

template <class T>
void launch_add_circular_wave(const PulseArgs &a, T *phi, T *vel, const int16_t *xy, const uint32_t *nz,
                              cudaStream_t st)
{
    if (a.ni <= 0 || a.nj <= 0) return;
    dim3 grd((a.nj + 127) / 128, a.ni);
    if (xy) k_add_circular_wave<T, 0><<<grd, 128, 0, st>>>(a, phi, vel, xy, nz);
    else k_add_circular_wave<T, 1><<<grd, 128, 0, st>>>(a, phi, vel, xy, nz);
}
template void launch_add_circular_wave<float>(const PulseArgs &, float *, float *, const int16_t *, const uint32_t *,
                                              cudaStream_t);
template void launch_add_circular_wave<double>(const PulseArgs &, double *, double *, const int16_t *,
                                               const uint32_t *, cudaStream_t);

}  // namespace wg

using namespace wg;

extern "C" wg_status wg_scene_add_circular_wave(wg_scene *s, double init_amp, double factor, double x, double y,
                                                double variance, double wavelength)
{
    if (!s) { set_error("NULL scene"); return WG_ERR_INVALID; }
    if (!s->uploaded) { set_error("scene has no state: upload first"); return WG_ERR_STATE; }
    PulseArgs a;
    wg_status st = pulse_args(s->prm, s->pitch, s->dp.wpitch, init_amp, factor, x, y, variance, wavelength, &a);
    if (st) return st;
    void *phi = s->f[s->cur];
    if (s->prec == WG_FP32)
        launch_add_circular_wave<float>(a, (float *)phi, (float *)s->f[1 - s->cur], nullptr, s->nz, s->st);
    else
        launch_add_circular_wave<double>(a, (double *)phi, nullptr, nullptr, s->nz, s->st);
    s->launches++;
    WG_CUDA(cudaGetLastError());
    return WG_OK;
}
