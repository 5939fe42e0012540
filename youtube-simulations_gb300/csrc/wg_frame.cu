// wg_frame.cu — colour-mapped RGB8 frames of a scene (the serving output).
//
// draw_wave_highres_palette (wave_common.c:1750-1848) with wave_value (wave_common.c:
// 1053-1162) for the C_ONEDIM colour scheme (colors_waves.c:3-22, 161-258;
// colormaps.c:2449-2482) at every size-th cell.  The value of a sampled cell comes
// from the plot mode (phi, compute_energy, compute_energy_flux, and the running sums of
// the mean, exponential-average and total-flux modes, kept per sampled cell);
// amplitude = COLOR_RANGE*tanh(SLOPE*value/scale)*exp(-time*ATTENUATION); palette
// index (int)(256*h) with h = 0.5*(1 + amplitude) (color_scheme_palette) or h =
// amplitude (color_scheme_asym_palette: the energy and flux modes), clamped to 0..255.
// Drawn cells (TWOSPEEDS or xy != 0) get that palette colour times the optional
// factors, other cells black.  The reference hands floats to glColor3f; here the
// palette is the caller's byte table and the faded colour is rounded to bytes.
#include <cmath>
#include "wg_internal.h"
#include "wg_scene.h"

namespace wg {

// argument() of sub_wave.c:287-302 with the reference's PI and PID constants.
__device__ __forceinline__ double ref_argument(double x, double y)
{
    const double PI_ = 3.141592654, PID_ = 1.570796327;
    double alph;
    if (x != 0.0) {
        alph = atan(y / x);
        if (x < 0.0) alph += PI_;
    } else {
        alph = PID_;
        if (y < 0.0) alph = PI_ * 1.5;
    }
    return alph;
}

template <class T, int COEF>
__global__ void k_frame_rgb8(const __grid_constant__ DevParams p, const T *__restrict__ phi,
                             const T *__restrict__ psi, const uint32_t *__restrict__ nz, const T *__restrict__ tcc,
                             const uint8_t *__restrict__ lut, wg_frame_params fp, double *__restrict__ acc,
                             uint8_t *__restrict__ out, int w, int h)
{
    const int col = blockIdx.x * blockDim.x + threadIdx.x, row = blockIdx.y;
    if (col >= w || row >= h) return;
    const int i = col * fp.size, j = row * fp.size;
    const size_t o = ((size_t)row * w + col) * 3, k = (size_t)row * w + col;
    const int m = (nz[(size_t)i * p.wpitch + (j >> 5)] >> (j & 31)) & 1u;
    const int plot = fp.plot;
    const size_t c = (size_t)i * p.pitch + j;
    const double x = (double)phi[c];
    // compute_energy / compute_energy_flux neighbours, clamped at the edges
    double energy = 0.0, vel = 0.0, gx = 0.0, gy = 0.0;
    if (plot != WG_P_AMPLITUDE) {
        const int ip = (i + 1 == p.nx) ? p.nx - 1 : i + 1, im = (i == 0) ? 0 : i - 1;
        const int jp = (j + 1 == p.ny) ? p.ny - 1 : j + 1, jm = (j == 0) ? 0 : j - 1;
        const double e = (double)phi[(size_t)ip * p.pitch + j], wv = (double)phi[(size_t)im * p.pitch + j];
        const double n = (double)phi[(size_t)i * p.pitch + jp], sv = (double)phi[(size_t)i * p.pitch + jm];
        // psi of FP64 fields; FP32 fields hold the velocity: psi = phi - v (exact in FP64)
        const double y = sizeof(T) == 4 ? S_(x, (double)psi[c]) : (double)psi[c];
        if (plot == WG_P_ENERGY_FLUX || plot == WG_P_TOTAL_ENERGY_FLUX) {
            vel = fabs(S_(x, y));
            gx = S_(e, wv);
            gy = S_(n, sv);
        } else {
            energy = cell_energy(p, x, y, e, wv, n, sv, m);
        }
    }
    double value = 0.0, dim = 1.0;
    int asym = 0, linear = 0;
    switch (plot) {
    case WG_P_AMPLITUDE: value = A_(fp.vshift, M_(fp.vscale, x)); break;
    case WG_P_ENERGY: value = energy; asym = 1; break;
    case WG_P_MIXED: value = (j > p.ny / 2) ? x : energy; break;
    case WG_P_MEAN_ENERGY:
        acc[k] = A_(acc[k], energy);
        value = D_(acc[k], (double)(fp.time + 1));
        asym = 1;
        break;
    case WG_P_LOG_ENERGY:
        if (energy < 1.0e-20) energy = 1.0e-20;
        value = A_(fp.log_shift, M_(fp.log_scale, log(energy)));
        break;
    case WG_P_LOG_MEAN_ENERGY:
        if (energy == 0.0) energy = 1.0e-20;
        acc[k] = A_(acc[k], energy);
        value = A_(fp.log_shift, M_(fp.log_scale, log(D_(acc[k], (double)(fp.time + 1)))));
        break;
    case WG_P_ENERGY_FLUX: {
        const double mod = (m || p.twospeeds) ? M_(vel, sqrt(A_(M_(gx, gx), M_(gy, gy)))) : 0.0;
        value = M_(mod, fp.flux_scale);
        asym = 1;
        break;
    }
    case WG_P_TOTAL_ENERGY_FLUX: {
        const double fx = (m || p.twospeeds) ? M_(vel, gx) : 0.0, fy = (m || p.twospeeds) ? M_(vel, gy) : 0.0;
        const double mgx = A_(M_(acc[2 * k], 0.99), fx), mgy = A_(M_(acc[2 * k + 1], 0.99), fy);
        acc[2 * k] = mgx;
        acc[2 * k + 1] = mgy;
        const double mod = sqrt(A_(M_(mgx, mgx), M_(mgy, mgy)));
        double arg = ref_argument(mgx, mgy);
        if (arg < 0.0) arg = A_(arg, 6.283185307);
        value = D_(arg, 6.283185307);
        linear = 1;
        dim = tanh(M_(mod, fp.flux_scale));
        break;
    }
    case WG_P_AVERAGE_ENERGY:
        acc[k] = A_(M_(fp.avrg_e_factor, acc[k]), M_(S_(1.0, fp.avrg_e_factor), energy));
        value = acc[k];
        asym = 1;
        break;
    default:  // WG_P_LOG_AVERAGE_ENERGY
        acc[k] = A_(M_(fp.avrg_e_factor, acc[k]), M_(S_(1.0, fp.avrg_e_factor), energy));
        value = (acc[k] == 0.0) ? S_(fp.log_shift, M_(10.0, fp.log_scale))
                                : A_(fp.log_shift, M_(fp.log_scale, log(acc[k])));
        break;
    }
    if (!(p.twospeeds || m)) {
        out[o] = out[o + 1] = out[o + 2] = 0;
        return;
    }
    double hh;
    if (linear) {  // C_ONEDIM_LINEAR with scale 1 (colors_waves.c:198-205)
        hh = M_(fp.slope, value);
        if (hh > 1.0) hh = S_(hh, 1.0);
        else if (hh < 0.0) hh = A_(hh, 1.0);
    } else {
        double amp = M_(fp.color_range, tanh(D_(M_(fp.slope, value), fp.scale)));
        if (fp.attenuation != 0.0) amp = M_(amp, exp(-M_((double)fp.time, fp.attenuation)));
        hh = asym ? amp : M_(0.5, A_(1.0, amp));
    }
    const double hv = M_(256.0, hh);
    int hue = hv >= 255.0 ? 255 : (hv <= 0.0 ? 0 : (int)hv);
    double f = dim;
    if (fp.fade_in_obstacle) {
        const double cc = (COEF == WG_COEF_TABLE) ? (double)tcc[c] : (m ? p.c2 : p.c2b);
        f *= pow(cc / p.c2, 0.1);
    }
    if (fp.fade) f *= fp.fade_value;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const double v = (double)lut[hue * 3 + q] * f;
        int b = (int)(v + 0.5);
        out[o + q] = (uint8_t)(b > 255 ? 255 : (b < 0 ? 0 : b));
    }
}

// doubles of running state per sampled cell for a plot mode
static int frame_acc_per_cell(int plot)
{
    switch (plot) {
    case WG_P_MEAN_ENERGY: case WG_P_LOG_MEAN_ENERGY: case WG_P_AVERAGE_ENERGY: case WG_P_LOG_AVERAGE_ENERGY: return 1;
    case WG_P_TOTAL_ENERGY_FLUX: return 2;
    default: return 0;
    }
}

wg_status frame_launch(const DevParams &p, const void *phi, const void *psi, int prec, int coef, const uint32_t *nz,
                       const void *tcc, const uint8_t *lut, const wg_frame_params &fp, double *acc, uint8_t *out,
                       cudaStream_t st)
{
    const int w = p.nx / fp.size, h = p.ny / fp.size;
    dim3 grd((w + 127) / 128, h);
    if (prec == WG_FP32) {
        if (coef == WG_COEF_TABLE) k_frame_rgb8<float, WG_COEF_TABLE><<<grd, 128, 0, st>>>(p, (const float *)phi, (const float *)psi, nz, (const float *)tcc, lut, fp, acc, out, w, h);
        else k_frame_rgb8<float, WG_COEF_MASK><<<grd, 128, 0, st>>>(p, (const float *)phi, (const float *)psi, nz, nullptr, lut, fp, acc, out, w, h);
    } else {
        if (coef == WG_COEF_TABLE) k_frame_rgb8<double, WG_COEF_TABLE><<<grd, 128, 0, st>>>(p, (const double *)phi, (const double *)psi, nz, (const double *)tcc, lut, fp, acc, out, w, h);
        else k_frame_rgb8<double, WG_COEF_MASK><<<grd, 128, 0, st>>>(p, (const double *)phi, (const double *)psi, nz, nullptr, lut, fp, acc, out, w, h);
    }
    WG_CUDA(cudaGetLastError());
    return WG_OK;
}

wg_status frame_validate(const wg_params &p, const wg_frame_params *fp, const uint8_t *lut)
{
    if (!fp || !lut) { set_error("frame parameters and palette are required"); return WG_ERR_INVALID; }
    if (fp->size < 1 || fp->size > p.nx || fp->size > p.ny) { set_error("frame size (downsampling) out of range"); return WG_ERR_INVALID; }
    if (!(fp->scale != 0.0)) { set_error("frame scale must be non-zero"); return WG_ERR_INVALID; }
    if (fp->plot < WG_P_AMPLITUDE || fp->plot > WG_P_LOG_AVERAGE_ENERGY) { set_error("unknown plot mode %d", fp->plot); return WG_ERR_INVALID; }
    return WG_OK;
}

}  // namespace wg

using namespace wg;

extern "C" wg_status wg_scene_frame_rgb8(wg_scene *s, const wg_frame_params *fp, const uint8_t *lut, uint8_t *rgb_host,
                                         void *rgb_device)
{
    if (!s) { set_error("NULL scene"); return WG_ERR_INVALID; }
    wg_status st = frame_validate(s->prm, fp, lut);
    if (st) return st;
    const size_t bytes = (size_t)(s->prm.nx / fp->size) * (s->prm.ny / fp->size) * 3;
    if (!s->lut) WG_CUDA(cudaMalloc(&s->lut, 768));
    WG_CUDA(cudaMemcpyAsync(s->lut, lut, 768, cudaMemcpyHostToDevice, s->st));
    uint8_t *dst = (uint8_t *)rgb_device;
    if (!dst) {
        if (s->rgb_bytes < bytes) {
            if (s->rgb) cudaFree(s->rgb);
            s->rgb = nullptr;
            s->rgb_bytes = 0;
            WG_CUDA(cudaMalloc(&s->rgb, bytes));
            s->rgb_bytes = bytes;
        }
        dst = s->rgb;
    }
    // running sums of the mean / average / total-flux modes, at frame resolution
    const int per = frame_acc_per_cell(fp->plot);
    if (per) {
        const size_t n = (size_t)(s->prm.nx / fp->size) * (s->prm.ny / fp->size) * per;
        if (!s->facc || s->facc_n != n || s->facc_plot != fp->plot || s->facc_size != fp->size) {
            if (s->facc) cudaFree(s->facc);
            s->facc = nullptr;
            WG_CUDA(cudaMalloc(&s->facc, n * sizeof(double)));
            WG_CUDA(cudaMemsetAsync(s->facc, 0, n * sizeof(double), s->st));
            s->facc_n = n;
            s->facc_plot = fp->plot;
            s->facc_size = fp->size;
        }
    }
    if ((st = frame_launch(s->dp, s->f[s->cur], s->f[1 - s->cur], s->prec, s->coef, s->nz, s->tcc, s->lut, *fp,
                           per ? s->facc : nullptr, dst, s->st)))
        return st;
    s->launches++;
    if (rgb_host) WG_CUDA(cudaMemcpyAsync(rgb_host, dst, bytes, cudaMemcpyDeviceToHost, s->st));
    return scene_check_flag(s);  // synchronises the stream (the image is ready on return)
}

extern "C" wg_status wg_scene_frame_reset(wg_scene *s)
{
    if (!s) { set_error("NULL scene"); return WG_ERR_INVALID; }
    if (s->facc) WG_CUDA(cudaMemsetAsync(s->facc, 0, s->facc_n * sizeof(double), s->st));
    return WG_OK;
}
