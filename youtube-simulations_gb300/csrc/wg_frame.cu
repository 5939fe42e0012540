// wg_frame.cu — colour-mapped RGB8 frames of a scene (the serving output).
//
// P_AMPLITUDE / C_ONEDIM colour map of draw_wave_highres_palette (wave_common.c:
// 1053-1065, 1750-1848; colors_waves.c:3-16, 161-218; colormaps.c:2449-2482) at every
// size-th cell: value = VSHIFT + VSCALE*phi, amplitude = COLOR_RANGE*tanh(SLOPE*value/
// scale), palette index min(255, (int)(256*0.5*(1 + amplitude))); drawn cells (TWOSPEEDS
// or xy != 0) get that palette colour times the optional fades, other cells black.
// The reference hands floats to glColor3f; here the palette is the caller's byte table
// and the faded colour is rounded to bytes.
#include <cmath>
#include "wg_internal.h"
#include "wg_scene.h"

namespace wg {

template <class T, int COEF>
__global__ void k_frame_rgb8(const __grid_constant__ DevParams p, const T *__restrict__ phi,
                             const uint32_t *__restrict__ nz, const T *__restrict__ tcc, const uint8_t *__restrict__ lut,
                             wg_frame_params fp, uint8_t *__restrict__ out, int w, int h)
{
    const int col = blockIdx.x * blockDim.x + threadIdx.x, row = blockIdx.y;
    if (col >= w || row >= h) return;
    const int i = col * fp.size, j = row * fp.size;
    const size_t o = ((size_t)row * w + col) * 3;
    const int m = (nz[(size_t)i * p.wpitch + (j >> 5)] >> (j & 31)) & 1u;
    if (!(p.twospeeds || m)) {
        out[o] = out[o + 1] = out[o + 2] = 0;
        return;
    }
    const double value = fp.vshift + fp.vscale * (double)phi[(size_t)i * p.pitch + j];
    const double amp = fp.color_range * tanh(fp.slope * value / fp.scale);
    int hue = (int)(256.0 * (0.5 * (1.0 + amp)));
    if (hue > 255) hue = 255;
    if (hue < 0) hue = 0;
    double f = 1.0;
    if (fp.fade_in_obstacle) {
        const double cc = (COEF == WG_COEF_TABLE) ? (double)tcc[(size_t)i * p.pitch + j] : (m ? p.c2 : p.c2b);
        f *= pow(cc / p.c2, 0.1);
    }
    if (fp.fade) f *= fp.fade_value;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double v = (double)lut[hue * 3 + k] * f;
        int b = (int)(v + 0.5);
        out[o + k] = (uint8_t)(b > 255 ? 255 : (b < 0 ? 0 : b));
    }
}

wg_status frame_launch(const DevParams &p, const void *phi, int prec, int coef, const uint32_t *nz, const void *tcc,
                       const uint8_t *lut, const wg_frame_params &fp, uint8_t *out, cudaStream_t st)
{
    const int w = p.nx / fp.size, h = p.ny / fp.size;
    dim3 grd((w + 127) / 128, h);
    if (prec == WG_FP32) {
        if (coef == WG_COEF_TABLE) k_frame_rgb8<float, WG_COEF_TABLE><<<grd, 128, 0, st>>>(p, (const float *)phi, nz, (const float *)tcc, lut, fp, out, w, h);
        else k_frame_rgb8<float, WG_COEF_MASK><<<grd, 128, 0, st>>>(p, (const float *)phi, nz, nullptr, lut, fp, out, w, h);
    } else {
        if (coef == WG_COEF_TABLE) k_frame_rgb8<double, WG_COEF_TABLE><<<grd, 128, 0, st>>>(p, (const double *)phi, nz, (const double *)tcc, lut, fp, out, w, h);
        else k_frame_rgb8<double, WG_COEF_MASK><<<grd, 128, 0, st>>>(p, (const double *)phi, nz, nullptr, lut, fp, out, w, h);
    }
    WG_CUDA(cudaGetLastError());
    return WG_OK;
}

wg_status frame_validate(const wg_params &p, const wg_frame_params *fp, const uint8_t *lut)
{
    if (!fp || !lut) { set_error("frame parameters and palette are required"); return WG_ERR_INVALID; }
    if (fp->size < 1 || fp->size > p.nx || fp->size > p.ny) { set_error("frame size (downsampling) out of range"); return WG_ERR_INVALID; }
    if (!(fp->scale != 0.0)) { set_error("frame scale must be non-zero"); return WG_ERR_INVALID; }
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
    if ((st = frame_launch(s->dp, s->f[s->cur], s->prec, s->coef, s->nz, s->tcc, s->lut, *fp, dst, s->st))) return st;
    s->launches++;
    if (rgb_host) WG_CUDA(cudaMemcpyAsync(rgb_host, dst, bytes, cudaMemcpyDeviceToHost, s->st));
    WG_CUDA(cudaStreamSynchronize(s->st));
    return scene_check_flag(s);
}
