// wg_domain.cu — masks and coefficient tables built on the device.
//
// xy_in_billiard_single_domain for the shapes of the workloads (sub_wave.c:5712-6252:
// rectangle, ellipse, stadium, polygon, discs, discs in a rectangle) at every cell
// centre (ij_to_xy, sub_wave.c:469-476), and the constant / two-speed branch of
// init_ior_2d (sub_wave.c:12983-13002) for WG_COEF_TABLE scenes.  The FP64 tests run in
// the reference's order without contraction; only the polygon uses cos and sin (CUDA's),
// so a cell within rounding of a polygon edge may fall on the other side than the
// host's.  Replaces the host mask and tables of wg_scene_upload; phi and psi then come
// from wg_scene_upload_state.  Masks are 0/1, so the "active" and "nonzero" planes match.
#include <cmath>
#include <vector>
#include "wg_internal.h"
#include "wg_scene.h"

namespace wg {

struct DomainArgs {
    int nx, ny, wpitch, domain, npoly, ncirc;
    double lambda, apoly, xmin, xspan, ymin, yspan, rect_h;  // rect_h = YMAX - XMAX + lambda
    const double *circ;                                       // ncirc x (xc, yc, radius)
};

__device__ int dom_inside(const DomainArgs &d, double x, double y)
{
    const double R_DPI = 6.283185307, R_PID = 1.570796327;
    switch (d.domain) {
    case 0:  // D_RECTANGLE
        return (fabs(x) < d.lambda) && (fabs(y) < 1.0);
    case 1:  // D_ELLIPSE
        return A_(D_(M_(x, x), M_(d.lambda, d.lambda)), M_(y, y)) < 1.0;
    case 2: {  // D_STADIUM
        const double h = M_(0.5, d.lambda);
        if ((x > -h) && (x < h) && (y > -1.0) && (y < 1.0)) return 1;
        const double a = A_(x, h), b = S_(x, h);
        if (sqrt(A_(M_(a, a), M_(y, y))) < 1.0) return 1;
        if (sqrt(A_(M_(b, b), M_(y, y))) < 1.0) return 1;
        return 0;
    }
    case 8: {  // D_POLYGON
        int cond = 1;
        const double omega = D_(R_DPI, (double)d.npoly);
        const double c = M_(d.lambda, cos(M_(omega, 0.5)));
        for (int k = 0; k < d.npoly; k++) {
            const double angle = A_(M_(d.apoly, R_PID), M_((double)k + 0.5, omega));
            cond = cond * (A_(M_(x, cos(angle)), M_(y, sin(angle))) < c);
        }
        return cond;
    }
    case 20:
    case 201: {  // D_CIRCLES, D_CIRCLES_IN_RECT
        for (int k = 0; k < d.ncirc; k++) {
            const double dx = S_(x, d.circ[3 * k]), dy = S_(y, d.circ[3 * k + 1]);
            const double r = d.circ[3 * k + 2];
            if (A_(M_(dx, dx), M_(dy, dy)) < M_(r, r)) return 0;
        }
        if (d.domain == 20) return 1;
        return !((fabs(x) >= d.lambda) || (fabs(y) >= d.rect_h));
    }
    default:
        return 1;
    }
}

// one thread per 32-bit mask word of row i
__global__ void k_build_mask(DomainArgs d, uint32_t *__restrict__ act, uint32_t *__restrict__ nz)
{
    const int wj = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (wj >= d.wpitch) return;
    const double x = A_(d.xmin, D_(M_((double)i, d.xspan), (double)d.nx));
    uint32_t bits = 0;
    for (int b = 0; b < 32; b++) {
        const int j = wj * 32 + b;
        if (j >= d.ny) break;
        const double y = A_(d.ymin, D_(M_((double)j, d.yspan), (double)d.ny));
        if (dom_inside(d, x, y)) bits |= 1u << b;
    }
    act[(size_t)i * d.wpitch + wj] = bits;
    nz[(size_t)i * d.wpitch + wj] = bits;
}

// init_ior_2d's constant / two-speed branch from the mask bits
template <class T>
__global__ void k_build_tables(DevParams p, const uint32_t *__restrict__ nz, T *__restrict__ tcc, T *__restrict__ tc,
                               T *__restrict__ tg, double courant, double courantb, double gamma, double gammab)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= p.ny) return;
    const size_t c = (size_t)i * p.pitch + j;
    const int m = (nz[(size_t)i * p.wpitch + (j >> 5)] >> (j & 31)) & 1u;
    if (m) {
        tcc[c] = (T)M_(courant, courant);
        if (tc) tc[c] = (T)courant;
        if (tg) tg[c] = (T)gamma;
    } else if (p.twospeeds) {
        tcc[c] = (T)M_(courantb, courantb);
        if (tc) tc[c] = (T)courantb;
        if (tg) tg[c] = (T)gammab;
    }
}

}  // namespace wg

using namespace wg;

extern "C" wg_status wg_scene_build_domain(wg_scene *s, int32_t domain, double lambda, int32_t npoly, double apoly,
                                           const double *circles, int32_t ncircles)
{
    if (!s) { set_error("NULL scene"); return WG_ERR_INVALID; }
    if (s->prm.bc_neumann) {
        set_error("Neumann scenes take their mask and records from the host (wg_scene_upload, wg_scene_set_neumann)");
        return WG_ERR_INVALID;
    }
    const bool circ = domain == 20 || domain == 201;
    if (!(domain == 0 || domain == 1 || domain == 2 || domain == 8 || circ)) {
        set_error("domain %d: built on the device are 0 rectangle, 1 ellipse, 2 stadium, 8 polygon, 20 discs, "
                  "201 discs in a rectangle", domain);
        return WG_ERR_INVALID;
    }
    if (domain == 8 && npoly < 3) { set_error("a polygon needs npoly >= 3"); return WG_ERR_INVALID; }
    if (circ && ncircles > 0 && !circles) { set_error("circles is NULL"); return WG_ERR_INVALID; }
    if (ncircles < 0) { set_error("negative circle count"); return WG_ERR_INVALID; }
    DomainArgs d{};
    d.nx = s->prm.nx;
    d.ny = s->prm.ny;
    d.wpitch = s->dp.wpitch;
    d.domain = domain;
    d.npoly = npoly;
    d.ncirc = circ ? ncircles : 0;
    d.lambda = lambda;
    d.apoly = apoly;
    d.xmin = s->prm.xmin;
    d.xspan = s->prm.xmax - s->prm.xmin;
    d.ymin = s->prm.ymin;
    d.yspan = s->prm.ymax - s->prm.ymin;
    d.rect_h = s->prm.ymax - s->prm.xmax + lambda;
    double *dcirc = nullptr;
    if (d.ncirc > 0) {
        WG_CUDA(cudaMalloc(&dcirc, sizeof(double) * 3 * d.ncirc));
        WG_CUDA(cudaMemcpy(dcirc, circles, sizeof(double) * 3 * d.ncirc, cudaMemcpyHostToDevice));
    }
    d.circ = dcirc;
    k_build_mask<<<dim3((d.wpitch + 127) / 128, d.nx), 128, 0, s->st>>>(d, s->act, s->nz);
    s->launches++;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && s->coef == WG_COEF_TABLE) {
        // tgamma: a scalar when it is the same on every cell the stepper updates
        const bool uniform = !s->prm.twospeeds || s->prm.gamma == s->prm.gammab;
        if (s->tg) { cudaFree(s->tg); s->tg = nullptr; }
        if (uniform) {
            s->dp.gam = s->prm.gamma;
            s->dp.gamb = s->prm.gamma;
        } else {
            const size_t fb = (size_t)s->prm.nx * s->pitch * s->esz;
            e = cudaMalloc(&s->tg, fb);
            if (e == cudaSuccess) e = cudaMemsetAsync(s->tg, 0, fb, s->st);
        }
        const dim3 grd((s->prm.ny + 127) / 128, s->prm.nx);
        if (e == cudaSuccess) {
            if (s->prec == WG_FP32)
                k_build_tables<float><<<grd, 128, 0, s->st>>>(s->dp, s->nz, (float *)s->tcc, (float *)s->tc, (float *)s->tg,
                                                              s->prm.courant, s->prm.courantb, s->prm.gamma, s->prm.gammab);
            else
                k_build_tables<double><<<grd, 128, 0, s->st>>>(s->dp, s->nz, (double *)s->tcc, (double *)s->tc,
                                                               (double *)s->tg, s->prm.courant, s->prm.courantb,
                                                               s->prm.gamma, s->prm.gammab);
            s->launches++;
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (dcirc) cudaFree(dcirc);
    if (e != cudaSuccess) return cuda_fail(e, "wg_scene_build_domain");
    s->has_ghosts = 0;
    s->xy_host.clear();
    s->has_mask = true;
    s->tb_k = 0;  // autotuned again for the new geometry
    return WG_OK;
}

extern "C" wg_status wg_scene_download_mask(wg_scene *s, int16_t *xy)
{
    if (!s || !xy) { set_error("NULL argument"); return WG_ERR_INVALID; }
    if (!s->has_mask) { set_error("the scene has no mask yet"); return WG_ERR_STATE; }
    const int nx = s->prm.nx, ny = s->prm.ny, wp = s->dp.wpitch;
    std::vector<uint32_t> bits((size_t)nx * wp);
    WG_CUDA(cudaMemcpyAsync(bits.data(), s->nz, sizeof(uint32_t) * bits.size(), cudaMemcpyDeviceToHost, s->st));
    WG_CUDA(cudaStreamSynchronize(s->st));
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) xy[(size_t)i * ny + j] = (int16_t)((bits[(size_t)i * wp + (j >> 5)] >> (j & 31)) & 1u);
    return WG_OK;
}
