// wg_domain.cu — masks and coefficient tables built on the device.
//
// xy_in_billiard_single_domain for the shapes of the workloads (sub_wave.c:5712-6252:
// rectangle, ellipse, stadium, polygon, discs, discs in a rectangle) at every cell
// centre (ij_to_xy, sub_wave.c:469-476), and the constant / two-speed branch of
// init_ior_2d (sub_wave.c:12983-13002) for WG_COEF_TABLE scenes.  The FP64 tests run in
// the reference's order without contraction; only the polygon uses cos and sin (CUDA's),
// so a cell within rounding of a polygon edge may fall on the other side than the
// host's.  Replaces the host mask and tables of wg_scene_upload; phi and psi then come
// from wg_scene_upload_state.  Masks are 0/1, so the "active" and "nonzero" planes match,
// except for Neumann scenes (BC_NEUMANN, ellipse or polygon): after the tables, the
// ghost cells of init_neumann_bc (sub_wave.c:13910-13947) are found on the device, their
// records built in the reference's row-major order (compute_normal_vector and
// build_neumann_data, sub_wave.c:13720-13848; test_neumann_data, :13850-13880), and the
// ghost cells marked in the "nonzero" plane (xy_in = -1: not active, nonzero).
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

// ---------------------------------------------------------------------------
// Neumann set-up on the device
// ---------------------------------------------------------------------------
__device__ __forceinline__ int inside_bit(const uint32_t *in, int wpitch, int i, int j)
{
    return (in[(size_t)i * wpitch + (j >> 5)] >> (j & 31)) & 1u;
}

// init_neumann_bc's test: an interior cell (1..NX-2 x 1..NY-2) outside the domain with a
// 4-neighbour inside (xy_in == 1).  Marking cells -1 in the reference's loop does not
// change the test for later cells (it asks for neighbours equal to 1), so the set does
// not depend on the order of the loop.
__device__ __forceinline__ bool ghost_cell(const uint32_t *in, int wpitch, int nx, int ny, int i, int j)
{
    if (i < 1 || i > nx - 2 || j < 1 || j > ny - 2 || inside_bit(in, wpitch, i, j)) return false;
    return inside_bit(in, wpitch, i - 1, j) || inside_bit(in, wpitch, i + 1, j) || inside_bit(in, wpitch, i, j - 1) ||
           inside_bit(in, wpitch, i, j + 1);
}

// ghost cells per row i (one block per row)
__global__ void k_ghost_count(const uint32_t *__restrict__ in, int wpitch, int nx, int ny, int *__restrict__ rows)
{
    const int i = blockIdx.x;
    int c = 0;
    for (int j = threadIdx.x; j < ny; j += blockDim.x) c += ghost_cell(in, wpitch, nx, ny, i, j);
    __shared__ int sh[32];
    for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        rows[i] = t;
    }
}

// exclusive scan of the row counts (one block); base[nx] = the total
__global__ void k_row_scan(const int *__restrict__ rows, int nx, int *__restrict__ base)
{
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int start = 0; start < nx; start += blockDim.x) {
        const int i = start + threadIdx.x;
        int v = i < nx ? rows[i] : 0;
        // inclusive scan within the block (warp shuffles, then warp totals)
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        int x = v;
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        __shared__ int wsum[32];
        if (lane == 31) wsum[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int w = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= off) w += y;
            }
            wsum[lane] = w;
        }
        __syncthreads();
        const int incl = x + (wid > 0 ? wsum[wid - 1] : 0);
        if (i < nx) base[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) base[nx] = carry;
}

struct NeumannArgs {
    int nx, ny, wpitch, pitch, domain, npoly;
    double lambda, apoly, xmin, xspan, ymin, yspan;
};

// argument() of sub_wave.c:287-302 (CUDA's atan)
__device__ double dom_argument(double x, double y)
{
    const double R_PI = 3.141592654, R_PID = 1.570796327;
    if (x != 0.0) {
        double a = atan(D_(y, x));
        if (x < 0.0) a = A_(a, R_PI);
        return a;
    }
    return (y < 0.0) ? M_(R_PI, 1.5) : R_PID;
}

// One block per row: the row's ghost cells in order of j get records base[i], base[i]+1,
// ...; each record is the reference's (normal vector, neighbours, the deactivation of
// test_neumann_data), and a gather entry for the stepping kernels (flag bit 1: inactive).
__global__ void k_neumann_records(NeumannArgs d, const uint32_t *__restrict__ in, const int *__restrict__ base,
                                  wg_neumann_bc *__restrict__ rec, int4 *__restrict__ idx, double2 *__restrict__ w)
{
    const double R_DPI = 6.283185307, R_PID = 1.570796327;
    const int i = blockIdx.x, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __shared__ int wcount[32];
    int offset = base[i];
    for (int j0 = 0; j0 < d.ny; j0 += blockDim.x) {
        const int j = j0 + threadIdx.x;
        const bool g = j < d.ny && ghost_cell(in, d.wpitch, d.nx, d.ny, i, j);
        const unsigned ball = __ballot_sync(0xffffffffu, g);
        if (lane == 0) wcount[wid] = __popc(ball);
        __syncthreads();
        int before = 0, total = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) {
            if (q < wid) before += wcount[q];
            total += wcount[q];
        }
        if (g) {
            const int r = offset + before + __popc(ball & ((1u << lane) - 1u));
            const double x = A_(d.xmin, D_(M_((double)i, d.xspan), (double)d.nx));
            const double y = A_(d.ymin, D_(M_((double)j, d.yspan), (double)d.ny));
            double v1, v2;
            if (d.domain == 1) {  // ellipse: the gradient of x^2/lambda^2 + y^2
                v1 = D_(M_(2.0, x), M_(d.lambda, d.lambda));
                v2 = M_(2.0, y);
            } else {  // polygon: the outward normal of the side the cell faces
                const double theta = D_(R_DPI, (double)d.npoly);
                double angle = A_(S_(dom_argument(x, y), M_(R_PID, d.apoly)), R_DPI);
                const int side = (int)D_(angle, theta);
                angle = A_(A_(M_(R_PID, d.apoly), M_(0.5, theta)), M_((double)side, theta));
                v1 = cos(angle);
                v2 = sin(angle);
            }
            wg_neumann_bc b;
            b.signx1 = (int16_t)(v1 >= 0.0 ? -1 : 1);
            b.signy1 = 0;
            b.signx2 = 0;
            b.signy2 = (int16_t)(v2 >= 0.0 ? -1 : 1);
            v1 = fabs(v1);
            v2 = fabs(v2);
            const double sum = A_(v1, v2);
            const double n1 = D_(v1, sum), n2 = D_(v2, sum);
            b.nx = n1;
            b.ny = n2;
            if (n1 > n2) {
                b.nx = D_(S_(n1, n2), n1);
                b.ny = D_(n2, n1);
                b.signx2 = b.signx1;
            } else if (n2 > n1) {
                b.nx = D_(n1, n2);
                b.ny = D_(S_(n2, n1), n2);
                b.signy1 = b.signy2;
            }
            b.top = (int16_t)(y > 0.0);
            b.i = i;
            b.j = j;
            b.k = 0;
            b.nbi1 = i + b.signx1;
            b.nbj1 = j + b.signy1;
            b.nbi2 = i + b.signx2;
            b.nbj2 = j + b.signy2;
            b.nbk1 = b.nbk2 = 0;
            const bool dead = ghost_cell(in, d.wpitch, d.nx, d.ny, b.nbi1, b.nbj1) ||
                              ghost_cell(in, d.wpitch, d.nx, d.ny, b.nbi2, b.nbj2);
            b.active = (int16_t)(dead ? 0 : 1);
            rec[r] = b;
            idx[r] = make_int4(i * d.pitch + j, b.nbi1 * d.pitch + b.nbj1, b.nbi2 * d.pitch + b.nbj2, 1 | (dead ? 2 : 0));
            w[r] = make_double2(b.nx, b.ny);
        }
        offset += total;
        __syncthreads();  // wcount is reused by the next chunk
    }
}

// the ghost cells into the "nonzero" plane (one thread per word)
__global__ void k_mark_ghosts(const uint32_t *__restrict__ in, int wpitch, int nx, int ny, uint32_t *__restrict__ nz)
{
    const int wj = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (wj >= wpitch) return;
    uint32_t add = 0;
    for (int b = 0; b < 32; b++) {
        const int j = wj * 32 + b;
        if (j >= ny) break;
        if (ghost_cell(in, wpitch, nx, ny, i, j)) add |= 1u << b;
    }
    nz[(size_t)i * wpitch + wj] |= add;
}

}  // namespace wg

using namespace wg;

// The Neumann set-up of a scene whose mask was just built: ghost cells counted per row,
// a scan gives each row's first record, then the records, the gather entries and the
// ghost marks.  The records stay on the device (wg_scene_neumann_records reads them).
static cudaError_t build_neumann_device(wg_scene *s, int domain, double lambda, int npoly, double apoly, int *nrec)
{
    const int nx = s->prm.nx, ny = s->prm.ny, wp = s->dp.wpitch;
    int *rows = nullptr;
    cudaError_t e = cudaMalloc(&rows, sizeof(int) * (2 * (size_t)nx + 1));
    if (e != cudaSuccess) return e;
    int *base = rows + nx;
    k_ghost_count<<<nx, 256, 0, s->st>>>(s->act, wp, nx, ny, rows);
    k_row_scan<<<1, 1024, 0, s->st>>>(rows, nx, base);
    s->launches += 2;
    int n = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&n, base + nx, sizeof(int), cudaMemcpyDeviceToHost, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (s->nidx) cudaFree(s->nidx);
    if (s->nw) cudaFree(s->nw);
    if (s->nrec_dev) cudaFree(s->nrec_dev);
    s->nidx = nullptr;
    s->nw = nullptr;
    s->nrec_dev = nullptr;
    s->nrec = 0;
    s->nrec_all = 0;
    if (e == cudaSuccess && n > 0) {
        e = cudaMalloc(&s->nrec_dev, sizeof(wg_neumann_bc) * n);
        if (e == cudaSuccess) e = cudaMalloc(&s->nidx, sizeof(int4) * n);
        if (e == cudaSuccess) e = cudaMalloc(&s->nw, sizeof(double2) * n);
        if (e == cudaSuccess) {
            NeumannArgs d{nx, ny, wp, s->pitch, domain, npoly, lambda, apoly, s->prm.xmin, s->prm.xmax - s->prm.xmin,
                          s->prm.ymin, s->prm.ymax - s->prm.ymin};
            k_neumann_records<<<nx, 256, 0, s->st>>>(d, s->act, base, s->nrec_dev, s->nidx, s->nw);
            k_mark_ghosts<<<dim3((wp + 127) / 128, nx), 128, 0, s->st>>>(s->act, wp, nx, ny, s->nz);
            s->launches += 2;
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            s->nrec = n;
            s->nrec_all = n;
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    cudaFree(rows);
    *nrec = n;
    return e;
}

extern "C" wg_status wg_scene_build_domain(wg_scene *s, int32_t domain, double lambda, int32_t npoly, double apoly,
                                           const double *circles, int32_t ncircles)
{
    if (!s) { set_error("NULL scene"); return WG_ERR_INVALID; }
    if (s->prm.bc_neumann && !(domain == 1 || domain == 8)) {
        set_error("Neumann records are built for the ellipse (1) and the polygon (8), as init_neumann_bc does");
        return WG_ERR_INVALID;
    }
    if (s->prm.bc_neumann && s->coef != WG_COEF_TABLE) {
        set_error("Neumann scenes keep their coefficients in tables (WG_COEF_TABLE)");
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
    int nrec = 0;
    if (e == cudaSuccess && s->prm.bc_neumann) e = build_neumann_device(s, domain, lambda, npoly, apoly, &nrec);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (dcirc) cudaFree(dcirc);
    if (e != cudaSuccess) return cuda_fail(e, "wg_scene_build_domain");
    s->has_ghosts = nrec > 0;
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
    std::vector<uint32_t> bits((size_t)nx * wp), act((size_t)nx * wp);
    WG_CUDA(cudaMemcpyAsync(bits.data(), s->nz, sizeof(uint32_t) * bits.size(), cudaMemcpyDeviceToHost, s->st));
    WG_CUDA(cudaMemcpyAsync(act.data(), s->act, sizeof(uint32_t) * act.size(), cudaMemcpyDeviceToHost, s->st));
    WG_CUDA(cudaStreamSynchronize(s->st));
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            const size_t w = (size_t)i * wp + (j >> 5);
            const int z = (bits[w] >> (j & 31)) & 1u, a = (act[w] >> (j & 31)) & 1u;
            // nonzero but not active away from the boundary lines: a Neumann ghost cell (-1)
            const bool line = i == 0 || i == nx - 1 || j == 0 || j == ny - 1;
            xy[(size_t)i * ny + j] = (int16_t)(z ? (a || line ? 1 : -1) : 0);
        }
    return WG_OK;
}

extern "C" wg_status wg_scene_neumann_records(wg_scene *s, wg_neumann_bc *out, int32_t capacity, int32_t *count)
{
    if (!s || !count) { set_error("NULL argument"); return WG_ERR_INVALID; }
    if (!s->prm.bc_neumann) { *count = 0; return WG_OK; }
    if (s->nrec_all > 0 && !s->nrec_dev) {
        set_error("the records of this scene came from the host (wg_scene_set_neumann)");
        return WG_ERR_STATE;
    }
    *count = s->nrec_all;
    if (!out) return WG_OK;
    if (capacity < s->nrec_all) { set_error("%d records, room for %d", s->nrec_all, capacity); return WG_ERR_INVALID; }
    if (s->nrec_all > 0) {
        WG_CUDA(cudaMemcpyAsync(out, s->nrec_dev, sizeof(wg_neumann_bc) * s->nrec_all, cudaMemcpyDeviceToHost, s->st));
        WG_CUDA(cudaStreamSynchronize(s->st));
    }
    return WG_OK;
}
