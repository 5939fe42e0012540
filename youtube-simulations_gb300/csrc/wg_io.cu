// wg_io.cu — frame files and time-series probes (the output side of animation()).
//
// wg_write_tiff: the file writetiff (sub_wave.c:62-122) makes from the GL window with
// libtiff, written here from an RGB8 frame without libtiff: baseline TIFF, little
// endian, 8-bit RGB, uncompressed, one row per strip, ORIENTATION_BOTLEFT, the
// description as ImageDescription.  writetiff stores GL row k (k = 0 at the bottom) as
// scanline height-1-k; the frames here have row 0 at the bottom, so scanline s holds
// frame row height-1-s, as there.  wg_write_ppm: binary PPM (P6), top row first.
//
// Probes: SAVE_TIME_SERIES (wave_billiard.c:667-672, 900-908) samples phi at given
// cells; a scene with probes records phi at each probe after every update.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "wg_internal.h"
#include "wg_scene.h"

namespace wg {

template <class T>
__global__ void k_probe(const T *__restrict__ phi, int pitch, const int2 *__restrict__ cells, int n,
                        double *__restrict__ out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = (double)phi[(size_t)cells[k].x * pitch + cells[k].y];
}

void probe_record(wg_scene *s)
{
    if (!s->probe_n || s->probe_count >= s->probe_cap) return;
    double *dst = s->probe_buf + (size_t)s->probe_count * s->probe_n;
    if (s->prec == WG_FP32) k_probe<float><<<(s->probe_n + 127) / 128, 128, 0, s->st>>>((const float *)s->f[s->cur], s->pitch, s->probe_cells, s->probe_n, dst);
    else k_probe<double><<<(s->probe_n + 127) / 128, 128, 0, s->st>>>((const double *)s->f[s->cur], s->pitch, s->probe_cells, s->probe_n, dst);
    s->probe_count++;
    s->launches++;
}

static void put16(std::vector<uint8_t> &b, size_t at, uint16_t v) { b[at] = v & 0xFF; b[at + 1] = v >> 8; }
static void put32(std::vector<uint8_t> &b, size_t at, uint32_t v)
{
    for (int k = 0; k < 4; k++) b[at + k] = (v >> (8 * k)) & 0xFF;
}

}  // namespace wg

using namespace wg;

extern "C" {

wg_status wg_write_tiff(const char *path, const char *description, const uint8_t *rgb, int32_t width, int32_t height)
{
    if (!path || !rgb || width < 1 || height < 1) { set_error("bad arguments"); return WG_ERR_INVALID; }
    const std::string desc = description ? description : "";
    const uint32_t row = (uint32_t)width * 3, h = (uint32_t)height;
    const int ntags = 12;
    const size_t ifd = 8, ifd_bytes = 2 + 12 * (size_t)ntags + 4;
    const size_t bps_at = ifd + ifd_bytes;                 // 3 x SHORT
    const size_t desc_at = bps_at + 6;                     // ASCII, NUL-terminated
    const size_t offs_at = (desc_at + desc.size() + 1 + 3) & ~(size_t)3;
    const size_t cnts_at = offs_at + 4 * (size_t)h;
    const size_t data_at = cnts_at + 4 * (size_t)h;
    std::vector<uint8_t> b(data_at + (size_t)row * h, 0);
    b[0] = 'I';
    b[1] = 'I';
    put16(b, 2, 42);
    put32(b, 4, (uint32_t)ifd);
    put16(b, ifd, ntags);
    size_t e = ifd + 2;
    auto tag = [&](uint16_t id, uint16_t type, uint32_t count, uint32_t value) {
        put16(b, e, id);
        put16(b, e + 2, type);
        put32(b, e + 4, count);
        if (type == 3 && count == 1) put16(b, e + 8, (uint16_t)value);
        else put32(b, e + 8, value);
        e += 12;
    };
    const uint16_t SHORT = 3, LONG = 4, ASCII = 2;
    tag(256, LONG, 1, (uint32_t)width);                    // ImageWidth
    tag(257, LONG, 1, h);                                  // ImageLength
    tag(258, SHORT, 3, (uint32_t)bps_at);                  // BitsPerSample 8,8,8
    tag(259, SHORT, 1, 1);                                 // Compression: none
    tag(262, SHORT, 1, 2);                                 // Photometric: RGB
    tag(270, ASCII, (uint32_t)desc.size() + 1, (uint32_t)desc_at);  // ImageDescription
    tag(273, LONG, h, h == 1 ? (uint32_t)data_at : (uint32_t)offs_at);  // StripOffsets
    tag(274, SHORT, 1, 4);                                 // Orientation: BOTLEFT
    tag(277, SHORT, 1, 3);                                 // SamplesPerPixel
    tag(278, LONG, 1, 1);                                  // RowsPerStrip
    tag(279, LONG, h, h == 1 ? row : (uint32_t)cnts_at);   // StripByteCounts
    tag(284, SHORT, 1, 1);                                 // PlanarConfiguration: contiguous
    put32(b, e, 0);                                        // no next IFD
    for (int k = 0; k < 3; k++) put16(b, bps_at + 2 * k, 8);
    memcpy(&b[desc_at], desc.c_str(), desc.size() + 1);
    for (uint32_t s = 0; s < h; s++) {
        put32(b, offs_at + 4 * (size_t)s, (uint32_t)(data_at + (size_t)s * row));
        put32(b, cnts_at + 4 * (size_t)s, row);
        memcpy(&b[data_at + (size_t)s * row], rgb + (size_t)(h - 1 - s) * row, row);
    }
    FILE *f = fopen(path, "wb");
    if (!f) { set_error("cannot open %s for writing", path); return WG_ERR_INVALID; }
    const bool ok = fwrite(b.data(), 1, b.size(), f) == b.size();
    if (fclose(f) != 0 || !ok) { set_error("short write to %s", path); return WG_ERR_INVALID; }
    return WG_OK;
}

wg_status wg_write_ppm(const char *path, const uint8_t *rgb, int32_t width, int32_t height)
{
    if (!path || !rgb || width < 1 || height < 1) { set_error("bad arguments"); return WG_ERR_INVALID; }
    FILE *f = fopen(path, "wb");
    if (!f) { set_error("cannot open %s for writing", path); return WG_ERR_INVALID; }
    bool ok = fprintf(f, "P6\n%d %d\n255\n", width, height) > 0;
    const size_t row = (size_t)width * 3;
    for (int r = height - 1; r >= 0 && ok; r--) ok = fwrite(rgb + (size_t)r * row, 1, row, f) == row;
    if (fclose(f) != 0 || !ok) { set_error("short write to %s", path); return WG_ERR_INVALID; }
    return WG_OK;
}

wg_status wg_scene_set_probes(wg_scene *s, int32_t n, const int32_t *i, const int32_t *j, int32_t capacity)
{
    if (!s || n < 0 || (n > 0 && (!i || !j || capacity < 1))) { set_error("bad arguments"); return WG_ERR_INVALID; }
    for (int k = 0; k < n; k++)
        if (i[k] < 0 || i[k] >= s->prm.nx || j[k] < 0 || j[k] >= s->prm.ny) {
            set_error("probe %d at (%d, %d) is outside the %d x %d grid", k, i[k], j[k], s->prm.nx, s->prm.ny);
            return WG_ERR_INVALID;
        }
    WG_CUDA(cudaStreamSynchronize(s->st));
    if (s->probe_cells) cudaFree(s->probe_cells);
    if (s->probe_buf) cudaFree(s->probe_buf);
    s->probe_cells = nullptr;
    s->probe_buf = nullptr;
    s->probe_n = s->probe_cap = s->probe_count = 0;
    if (n == 0) return WG_OK;
    std::vector<int2> cells(n);
    for (int k = 0; k < n; k++) cells[k] = make_int2(i[k], j[k]);
    WG_CUDA(cudaMalloc(&s->probe_cells, sizeof(int2) * n));
    WG_CUDA(cudaMalloc(&s->probe_buf, sizeof(double) * (size_t)n * capacity));
    WG_CUDA(cudaMemcpy(s->probe_cells, cells.data(), sizeof(int2) * n, cudaMemcpyHostToDevice));
    s->probe_n = n;
    s->probe_cap = capacity;
    return WG_OK;
}

wg_status wg_scene_read_probes(wg_scene *s, double *out, int32_t max_updates, int32_t *count)
{
    if (!s || !count || (max_updates > 0 && !out)) { set_error("bad arguments"); return WG_ERR_INVALID; }
    const int c = s->probe_count < max_updates ? s->probe_count : max_updates;
    if (c > 0)
        WG_CUDA(cudaMemcpyAsync(out, s->probe_buf, sizeof(double) * (size_t)c * s->probe_n, cudaMemcpyDeviceToHost, s->st));
    WG_CUDA(cudaStreamSynchronize(s->st));
    *count = c;
    if (c < s->probe_count && c > 0) {  // keep the rest, in order (through a temporary: the ranges overlap)
        const size_t rest = sizeof(double) * (size_t)(s->probe_count - c) * s->probe_n;
        double *tmp = nullptr;
        WG_CUDA(cudaMalloc(&tmp, rest));
        cudaError_t e = cudaMemcpy(tmp, s->probe_buf + (size_t)c * s->probe_n, rest, cudaMemcpyDeviceToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(s->probe_buf, tmp, rest, cudaMemcpyDeviceToDevice);
        cudaFree(tmp);
        if (e != cudaSuccess) return cuda_fail(e, "wg_scene_read_probes");
    }
    s->probe_count -= c;
    return WG_OK;
}

}  // extern "C"
