/*
 * ref_driver.c — headless driver around the reference's own code (test
 * infrastructure).  oracle/build_ref.py compiles it once per configuration with
 * REF_TU naming the generated, macro-patched reference translation unit:
 *   REF_KIND_WB   wave_billiard.c: evolve_wave / evolve_wave_half / compute_energy
 *   REF_KIND_WE   wave_energy.c: its evolve_wave variant, compute_energy_x/_tblr
 *   REF_KIND_OSC  oscillating_bc only
 *   REF_FULL      the whole program is in the TU (setup functions available)
 *
 * Usage: ref_<variant> <in.bin> <out.bin>.  The input holds a header of 16 int64,
 * 4 doubles, circles, then the fields; see oracle/refio.py for the exact layout.
 * Modes: 0 STEP, 1 SETUP (full builds), 2 TIME, 3 OSC, 4 PULSE (full builds:
 * add_circular_wave(hd[0], hd[2], hd[3], phi, psi, xy_in) on the given fields).
 * STEP with h[14] = R > 0 also reports the total energy (the sum of compute_energy
 * over every cell) after every R updates; the reports follow the usual output.
 * 5 FRAME (full builds): the colours of draw_wave_highres_palette's sampled cells, from
 * the reference's own wave_value (wave_common.c) with the palette COL_TURBO, for plot
 * mode h[12], sampling step h[7], h[13] frames at times h[8], h[8]+1, ... on the given
 * phi/psi (the running sums of the mean, average and flux modes carried between
 * them), scale hd[0].  Output: the last frame's rgb doubles [NY/size][NX/size][3] and
 * its values [NY/size][NX/size], then init_fade_table's factors at the same cells.
 */
#define main ref_main
#include REF_TU
#undef main
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

enum { M_STEP = 0, M_SETUP = 1, M_TIME = 2, M_OSC = 3, M_PULSE = 4, M_FRAME = 5 };

static void rd(FILE *f, void *p, size_t n)
{
    if (n && fread(p, 1, n, f) != n) { fprintf(stderr, "ref_driver: short read\n"); exit(2); }
}
static void wr(FILE *f, const void *p, size_t n)
{
    if (n && fwrite(p, 1, n, f) != n) { fprintf(stderr, "ref_driver: short write\n"); exit(2); }
}

#ifndef REF_KIND_OSC
static t_neumann_bc drv_nbc[N_NEUMANN_POINTS];

/* total energy of a field pair: compute_energy summed over every cell (rows in
 * parallel, each row in order, then the rows in order) */
static double total_energy(double **a, double **b, short int **xyr)
{
    static double rowsum[NX];
    #pragma omp parallel for
    for (int i = 0; i < NX; i++) {
        double e = 0.0;
        for (int j = 0; j < NY; j++) e += compute_energy(a, b, xyr, i, j);
        rowsum[i] = e;
    }
    double e = 0.0;
    for (int i = 0; i < NX; i++) e += rowsum[i];
    return e;
}
#endif

int main(int argc, char **argv)
{
    if (argc < 3) { fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]); return 2; }
    FILE *fi = fopen(argv[1], "rb");
    if (!fi) { perror("in"); return 2; }
    int64_t h[16];
    double hd[4];
    rd(fi, h, sizeof h);
    rd(fi, hd, sizeof hd);
    const int64_t nx = h[1], ny = h[2], mode = h[3], nsteps = h[4], n_nbc = h[5];
    const int64_t ncirc = h[6], src_on = h[9], src_i = h[10], src_j = h[11], report = h[14];
    const double src_amp = hd[0], src_period = hd[1];
    if (h[0] != 0x57415645 || nx != NX || ny != NY) {
        fprintf(stderr, "ref_driver: header mismatch (built for %d x %d)\n", NX, NY);
        return 3;
    }
    double *circ = malloc(sizeof(double) * 3 * (ncirc > 0 ? ncirc : 1));
    rd(fi, circ, sizeof(double) * 3 * ncirc);
    FILE *fo = fopen(argv[2], "wb");
    if (!fo) { perror("out"); return 2; }

#ifdef REF_KIND_OSC
    /* h[12] = time count, followed by that many int32 times */
    {
        int64_t nt = h[12];
        int32_t *times = malloc(sizeof(int32_t) * (nt > 0 ? nt : 1));
        rd(fi, times, sizeof(int32_t) * nt);
        for (int64_t a = 0; a < nt; a++)
            for (int j = 0; j < NY; j++) {
                double v = oscillating_bc(times[a], j);
                wr(fo, &v, sizeof v);
            }
        fclose(fo);
        return 0;
    }
#else
    const size_t cells = (size_t)NX * NY;
    double *A[6];
    double *rows[6][NX];
    short int *xyrows[NX];
    short int *xy = calloc(cells, sizeof(short int));
    for (int k = 0; k < 6; k++) {
        A[k] = calloc(cells, sizeof(double));
        if (mode != M_TIME) rd(fi, A[k], sizeof(double) * cells);
        for (int i = 0; i < NX; i++) rows[k][i] = A[k] + (size_t)i * NY;
    }
    if (mode != M_TIME) rd(fi, xy, sizeof(short int) * cells);
    for (int i = 0; i < NX; i++) xyrows[i] = xy + (size_t)i * NY;
    if (n_nbc > N_NEUMANN_POINTS) { fprintf(stderr, "too many records\n"); return 3; }
    if (mode != M_TIME) rd(fi, drv_nbc, sizeof(t_neumann_bc) * n_nbc);
    fclose(fi);
    int64_t nrec = n_nbc;
    double **phi = rows[0], **psi = rows[1], **tmp = rows[2];
    double **tcc = rows[3], **tc = rows[4], **tg = rows[5];
    double elapsed = 0.0;
    int64_t nrep = 0;
    double *reports = NULL;
    (void)tcc; (void)tc; (void)tg; (void)circ; (void)src_i; (void)src_j;
    (void)src_on; (void)src_amp; (void)src_period;

    courant2 = COURANT * COURANT;
    courantb2 = COURANTB * COURANTB;
#ifdef REF_KIND_WB
    n_neumann_points = (int)nrec;
#endif

    if (mode == M_TIME) {
#if defined(REF_FULL) && defined(REF_KIND_WB)
        /* inputs made by the reference's own set-up: mask (init_wave_flat with the
         * given circles), tables (init_ior_2d), one pulse (add_circular_wave at
         * hd[2], hd[3]), psi = phi; then nsteps timed updates */
        ncircles = (int)ncirc;
        for (int c = 0; c < ncirc; c++) {
            circles[c].xc = circ[3 * c];
            circles[c].yc = circ[3 * c + 1];
            circles[c].radius = circ[3 * c + 2];
            circles[c].active = 1;
        }
        init_wave_flat(phi, psi, xyrows);
        init_ior_2d(xyrows, tcc, tc, tg, 0.0);
        add_circular_wave(1.0, hd[2], hd[3], phi, psi, xyrows);
        for (int i = 0; i < NX; i++) memcpy(psi[i], phi[i], sizeof(double) * NY);
        double **b[3] = {phi, psi, tmp};
        int cur = 0, prv = 1, fre = 2;
        const int64_t nseg = h[13] > 0 ? h[13] : 1;  /* timed segments of nsteps updates */
        int64_t done = 0;
        double *seg = calloc(nseg, sizeof(double));
        for (int64_t g = 0; g < nseg; g++) {
            double t0 = omp_get_wtime();
            for (int64_t s = 0; s < nsteps; s++, done++) {
                evolve_wave_half(b[cur], b[prv], b[fre], xyrows, tcc, tc, tg, drv_nbc);
                if (src_on) b[fre][src_i][src_j] += src_amp * sin(6.283185307179586 * (double)(done + 1) / src_period);
                int nc = fre, np = cur, nf = prv;
                cur = nc; prv = np; fre = nf;
            }
            seg[g] = omp_get_wtime() - t0;
            elapsed += seg[g];
        }
        double e = 0.0;
        for (int i = 0; i < NX; i++)
            for (int j = 0; j < NY; j++) e += compute_energy(b[cur], b[prv], xyrows, i, j);
        int64_t threads = omp_get_max_threads();
        wr(fo, &elapsed, sizeof elapsed);
        wr(fo, &e, sizeof e);
        wr(fo, &threads, sizeof threads);
        wr(fo, seg, sizeof(double) * nseg);
        fclose(fo);
        return 0;
#else
        fprintf(stderr, "TIME needs a full build\n");
        return 3;
#endif
    }
    if (mode == M_FRAME) {
#if defined(REF_FULL) && defined(REF_KIND_WB)
        const int size = (int)h[7], plot = (int)h[12];
        const int64_t nframes = h[13] > 0 ? h[13] : 1, t0 = h[8];
        const int w = NX / size, hh = NY / size;
        double *te[NX], *ae[NX], *cs[NX];
        double *flux = calloc((size_t)4 * NX * NY, sizeof(double));
        double *fade = calloc(cells, sizeof(double));
        double *rgbout = calloc((size_t)3 * w * hh, sizeof(double)), *valout = calloc((size_t)w * hh, sizeof(double));
        for (int i = 0; i < NX; i++) {
            te[i] = calloc(NY, sizeof(double));
            ae[i] = calloc(NY, sizeof(double));
            cs[i] = calloc(NY, sizeof(double));
        }
        init_fade_table(tcc, xyrows, fade);
        for (int64_t f = 0; f < nframes; f++)
            for (int i = 0; i < NX; i += size)
                for (int j = 0; j < NY; j += size) {
                    double rgb[3];
                    const double v = wave_value(i, j, phi, psi, te, ae, flux, cs, xyrows, hd[0], (int)(t0 + f), plot,
                                                COL_TURBO, rgb);
                    if (f == nframes - 1 && i / size < w && j / size < hh) {
                        const size_t k = (size_t)(j / size) * w + i / size;
                        for (int c = 0; c < 3; c++) rgbout[3 * k + c] = rgb[c];
                        valout[k] = v;
                    }
                }
        wr(fo, rgbout, sizeof(double) * 3 * w * hh);
        wr(fo, valout, sizeof(double) * w * hh);
        for (int j = 0; j < hh; j++)
            for (int i = 0; i < w; i++) wr(fo, &fade[(size_t)(i * size) * NY + j * size], sizeof(double));
        fclose(fo);
        return 0;
#else
        fprintf(stderr, "FRAME needs a full build\n");
        return 3;
#endif
    }
    if (mode == M_PULSE) {
#if defined(REF_FULL) && defined(REF_KIND_WB)
        add_circular_wave(hd[0], hd[2], hd[3], phi, psi, xyrows);
#else
        fprintf(stderr, "PULSE needs a full build\n");
        return 3;
#endif
    } else if (mode == M_SETUP) {
#if defined(REF_FULL) && defined(REF_KIND_WB)
        ncircles = (int)ncirc;
        for (int c = 0; c < ncirc; c++) {
            circles[c].xc = circ[3 * c];
            circles[c].yc = circ[3 * c + 1];
            circles[c].radius = circ[3 * c + 2];
            circles[c].active = 1;
        }
        init_wave_flat(phi, psi, xyrows);
        init_ior_2d(xyrows, tcc, tc, tg, 0.0);
        nrec = 0;
        if (BC_NEUMANN) nrec = init_neumann_bc(xyrows, drv_nbc, circles, 0);
#else
        fprintf(stderr, "SETUP needs a full build\n");
        return 3;
#endif
    } else {
        /* rotation state: which of phi/psi/tmp holds the newest level */
        double **b[3] = {phi, psi, tmp};
        int cur = 0, prv = 1, fre = 2;
        double t0 = omp_get_wtime();
#ifdef REF_KIND_WB
        if (report > 0) reports = calloc(nsteps / report + 1, sizeof(double));
        if (!src_on && report <= 0 && nsteps % 3 == 0) {
            for (int64_t s = 0; s < nsteps / 3; s++) evolve_wave(phi, psi, tmp, xyrows, tcc, tc, tg, drv_nbc);
        } else {
            for (int64_t s = 0; s < nsteps; s++) {
                evolve_wave_half(b[cur], b[prv], b[fre], xyrows, tcc, tc, tg, drv_nbc);
                if (src_on) b[fre][src_i][src_j] += src_amp * sin(6.283185307179586 * (double)(s + 1) / src_period);
                int nc = fre, np = cur, nf = prv;
                cur = nc; prv = np; fre = nf;
                if (report > 0 && (s + 1) % report == 0) reports[nrep++] = total_energy(b[cur], b[prv], xyrows);
            }
        }
#else /* REF_KIND_WE */
        if (nsteps % 3 == 0) {
            for (int64_t s = 0; s < nsteps / 3; s++) evolve_wave(phi, psi, tmp, xyrows);
        } else {
            for (int64_t s = 0; s < nsteps; s++) {
                evolve_wave_half(b[cur], b[prv], b[fre], xyrows);
                int nc = fre, np = cur, nf = prv;
                cur = nc; prv = np; fre = nf;
            }
        }
#endif
        elapsed = omp_get_wtime() - t0;
        /* present the newest level as "phi", the previous one as "psi" */
#ifdef REF_KIND_WB
        if (!(nsteps % 3 == 0 && !src_on && report <= 0)) {
#else
        if (!(nsteps % 3 == 0 && !src_on)) {
#endif
            double *o0 = A[0], *o1 = A[1], *o2 = A[2];
            double *src[3] = {o0, o1, o2};
            double *newest = src[cur], *prev = src[prv], *third = src[fre];
            A[0] = newest; A[1] = prev; A[2] = third;
        }
    }

    /* outputs: fields, mask, records, energies, elapsed */
    for (int k = 0; k < 6; k++) wr(fo, A[k], sizeof(double) * cells);
    wr(fo, xy, sizeof(short int) * cells);
    wr(fo, &nrec, sizeof nrec);
    wr(fo, drv_nbc, sizeof(t_neumann_bc) * nrec);
    for (int i = 0; i < NX; i++) rows[0][i] = A[0] + (size_t)i * NY;
    for (int i = 0; i < NX; i++) rows[1][i] = A[1] + (size_t)i * NY;
    double etot = 0.0;
    if (mode != M_TIME) {
        for (int i = 0; i < NX; i++)
            for (int j = 0; j < NY; j++) etot += compute_energy(rows[0], rows[1], xyrows, i, j);
    }
    wr(fo, &etot, sizeof etot);
    double *ex = calloc(NX, sizeof(double));
    double tblr[6] = {0, 0, 0, 0, 0, 0};
#ifdef REF_KIND_WE
    if (mode != M_TIME) {
        for (int i = 0; i < NX; i++) ex[i] = compute_energy_x(i, rows[0], rows[1], xyrows);
        ncircles = (int)ncirc;
        for (int c = 0; c < ncirc; c++) {
            circles[c].xc = circ[3 * c];
            circles[c].yc = circ[3 * c + 1];
            circles[c].radius = circ[3 * c + 2];
            circles[c].active = 1;
        }
        compute_energy_tblr(rows[0], rows[1], xyrows, tblr);
    }
#endif
    wr(fo, ex, sizeof(double) * NX);
    wr(fo, tblr, sizeof tblr);
    wr(fo, &elapsed, sizeof elapsed);
    int64_t threads = omp_get_max_threads();
    wr(fo, &threads, sizeof threads);
    wr(fo, &nrep, sizeof nrep);
    wr(fo, reports, sizeof(double) * nrep);
    fclose(fo);
    return 0;
#endif
}
