/*
 * wavegpu_dropin.h — drop-in replacement of the reference's stepper for a
 * wave_billiard-style program.
 *
 * Include it after global_pdes.c and the configuration #defines, in place of the
 * program's own definitions of evolve_wave_half / evolve_wave (wave_billiard.c:
 * 302-631), and link with -lwavegpu.  The functions below keep the reference's
 * names and signatures (row-pointer fields `double *phi[NX]`, t_neumann_bc records,
 * the global n_neumann_points); the first call turns the program's macros into a
 * wg_params and configures the library.  Errors print wg_last_error() and exit, as
 * the reference has no error path for its stepper.
 *
 * By default every call copies the fields to the GPU and back (host arrays are
 * current after each call, as the reference's are).  Define WAVEGPU_RESIDENT before
 * including this header to keep the fields in HBM between calls; then call
 * wavegpu_sync() before the host reads phi/psi (draw, energy) and wavegpu_invalidate()
 * after the host writes them (e.g. the reference's own add_circular_wave; its device
 * counterpart wavegpu_add_circular_wave below needs neither).
 */
#ifndef WAVEGPU_DROPIN_H
#define WAVEGPU_DROPIN_H

#include <stdio.h>
#include <stdlib.h>
#include "wavegpu.h"

#ifndef OSCIL_LEFT_YSHIFT
#define OSCIL_LEFT_YSHIFT 0.0
#endif
#ifndef OMEGA_B
#define OMEGA_B OMEGA
#endif
#ifndef OSCIL_YMID
#define OSCIL_YMID 0.0
#endif
#ifndef WAVE_PACKET_SHIFT
#define WAVE_PACKET_SHIFT 200.0
#endif
#ifndef INITIAL_SHIFT
#define INITIAL_SHIFT 20.0
#endif
#ifndef ACHIRP
#define ACHIRP 0.25
#endif
#ifndef DAMPING
#define DAMPING 0.0
#endif

static void wavegpu_check_(wg_status s, const char *what)
{
    if (s != WG_OK) {
        fprintf(stderr, "wavegpu: %s failed: %s\n", what, wg_last_error());
        exit(1);
    }
}

/* wg_params from the program's compile-time configuration (wave_billiard.c:46-285). */
static void wavegpu_params_from_macros(wg_params *p)
{
    wg_params_default(p, NX, NY);
    p->b_cond = B_COND;
    p->twospeeds = TWOSPEEDS;
    p->bc_neumann = BC_NEUMANN;
    p->oscillate_left = OSCILLATE_LEFT;
    p->oscillate_topbot = OSCILLATE_TOPBOT;
    p->oscillation_schedule = OSCILLATION_SCHEDULE;
    p->floor_clamp = FLOOR;
    p->xmin = XMIN; p->xmax = XMAX; p->ymin = YMIN; p->ymax = YMAX;
    p->courant = COURANT; p->courantb = COURANTB;
    p->gamma = GAMMA; p->gammab = GAMMAB;
    p->kappa = KAPPA; p->kappa_sides = KAPPA_SIDES; p->kappa_topbot = KAPPA_TOPBOT;
    p->gamma_sides = GAMMA_SIDES; p->gamma_topbot = GAMMA_TOPBOT;
    p->omega = OMEGA; p->omega_b = OMEGA_B; p->amplitude = AMPLITUDE;
    p->damping = DAMPING; p->achirp = ACHIRP;
    p->oscil_ymax = OSCIL_YMAX; p->oscil_ymid = OSCIL_YMID; p->oscil_left_yshift = OSCIL_LEFT_YSHIFT;
    p->initial_variance = INITIAL_VARIANCE; p->initial_shift = INITIAL_SHIFT;
    p->wave_packet_shift = WAVE_PACKET_SHIFT;
    p->vmax = VMAX;
    p->e_scale = E_SCALE;
}

static void wavegpu_ensure_(void)
{
    static int done = 0;
    if (!done) {
        wg_params p;
        wavegpu_params_from_macros(&p);
        wavegpu_check_(wg_dropin_configure(&p), "wg_dropin_configure");
#ifdef WAVEGPU_RESIDENT
        wavegpu_check_(wg_dropin_set_mode(WG_DROPIN_RESIDENT), "wg_dropin_set_mode");
#endif
        done = 1;
    }
}

static inline void wavegpu_sync(void) { wavegpu_check_(wg_dropin_sync(), "wg_dropin_sync"); }
static inline void wavegpu_invalidate(void) { wavegpu_check_(wg_dropin_invalidate(), "wg_dropin_invalidate"); }

/* evolve_wave_half (wave_billiard.c:302-610) */
static void evolve_wave_half(double *phi_in[NX], double *psi_in[NX], double *phi_out[NX], short int *xy_in[NX],
                             double *tcc[NX], double *tc[NX], double *tgamma[NX],
                             t_neumann_bc neumann_bc[N_NEUMANN_POINTS])
{
    wavegpu_ensure_();
    wavegpu_check_(wg_evolve_wave_half(phi_in, psi_in, phi_out, (int16_t **)xy_in, tcc, tc, tgamma,
                                       (const wg_neumann_bc *)neumann_bc, BC_NEUMANN ? n_neumann_points : 0),
                   "evolve_wave_half");
}

/* evolve_wave (wave_billiard.c:613-631) */
static void evolve_wave(double *phi[NX], double *psi[NX], double *tmp[NX], short int *xy_in[NX],
                        double *tcc_table[NX], double *tc_table[NX], double *tgamma_table[NX],
                        t_neumann_bc neumann_bc[N_NEUMANN_POINTS])
{
    wavegpu_ensure_();
    wavegpu_check_(wg_evolve_wave(phi, psi, tmp, (int16_t **)xy_in, tcc_table, tc_table, tgamma_table,
                                  (const wg_neumann_bc *)neumann_bc, BC_NEUMANN ? n_neumann_points : 0),
                   "evolve_wave");
}

/* phi[i][j] for SAVE_TIME_SERIES sampling (wave_billiard.c:900-908): with
 * WAVEGPU_RESIDENT one cell of the device copy is read, without a full wavegpu_sync(). */
static double wavegpu_cell(double *phi[NX], int i, int j)
{
    double v = 0.0;
    wavegpu_ensure_();
    wavegpu_check_(wg_dropin_cell(phi, i, j, &v), "wg_dropin_cell");
    return v;
}

/* add_circular_wave (wave_common.c:337-351) on the GPU, with the program's INITIAL_AMP,
 * INITIAL_VARIANCE and INITIAL_WAVELENGTH.  With WAVEGPU_RESIDENT it adds the pulse to the
 * device copy of phi, so the periodic re-injection of animation() (wave_billiard.c:916-934)
 * needs no wavegpu_invalidate(); without it the host rows are updated as the reference's
 * function would update them. */
#if defined(INITIAL_AMP) && defined(INITIAL_VARIANCE) && defined(INITIAL_WAVELENGTH)
static void wavegpu_add_circular_wave(double factor, double x, double y, double *phi[NX], double *psi[NX],
                                      short int *xy_in[NX])
{
    wavegpu_ensure_();
    wavegpu_check_(wg_dropin_add_circular_wave(INITIAL_AMP, factor, x, y, INITIAL_VARIANCE, INITIAL_WAVELENGTH, phi,
                                               psi, (int16_t **)xy_in),
                   "add_circular_wave");
}
#endif

#endif /* WAVEGPU_DROPIN_H */
