/*
 * wave_oracle.h — CPU oracle for the wave stepper.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement, with runtime NX/NY, of the reference's hot path:
 *   evolve_wave_half / evolve_wave     wave_billiard.c:302-631
 *   oscillating_bc                     sub_wave.c:11965-12162
 *   wave_energy's evolve_wave_half     wave_energy.c:662-925
 *   compute_energy                     wave_common.c:453-472
 *   compute_energy_x                   wave_energy.c:292-302
 *   compute_energy_tblr                sub_wave_comp.c:1752-1858
 *   init_neumann_bc (ellipse/polygon)  sub_wave.c:13384-13761,13910-13947
 *   xy_in_billiard shapes              sub_wave.c:5712-6259
 *   init_ior_2d constant branch        sub_wave.c:12983-13002
 * Only tests/, the smoke check and bench.py's CPU-baseline leg may load it; the
 * product (libwavegpu.so) never links or calls it.
 *
 * Parity is pinned against the reference itself: oracle/build_ref.py compiles the
 * reference's own wave_billiard.c / wave_energy.c headlessly into oracle/_ref/ and
 * tests/test_oracle_vs_reference.py checks this restatement bit for bit against it;
 * tests/golden/ holds fixtures produced by that compiled reference.
 *
 * Layout: flat field[i*ny + j] (j contiguous), as the reference's rows.
 */
#ifndef WAVE_ORACLE_H
#define WAVE_ORACLE_H
#include <stdint.h>
#include "../include/wavegpu.h"

#ifdef __cplusplus
extern "C" {
#endif

double wo_oscillating_bc(const wg_params *p, int time, int j);

/* One update at step counter `time` (already incremented, as the reference's
 * `time++` at wave_billiard.c:315). */
void wo_evolve_wave_half(const wg_params *p, long time,
                         const double *phi_in, const double *psi_in, double *phi_out,
                         const int16_t *xy_in, const double *tcc, const double *tc,
                         const double *tgamma, const wg_neumann_bc *nbc, int n_nbc);

/* nsteps updates with the 3-buffer rotation of evolve_wave; *time is advanced.
 * After the call the newest level is in bufs[0] when nsteps % 3 == 0; in general
 * the function returns the index (0..2) of the buffer holding the newest level and
 * writes the index of the previous level to *prev. */
int wo_run(const wg_params *p, long *time, int nsteps, double *bufs[3],
           const int16_t *xy_in, const double *tcc, const double *tc, const double *tgamma,
           const wg_neumann_bc *nbc, int n_nbc, int *prev);

/* wave_energy.c:662-913 with its static tables built from the mask. */
void wo_evolve_wave_half_energy(const wg_params *p, long time,
                                const double *phi_in, const double *psi_in, double *phi_out,
                                const int16_t *xy_in);

double wo_compute_energy(const wg_params *p, const double *phi, const double *psi,
                         const int16_t *xy_in, int i, int j);
void wo_energy_x(const wg_params *p, const double *phi, const double *psi,
                 const int16_t *xy_in, double *out /* nx */);
void wo_energy_tblr(const wg_params *p, const double *phi, const double *psi,
                    const int16_t *xy_in, int ileft, int iright, double out[6]);
/* Sum of compute_energy over all cells: naive (reference order, i outer) and
 * Neumaier-compensated. */
double wo_energy_total_naive(const wg_params *p, const double *phi, const double *psi,
                             const int16_t *xy_in);
double wo_energy_total_comp(const wg_params *p, const double *phi, const double *psi,
                            const int16_t *xy_in);

/* Mask generators (xy_in_billiard_single_domain) on the reference grid
 * (ij_to_xy, sub_wave.c:469-476). */
enum { WO_D_RECTANGLE = 0, WO_D_ELLIPSE = 1, WO_D_STADIUM = 2, WO_D_POLYGON = 8,
       WO_D_CIRCLES = 20, WO_D_CIRCLES_IN_RECT = 201 };
typedef struct { double xc, yc, radius; int active; } wo_circle;
void wo_mask(const wg_params *p, int domain, double lambda, int npoly, double apoly,
             const wo_circle *circles, int ncircles, int16_t *xy_out);

/* init_ior_2d constant/two-speed branch (sub_wave.c:12983-13002). */
void wo_init_ior(const wg_params *p, const int16_t *xy_in, double *tcc, double *tc, double *tgamma);
/* compute_energy and the compute_energy_flux velocity/gradients at the sampled cells
 * of draw_wave_highres_palette (arrays [row][col], row = j/size, col = i/size). */
void wo_frame_cells(const wg_params *p, const double *phi, const double *psi, const int16_t *xy_in, int size,
                    double *energy, double *vel, double *gx, double *gy);
/* add_circular_wave (wave_common.c:337-351) on flat [nx][ny] arrays. */
void wo_add_circular_wave(const wg_params *p, double init_amp, double factor, double x, double y,
                          double variance, double wavelength, double *phi, const int16_t *xy_in);

/* init_neumann_bc for D_ELLIPSE (domain 1) / D_POLYGON (domain 8); marks ghost cells
 * -1 in xy_in and returns the record count (or -1 on overflow). */
int wo_init_neumann(const wg_params *p, int domain, double lambda, int npoly, double apoly,
                    int16_t *xy_in, wg_neumann_bc *out, int max_records);

#ifdef __cplusplus
}
#endif
#endif
