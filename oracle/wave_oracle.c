/*
 * wave_oracle.c — CPU oracle (test infrastructure only; see wave_oracle.h).
 *
 * Every function restates the reference statement by statement, with the same
 * operation order, so that with -ffp-contract=off (no FMA contraction) its FP64
 * results are bit-identical to the compiled reference.  Build: oracle/Makefile.
 */
#include "wave_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* The reference's truncated constants (global_pdes.c:8-10). */
#define R_PI  3.141592654
#define R_DPI 6.283185307
#define R_PID 1.570796327

#define BEAM_BC(p) ((p)->oscillation_schedule == WG_OSC_BEAM_SINE || \
                    (p)->oscillation_schedule == WG_OSC_BEAM_SINE_DECREASING || \
                    (p)->oscillation_schedule == WG_OSC_BEAM_SINE_TWOPERIODS || \
                    (p)->oscillation_schedule == WG_OSC_BEAM_SINE_CHIRP)

/* xy_to_ij, second coordinate only (sub_wave.c:412-422). */
static int wo_y_to_j(const wg_params *p, double y)
{
    double y1 = (y - p->ymin) / (p->ymax - p->ymin);
    return (int)(y1 * (double)p->ny);
}

/* ij_to_xy (sub_wave.c:469-476). */
static void wo_ij_to_xy(const wg_params *p, int i, int j, double xy[2])
{
    xy[0] = p->xmin + ((double)i) * (p->xmax - p->xmin) / ((double)p->nx);
    xy[1] = p->ymin + ((double)j) * (p->ymax - p->ymin) / ((double)p->ny);
}

/* oscillating_bc (sub_wave.c:11965-12162). */
double wo_oscillating_bc(const wg_params *p, int time, int j)
{
    const int NY = p->ny;
    const double OMEGA = p->omega, AMPLITUDE = p->amplitude, DAMPING = p->damping;
    const double YSH = p->oscil_left_yshift;
    int jmin, jmax, jmid;
    double t, t1, phase, a, envelope, amp, dist2;

    switch (p->oscillation_schedule) {
    case WG_OSC_PERIODIC:
        if (YSH > 0.0) t = (double)time * OMEGA - (double)j * YSH / (double)NY;
        else t = (double)time * OMEGA + (double)(NY - j) * YSH / (double)NY;
        if (t < 0.0) return 0.0;
        return AMPLITUDE * cos(t) * exp(-(double)t * DAMPING);
    case WG_OSC_SLOWING:
        a = 0.0025;
        t = (double)time * OMEGA;
        if (YSH > 0.0) t -= (double)j * YSH / (double)NY;
        phase = t - a * t * t;
        return AMPLITUDE * cos(phase) * exp(-phase * DAMPING);
    case WG_OSC_WAVE_PACKET:
        t = (double)time * OMEGA;
        if (YSH > 0.0) t -= (double)j * YSH / (double)NY;
        a = sqrt(p->initial_variance) / OMEGA;
        phase = AMPLITUDE * cos(t);
        envelope = exp(-(t - p->initial_shift) * (t - p->initial_shift) / (a * a)) * sqrt(R_DPI / a);
        return phase * envelope;
    case WG_OSC_WAVE_PACKETS:
        t = (double)time * OMEGA;
        if (YSH > 0.0) t -= (double)j * YSH / (double)NY;
        t1 = t - (double)((int)(t / p->wave_packet_shift + 0.5)) * p->wave_packet_shift;
        a = sqrt(p->initial_variance) / OMEGA;
        phase = AMPLITUDE * cos(t);
        envelope = exp(-(t1 - p->initial_shift) * (t1 - p->initial_shift) / (a * a)) * sqrt(R_DPI / a);
        return phase * envelope;
    case WG_OSC_CHIRP:
        t = (double)time * OMEGA;
        if (YSH > 0.0) t -= (double)j * YSH / (double)NY;
        phase = t + p->achirp * t * t;
        return AMPLITUDE * sin(phase) * exp(-phase * DAMPING);
    case WG_OSC_BEAM:
    case WG_OSC_BEAM_TWOPERIODS:
        jmax = wo_y_to_j(p, p->oscil_ymax);
        jmin = NY - jmax;
        if (j < jmin) dist2 = (double)(jmin - 1 - j) * (p->ymax - p->ymin) / (double)NY;
        else if (j > jmax) dist2 = (double)(j - jmax) * (p->ymax - p->ymin) / (double)NY;
        else dist2 = 0.0;
        dist2 = 500.0 * dist2 * dist2;
        t = (double)time * OMEGA;
        if (YSH > 0.0) t -= (double)j * YSH / (double)NY;
        if (p->oscillation_schedule == WG_OSC_BEAM)
            amp = AMPLITUDE * cos(t) * exp(-(double)t * DAMPING);
        else
            amp = AMPLITUDE * (0.5 * cos(t) + 0.5 * cos(sqrt(7.0) * t)) * exp(-(double)t * DAMPING);
        amp *= exp(-dist2 / p->initial_variance);
        return amp;
    case WG_OSC_BEAM_GAUSSIAN:
        dist2 = (double)(j - NY / 2) * (p->ymax - p->ymin) / (double)NY;
        dist2 = dist2 * dist2;
        t = (double)time * OMEGA;
        if (YSH > 0.0) t -= (double)j * YSH / (double)NY;
        amp = AMPLITUDE * cos(t) * exp(-(double)t * DAMPING);
        amp *= exp(-dist2 / p->initial_variance);
        return amp;
    case WG_OSC_BEAM_SINE:
    case WG_OSC_BEAM_SINE_DECREASING:
    case WG_OSC_BEAM_SINE_TWOPERIODS:
    case WG_OSC_BEAM_SINE_CHIRP:
        jmax = wo_y_to_j(p, p->oscil_ymid + p->oscil_ymax);
        jmin = wo_y_to_j(p, p->oscil_ymid - p->oscil_ymax);
        jmid = (jmin + jmax) / 2;
        dist2 = (double)(j - jmid) / (double)(jmax - jmid);
        if (j > jmax) return 0.0;
        if (j < jmin) return 0.0;
        t = (double)time * OMEGA;
        if (YSH > 0.0) t -= (double)j * YSH / (double)NY;
        if (p->oscillation_schedule == WG_OSC_BEAM_SINE) {
            amp = AMPLITUDE * cos(t) * exp(-(double)t * DAMPING);
        } else if (p->oscillation_schedule == WG_OSC_BEAM_SINE_DECREASING) {
            a = p->initial_variance / (OMEGA * OMEGA);
            amp = AMPLITUDE * cos(t) * exp(-(double)(t - p->initial_shift) * (t - p->initial_shift) / a);
        } else if (p->oscillation_schedule == WG_OSC_BEAM_SINE_TWOPERIODS) {
            amp = AMPLITUDE * (0.5 * cos(t) + 0.5 * cos(sqrt(7.0) * t)) * exp(-(double)t * DAMPING);
        } else {
            phase = t + p->achirp * t * t;
            amp = AMPLITUDE * sin(phase) * exp(-phase * DAMPING);
        }
        amp *= cos(R_PID * dist2);
        return amp;
    case WG_OSC_TWO_WAVES:
        t = (double)time * OMEGA + (double)(NY - j) * YSH / (double)NY;
        t1 = (double)time * OMEGA + (double)(j)*YSH / (double)NY;
        if (j < NY / 2) amp = cos(t);
        else amp = cos(t1);
        return AMPLITUDE * amp;
    case WG_OSC_TWO_WAVES_ADDED:
        t = (double)time * OMEGA + (double)(NY - j) * YSH / (double)NY;
        t1 = (double)time * OMEGA + (double)(j)*YSH / (double)NY;
        amp = 0.0;
        if (t > 0.0) amp += cos(t);
        if (t1 > 0.0) amp += cos(t1);
        return AMPLITUDE * amp;
    case WG_OSC_TWOFREQ_TOPBOT:
        if (j > NY / 2) t = (double)time * OMEGA + (double)(NY - j) * YSH / (double)NY;
        else t = (double)time * p->omega_b + (double)(NY - j) * YSH / (double)NY;
        return AMPLITUDE * cos(t) * exp(-(double)t * DAMPING);
    default:
        return 0.0; /* the reference falls off the end of the switch */
    }
}

/* Point source of the project: phi_out[src] += A*sin(2*pi*t/P) after update t. */
static void wo_point_source(const wg_params *p, long time, double *phi_out)
{
    if (!p->src_on) return;
    phi_out[(size_t)p->src_i * p->ny + p->src_j] +=
        p->src_amp * sin(6.283185307179586 * (double)time / p->src_period);
}

#define F(a, i, j) (a)[(size_t)(i) * NY + (j)]

/* evolve_wave_half (wave_billiard.c:302-610). */
void wo_evolve_wave_half(const wg_params *p, long time,
                         const double *phi_in, const double *psi_in, double *phi_out,
                         const int16_t *xy_in, const double *tcc, const double *tc,
                         const double *tgamma, const wg_neumann_bc *nbc, int n_nbc)
{
    const int NX = p->nx, NY = p->ny, TWOSPEEDS = p->twospeeds;
    const double KAPPA = p->kappa, KAPPA_SIDES = p->kappa_sides, KAPPA_TOPBOT = p->kappa_topbot;
    const double GAMMA_SIDES = p->gamma_sides, GAMMA_TOPBOT = p->gamma_topbot;
    int i, j, iplus, iminus, nc, bc_jmin, bc_jmax;
    double delta, x, y, tb_shift = 0.0;

    if (p->oscillate_topbot)
        tb_shift = (int)((p->xmax - p->xmin) * (double)NX / (p->xmax - p->xmin));

    /* beam range of the OSCILLATE_LEFT boundary (wave_billiard.c:320-339) */
    if (p->oscillate_left && BEAM_BC(p)) {
        bc_jmax = wo_y_to_j(p, p->oscil_ymid + p->oscil_ymax);
        bc_jmin = wo_y_to_j(p, p->oscil_ymid - p->oscil_ymax);
    } else {
        bc_jmin = 0;
        bc_jmax = NY - 1;
    }
#define LEFT_BC(j) ((j) < NY - 1 && p->oscillate_left && (j) > bc_jmin && (j) < bc_jmax)

    /* bulk (wave_billiard.c:361-377) */
    for (i = 1; i < NX - 1; i++)
        for (j = 1; j < NY - 1; j++)
            if (TWOSPEEDS || F(xy_in, i, j) > 0) {
                x = F(phi_in, i, j);
                y = F(psi_in, i, j);
                delta = F(phi_in, i + 1, j) + F(phi_in, i - 1, j) + F(phi_in, i, j + 1) + F(phi_in, i, j - 1) - 4.0 * x;
                F(phi_out, i, j) = -y + 2 * x + F(tcc, i, j) * delta - KAPPA * x - F(tgamma, i, j) * (x - y);
            }

    /* Neumann gather (wave_billiard.c:379-389) */
    if (p->bc_neumann)
        for (nc = 0; nc < n_nbc; nc++)
            if (nbc[nc].active) {
                i = nbc[nc].i;
                j = nbc[nc].j;
                F(phi_out, i, j) = nbc[nc].nx * F(phi_in, nbc[nc].nbi1, nbc[nc].nbj1);
                F(phi_out, i, j) += nbc[nc].ny * F(phi_in, nbc[nc].nbi2, nbc[nc].nbj2);
            }

    /* left boundary (wave_billiard.c:393-431) */
    for (j = 1; j < NY - 1; j++) {
        if (LEFT_BC(j)) F(phi_out, 0, j) = wo_oscillating_bc(p, (int)time, j);
        else if (TWOSPEEDS || F(xy_in, 0, j) != 0) {
            x = F(phi_in, 0, j);
            y = F(psi_in, 0, j);
            switch (p->b_cond) {
            case WG_BC_DIRICHLET:
                delta = F(phi_in, 1, j) + F(phi_in, 0, j + 1) + F(phi_in, 0, j - 1) - 3.0 * x;
                F(phi_out, 0, j) = -y + 2 * x + F(tcc, 0, j) * delta - KAPPA * x - F(tgamma, 0, j) * (x - y);
                break;
            case WG_BC_PERIODIC:
                delta = F(phi_in, 1, j) + F(phi_in, NX - 1, j) + F(phi_in, 0, j + 1) + F(phi_in, 0, j - 1) - 4.0 * x;
                F(phi_out, 0, j) = -y + 2 * x + F(tcc, 0, j) * delta - KAPPA * x - F(tgamma, 0, j) * (x - y);
                break;
            case WG_BC_ABSORBING:
            case WG_BC_VPER_HABS:
                F(phi_out, 0, j) = x - F(tc, 0, j) * (x - F(phi_in, 1, j)) - KAPPA_SIDES * x - GAMMA_SIDES * (x - y);
                break;
            }
        }
    }

    /* right boundary (wave_billiard.c:434-467) */
    for (j = 1; j < NY - 1; j++) {
        if (TWOSPEEDS || F(xy_in, NX - 1, j) != 0) {
            x = F(phi_in, NX - 1, j);
            y = F(psi_in, NX - 1, j);
            switch (p->b_cond) {
            case WG_BC_DIRICHLET:
                delta = F(phi_in, NX - 2, j) + F(phi_in, NX - 1, j + 1) + F(phi_in, NX - 1, j - 1) - 3.0 * x;
                F(phi_out, NX - 1, j) = -y + 2 * x + F(tcc, NX - 1, j) * delta - KAPPA * x - F(tgamma, NX - 1, j) * (x - y);
                break;
            case WG_BC_PERIODIC:
                delta = F(phi_in, NX - 2, j) + F(phi_in, 0, j) + F(phi_in, NX - 1, j + 1) + F(phi_in, NX - 1, j - 1) - 4.0 * x;
                F(phi_out, NX - 1, j) = -y + 2 * x + F(tcc, NX - 1, j) * delta - KAPPA * x - F(tgamma, NX - 1, j) * (x - y);
                break;
            case WG_BC_ABSORBING:
            case WG_BC_VPER_HABS:
                F(phi_out, NX - 1, j) = x - F(tc, NX - 1, j) * (x - F(phi_in, NX - 2, j)) - KAPPA_SIDES * x - GAMMA_SIDES * (x - y);
                break;
            }
        }
    }

    /* top (j = NY-1) and bottom (j = 0) boundaries (wave_billiard.c:470-583) */
    for (int side = 0; side < 2; side++) {
        const int jb = side == 0 ? NY - 1 : 0;     /* the boundary row */
        const int jn = side == 0 ? NY - 2 : 1;     /* its inner neighbour */
        const int jw = side == 0 ? 0 : NY - 1;     /* periodic wrap partner */
        for (i = 0; i < NX; i++) {
            if (TWOSPEEDS || F(xy_in, i, jb) != 0) {
                x = F(phi_in, i, jb);
                y = F(psi_in, i, jb);
                if (p->oscillate_topbot && (i < tb_shift) && (i < NX - 1) && (i > 0)) {
                    iplus = i + 1;
                    iminus = i - 1;
                    if (iminus < 0) iminus = 0;
                    delta = F(phi_in, iplus, jb) + F(phi_in, iminus, jb) + -2.0 * x;
                    F(phi_out, i, jb) = -y + 2 * x + F(tcc, i, jb) * delta - KAPPA * x - F(tgamma, i, jb) * (x - y);
                } else switch (p->b_cond) {
                    case WG_BC_DIRICHLET:
                        iplus = i + 1; if (iplus == NX) iplus = NX - 1;
                        iminus = i - 1; if (iminus == -1) iminus = 0;
                        delta = F(phi_in, iplus, jb) + F(phi_in, iminus, jb) + F(phi_in, i, jn) - 3.0 * x;
                        F(phi_out, i, jb) = -y + 2 * x + F(tcc, i, jb) * delta - KAPPA * x - F(tgamma, i, jb) * (x - y);
                        break;
                    case WG_BC_PERIODIC:
                        iplus = (i + 1) % NX;
                        iminus = (i - 1) % NX;
                        if (iminus < 0) iminus += NX;
                        delta = F(phi_in, iplus, jb) + F(phi_in, iminus, jb) + F(phi_in, i, jn) + F(phi_in, i, jw) - 4.0 * x;
                        F(phi_out, i, jb) = -y + 2 * x + F(tcc, i, jb) * delta - KAPPA * x - F(tgamma, i, jb) * (x - y);
                        break;
                    case WG_BC_ABSORBING:
                        F(phi_out, i, jb) = x - F(tc, i, jb) * (x - F(phi_in, i, jn)) - KAPPA_TOPBOT * x - GAMMA_TOPBOT * (x - y);
                        break;
                    case WG_BC_VPER_HABS:
                        iplus = (i + 1); if (iplus == NX) iplus = NX - 1;
                        iminus = (i - 1); if (iminus == -1) iminus = 0;
                        delta = F(phi_in, iplus, jb) + F(phi_in, iminus, jb) + F(phi_in, i, jn) + F(phi_in, i, jw) - 4.0 * x;
                        if (i == 0) F(phi_out, 0, jb) = x - F(tc, 0, jb) * (x - F(phi_in, 1, jb)) - KAPPA_SIDES * x - GAMMA_SIDES * (x - y);
                        else F(phi_out, i, jb) = -y + 2 * x + F(tcc, i, jb) * delta - KAPPA * x - F(tgamma, i, jb) * (x - y);
                        break;
                    }
            }
        }
    }

    /* oscillating corners (wave_billiard.c:586-590).  The reference writes
     * phi_out[0][NX-1]; that cell exists only when NX <= NY (for NX > NY the write
     * lands outside row 0), so the write is kept exactly when it is in bounds. */
    if (p->oscillate_left && !BEAM_BC(p)) {
        F(phi_out, 0, 0) = wo_oscillating_bc(p, (int)time, 0);
        if (NX <= NY) F(phi_out, 0, NX - 1) = wo_oscillating_bc(p, (int)time, NX - 1);
    }

    /* FLOOR clamp (wave_billiard.c:593-609) */
    if (p->floor_clamp)
        for (i = 0; i < NX; i++)
            for (j = 0; j < NY; j++)
                if (F(xy_in, i, j) != 0) {
                    if (F(phi_out, i, j) > p->vmax) F(phi_out, i, j) = p->vmax;
                    else if (F(phi_out, i, j) < -p->vmax) F(phi_out, i, j) = -p->vmax;
                }

    wo_point_source(p, time, phi_out);
#undef LEFT_BC
}

int wo_run(const wg_params *p, long *time, int nsteps, double *bufs[3],
           const int16_t *xy_in, const double *tcc, const double *tc, const double *tgamma,
           const wg_neumann_bc *nbc, int n_nbc, int *prev)
{
    int cur = 0, prv = 1, fre = 2;
    for (int s = 0; s < nsteps; s++) {
        (*time)++;
        wo_evolve_wave_half(p, *time, bufs[cur], bufs[prv], bufs[fre], xy_in, tcc, tc, tgamma, nbc, n_nbc);
        int nc = fre, np = cur, nf = prv;
        cur = nc; prv = np; fre = nf;
    }
    if (prev) *prev = prv;
    return cur;
}

/* wave_energy.c:662-913: stepper on the half domain j < NY/2. */
void wo_evolve_wave_half_energy(const wg_params *p, long time,
                                const double *phi_in, const double *psi_in, double *phi_out,
                                const int16_t *xy_in)
{
    const int NX = p->nx, NY = p->ny, TWOSPEEDS = p->twospeeds, jmid = NY / 2;
    const double KAPPA = p->kappa, KAPPA_SIDES = p->kappa_sides, KAPPA_TOPBOT = p->kappa_topbot;
    const double GAMMA_SIDES = p->gamma_sides, GAMMA_TOPBOT = p->gamma_topbot;
    const double courant2 = p->courant * p->courant, courantb2 = p->courantb * p->courantb;
    int i, j, iplus, iminus;
    double delta, x, y;

    /* the static tables of wave_energy.c:670-697, zero where neither branch applies */
#define TC(i, j)  (F(xy_in, i, j) ? p->courant : (TWOSPEEDS ? p->courantb : 0.0))
#define TCC(i, j) (F(xy_in, i, j) ? courant2 : (TWOSPEEDS ? courantb2 : 0.0))
#define TG(i, j)  (F(xy_in, i, j) ? p->gamma : (TWOSPEEDS ? p->gammab : 0.0))

    for (i = 1; i < NX - 1; i++)
        for (j = 1; j < jmid - 1; j++)
            if (TWOSPEEDS || F(xy_in, i, j) != 0) {
                x = F(phi_in, i, j);
                y = F(psi_in, i, j);
                delta = F(phi_in, i + 1, j) + F(phi_in, i - 1, j) + F(phi_in, i, j + 1) + F(phi_in, i, j - 1) - 4.0 * x;
                F(phi_out, i, j) = -y + 2 * x + TCC(i, j) * delta - KAPPA * x - TG(i, j) * (x - y);
            }

    if (p->oscillate_left) {
        for (j = 1; j < jmid; j++) F(phi_out, 0, j) = wo_oscillating_bc(p, (int)time, j);
    } else {
        for (j = 1; j < jmid - 1; j++) {
            if (TWOSPEEDS || F(xy_in, 0, j) != 0) {
                x = F(phi_in, 0, j);
                y = F(psi_in, 0, j);
                switch (p->b_cond) {
                case WG_BC_DIRICHLET:
                    delta = F(phi_in, 1, j) + F(phi_in, 0, j + 1) + F(phi_in, 0, j - 1) - 3.0 * x;
                    F(phi_out, 0, j) = -y + 2 * x + TCC(0, j) * delta - KAPPA * x - TG(0, j) * (x - y);
                    break;
                case WG_BC_PERIODIC:
                    delta = F(phi_in, 1, j) + F(phi_in, NX - 1, j) + F(phi_in, 0, j + 1) + F(phi_in, 0, j - 1) - 4.0 * x;
                    F(phi_out, 0, j) = -y + 2 * x + TCC(0, j) * delta - KAPPA * x - TG(0, j) * (x - y);
                    break;
                case WG_BC_ABSORBING:
                case WG_BC_VPER_HABS:
                    F(phi_out, 0, j) = x - TC(0, j) * (x - F(phi_in, 1, j)) - KAPPA_SIDES * x - GAMMA_SIDES * (x - y);
                    break;
                }
            }
        }
    }

    for (j = 1; j < jmid - 1; j++) {
        if (TWOSPEEDS || F(xy_in, NX - 1, j) != 0) {
            x = F(phi_in, NX - 1, j);
            y = F(psi_in, NX - 1, j);
            switch (p->b_cond) {
            case WG_BC_DIRICHLET:
                delta = F(phi_in, NX - 2, j) + F(phi_in, NX - 1, j + 1) + F(phi_in, NX - 1, j - 1) - 3.0 * x;
                F(phi_out, NX - 1, j) = -y + 2 * x + TCC(NX - 1, j) * delta - KAPPA * x - TG(NX - 1, j) * (x - y);
                break;
            case WG_BC_PERIODIC:
                delta = F(phi_in, NX - 2, j) + F(phi_in, 0, j) + F(phi_in, NX - 1, j + 1) + F(phi_in, NX - 1, j - 1) - 4.0 * x;
                F(phi_out, NX - 1, j) = -y + 2 * x + TCC(NX - 1, j) * delta - KAPPA * x - TG(NX - 1, j) * (x - y);
                break;
            case WG_BC_ABSORBING:
            case WG_BC_VPER_HABS:
                F(phi_out, NX - 1, j) = x - TC(NX - 1, j) * (x - F(phi_in, NX - 2, j)) - KAPPA_SIDES * x - GAMMA_SIDES * (x - y);
                break;
            }
        }
    }

    /* top (row jmid-1; the OSCILLATE_TOPBOT branch reads outside the static tables
     * and is not restated) and bottom (row 0) */
    for (int side = 0; side < 2; side++) {
        const int jb = side == 0 ? jmid - 1 : 0;
        const int jn = side == 0 ? jmid - 2 : 1;
        const int jw = side == 0 ? 0 : jmid - 1;
        for (i = 0; i < NX; i++) {
            if (TWOSPEEDS || F(xy_in, i, jb) != 0) {
                x = F(phi_in, i, jb);
                y = F(psi_in, i, jb);
                switch (p->b_cond) {
                case WG_BC_DIRICHLET:
                    iplus = i + 1; if (iplus == NX) iplus = NX - 1;
                    iminus = i - 1; if (iminus == -1) iminus = 0;
                    delta = F(phi_in, iplus, jb) + F(phi_in, iminus, jb) + F(phi_in, i, jn) - 3.0 * x;
                    F(phi_out, i, jb) = -y + 2 * x + TCC(i, jb) * delta - KAPPA * x - TG(i, jb) * (x - y);
                    break;
                case WG_BC_PERIODIC:
                    iplus = (i + 1) % NX;
                    iminus = (i - 1) % NX; if (iminus < 0) iminus += NX;
                    delta = F(phi_in, iplus, jb) + F(phi_in, iminus, jb) + F(phi_in, i, jn) + F(phi_in, i, jw) - 4.0 * x;
                    F(phi_out, i, jb) = -y + 2 * x + TCC(i, jb) * delta - KAPPA * x - TG(i, jb) * (x - y);
                    break;
                case WG_BC_ABSORBING:
                    F(phi_out, i, jb) = x - TC(i, jb) * (x - F(phi_in, i, jn)) - KAPPA_TOPBOT * x - GAMMA_TOPBOT * (x - y);
                    break;
                case WG_BC_VPER_HABS:
                    iplus = (i + 1); if (iplus == NX) iplus = NX - 1;
                    iminus = (i - 1); if (iminus == -1) iminus = 0;
                    delta = F(phi_in, iplus, jb) + F(phi_in, iminus, jb) + F(phi_in, i, jn) + F(phi_in, i, jw) - 4.0 * x;
                    if (i == 0) F(phi_out, 0, jb) = x - TC(0, jb) * (x - F(phi_in, 1, jb)) - KAPPA_SIDES * x - GAMMA_SIDES * (x - y);
                    else F(phi_out, i, jb) = -y + 2 * x + TCC(i, jb) * delta - KAPPA * x - TG(i, jb) * (x - y);
                    break;
                }
            }
        }
    }
    /* wave_energy.c:898-902 tests i == 0 after the loops (i == NX): never taken. */

    if (p->floor_clamp)
        for (i = 0; i < NX; i++)
            for (j = 0; j < jmid; j++)
                if (F(xy_in, i, j) != 0) {
                    if (F(phi_out, i, j) > p->vmax) F(phi_out, i, j) = p->vmax;
                    if (F(phi_out, i, j) < -p->vmax) F(phi_out, i, j) = -p->vmax;
                }
#undef TC
#undef TCC
#undef TG
}

/* compute_energy (wave_common.c:453-472). */
double wo_compute_energy(const wg_params *p, const double *phi, const double *psi,
                         const int16_t *xy_in, int i, int j)
{
    const int NX = p->nx, NY = p->ny;
    double velocity, gx2, gy2;
    int iplus, iminus, jplus, jminus;

    velocity = (F(phi, i, j) - F(psi, i, j));
    iplus = (i + 1); if (iplus == NX) iplus = NX - 1;
    iminus = (i - 1); if (iminus == -1) iminus = 0;
    jplus = (j + 1); if (jplus == NY) jplus = NY - 1;
    jminus = (j - 1); if (jminus == -1) jminus = 0;

    gx2 = (F(phi, iplus, j) - F(phi, i, j)) * (F(phi, iplus, j) - F(phi, i, j))
        + (F(phi, i, j) - F(phi, iminus, j)) * (F(phi, i, j) - F(phi, iminus, j));
    gy2 = (F(phi, i, jplus) - F(phi, i, j)) * (F(phi, i, jplus) - F(phi, i, j))
        + (F(phi, i, j) - F(phi, i, jminus)) * (F(phi, i, j) - F(phi, i, jminus));
    if (F(xy_in, i, j))
        return p->e_scale * p->e_scale * (velocity * velocity + 0.5 * p->courant * p->courant * (gx2 + gy2));
    else if (p->twospeeds)
        return p->e_scale * p->e_scale * (velocity * velocity + 0.5 * p->courantb * p->courantb * (gx2 + gy2));
    return 0.0;
}

/* compute_energy_x for all columns (wave_energy.c:292-302, :424). */
void wo_energy_x(const wg_params *p, const double *phi, const double *psi,
                 const int16_t *xy_in, double *out)
{
    for (int i = 0; i < p->nx; i++) {
        double energy = 0.0;
        for (int j = 0; j < p->ny / 2; j++) energy += wo_compute_energy(p, phi, psi, xy_in, i, j);
        out[i] = energy;
    }
}

/* compute_energy_tblr box sums (sub_wave_comp.c:1816-1854), FLOOR rescaling off. */
void wo_energy_tblr(const wg_params *p, const double *phi, const double *psi,
                    const int16_t *xy_in, int ileft, int iright, double out[6])
{
    const int NX = p->nx, NY = p->ny, jmid = NY / 2;
    const int ilo[3] = {0, ileft, iright}, ihi[3] = {ileft, iright, NX};
    for (int b = 0; b < 6; b++) {
        const int col = b % 3, top = b < 3;
        const int jlo = top ? jmid : 0, jhi = top ? NY : jmid;
        double energy = 0.0;
        for (int i = ilo[col]; i < ihi[col]; i++)
            for (int j = jlo; j < jhi; j++) energy += wo_compute_energy(p, phi, psi, xy_in, i, j);
        out[b] = energy;
    }
}

double wo_energy_total_naive(const wg_params *p, const double *phi, const double *psi,
                             const int16_t *xy_in)
{
    double e = 0.0;
    for (int i = 0; i < p->nx; i++)
        for (int j = 0; j < p->ny; j++) e += wo_compute_energy(p, phi, psi, xy_in, i, j);
    return e;
}

double wo_energy_total_comp(const wg_params *p, const double *phi, const double *psi,
                            const int16_t *xy_in)
{
    double s = 0.0, c = 0.0;
    for (int i = 0; i < p->nx; i++)
        for (int j = 0; j < p->ny; j++) {
            double v = wo_compute_energy(p, phi, psi, xy_in, i, j);
            double t = s + v;
            if (fabs(s) >= fabs(v)) c += (s - t) + v;
            else c += (v - t) + s;
            s = t;
        }
    return s + c;
}

/* xy_in_billiard_single_domain, the shapes used by the workloads (sub_wave.c:5712-6252). */
static int wo_in_domain(const wg_params *p, double x, double y, int domain, double lambda,
                        int npoly, double apoly, const wo_circle *circles, int ncircles)
{
    int k, condition;
    double omega, c, angle;
    switch (domain) {
    case WO_D_RECTANGLE:
        return (fabs(x) < lambda) && (fabs(y) < 1.0);
    case WO_D_ELLIPSE:
        return x * x / (lambda * lambda) + y * y < 1.0;
    case WO_D_STADIUM:
        if ((x > -0.5 * lambda) && (x < 0.5 * lambda) && (y > -1.0) && (y < 1.0)) return 1;
        if (sqrt((x + 0.5 * lambda) * (x + 0.5 * lambda) + y * y) < 1.0) return 1;
        if (sqrt((x - 0.5 * lambda) * (x - 0.5 * lambda) + y * y) < 1.0) return 1;
        return 0;
    case WO_D_POLYGON:
        condition = 1;
        omega = R_DPI / ((double)npoly);
        c = lambda * cos(omega * 0.5);
        for (k = 0; k < npoly; k++) {
            angle = apoly * R_PID + (k + 0.5) * omega;
            condition = condition * (x * cos(angle) + y * sin(angle) < c);
        }
        return condition;
    case WO_D_CIRCLES:
    case WO_D_CIRCLES_IN_RECT:
        for (k = 0; k < ncircles; k++)
            if (circles[k].active) {
                double x1 = circles[k].xc, y1 = circles[k].yc, r2 = circles[k].radius * circles[k].radius;
                if ((x - x1) * (x - x1) + (y - y1) * (y - y1) < r2) return 0;
            }
        if (domain == WO_D_CIRCLES) return 1;
        if ((fabs(x) >= lambda) || (fabs(y) >= p->ymax - p->xmax + lambda)) return 0;
        return 1;
    default:
        return 1;
    }
}

void wo_mask(const wg_params *p, int domain, double lambda, int npoly, double apoly,
             const wo_circle *circles, int ncircles, int16_t *xy_out)
{
    const int NY = p->ny;
    double xy[2];
    for (int i = 0; i < p->nx; i++)
        for (int j = 0; j < NY; j++) {
            wo_ij_to_xy(p, i, j, xy);
            F(xy_out, i, j) = (int16_t)wo_in_domain(p, xy[0], xy[1], domain, lambda, npoly, apoly, circles, ncircles);
        }
}

/* init_ior_2d, VARIABLE_IOR == 0 branch (sub_wave.c:12983-13002). */
void wo_init_ior(const wg_params *p, const int16_t *xy_in, double *tcc, double *tc, double *tgamma)
{
    const int NY = p->ny;
    const double courant2 = p->courant * p->courant, courantb2 = p->courantb * p->courantb;
    for (int i = 0; i < p->nx; i++)
        for (int j = 0; j < NY; j++) {
            if (F(xy_in, i, j) != 0) {
                F(tc, i, j) = p->courant;
                F(tcc, i, j) = courant2;
                if (F(xy_in, i, j) == 1) F(tgamma, i, j) = p->gamma;
                else F(tgamma, i, j) = p->gammab;
            } else if (p->twospeeds) {
                F(tc, i, j) = p->courantb;
                F(tcc, i, j) = courantb2;
                F(tgamma, i, j) = p->gammab;
            }
        }
}

/* argument (sub_wave.c:287-303) */
static double wo_argument(double x, double y)
{
    double alph;
    if (x != 0.0) {
        alph = atan(y / x);
        if (x < 0.0) alph += R_PI;
    } else {
        alph = R_PID;
        if (y < 0.0) alph = R_PI * 1.5;
    }
    return alph;
}

/* init_neumann_bc + compute_normal_vector + build_neumann_data
 * (sub_wave.c:13910-13947, 13384-13410, 13700-13761). */
int wo_init_neumann(const wg_params *p, int domain, double lambda, int npoly, double apoly,
                    int16_t *xy_in, wg_neumann_bc *out, int max_records)
{
    const int NX = p->nx, NY = p->ny;
    int n = 0;
    double xy[2], v1, v2, sum;
    memset(out, 0, sizeof(wg_neumann_bc) * (size_t)max_records);
    for (int i = 1; i < NX - 1; i++)
        for (int j = 1; j < NY - 1; j++)
            if (!F(xy_in, i, j)) {
                if ((F(xy_in, i - 1, j) == 1) || (F(xy_in, i + 1, j) == 1) ||
                    (F(xy_in, i, j - 1) == 1) || (F(xy_in, i, j + 1) == 1)) {
                    wo_ij_to_xy(p, i, j, xy);
                    if (domain == WO_D_ELLIPSE) {
                        v1 = 2.0 * xy[0] / (lambda * lambda);
                        v2 = 2.0 * xy[1];
                    } else { /* polygon */
                        double theta = R_DPI / (double)npoly;
                        double angle = wo_argument(xy[0], xy[1]) - R_PID * apoly + R_DPI;
                        int side = (int)(angle / theta);
                        angle = R_PID * apoly + 0.5 * theta + (double)side * theta;
                        v1 = cos(angle);
                        v2 = sin(angle);
                    }
                    out[n].signx1 = (int16_t)(v1 >= 0.0 ? -1 : 1);
                    out[n].signy1 = 0;
                    out[n].signx2 = 0;
                    out[n].signy2 = (int16_t)(v2 >= 0.0 ? -1 : 1);
                    v1 = fabs(v1);
                    v2 = fabs(v2);
                    sum = v1 + v2;
                    out[n].nx = v1 / sum;
                    out[n].ny = v2 / sum;
                    out[n].top = (int16_t)(xy[1] > 0.0);
                    F(xy_in, i, j) = -1;
                    out[n].i = i;
                    out[n].j = j;
                    n++;
                    if (n >= max_records) return -1;
                }
            }
    for (int q = 0; q < n; q++) {
        int i = out[q].i, j = out[q].j;
        double n1 = out[q].nx, n2 = out[q].ny;
        if (n1 > n2) {
            out[q].nx = (n1 - n2) / n1;
            out[q].ny = n2 / n1;
            out[q].signx2 = out[q].signx1;
        } else if (n2 > n1) {
            out[q].nx = n1 / n2;
            out[q].ny = (n2 - n1) / n2;
            out[q].signy1 = out[q].signy2;
        }
        out[q].nbi1 = i + out[q].signx1;
        out[q].nbj1 = j + out[q].signy1;
        out[q].nbi2 = i + out[q].signx2;
        out[q].nbj2 = j + out[q].signy2;
        out[q].active = 1;
    }
    /* test_neumann_data (sub_wave.c:13850-13880): a record whose neighbour is itself
     * a ghost cell is made inactive. */
    for (int q = 0; q < n; q++) {
        int i = out[q].i, j = out[q].j;
        if (F(xy_in, i + out[q].signx1, j + out[q].signy1) == -1) out[q].active = 0;
        if (F(xy_in, i + out[q].signx2, j + out[q].signy2) == -1) out[q].active = 0;
    }
    return n;
}

/* add_circular_wave (wave_common.c:337-351): adds INITIAL_AMP*factor*exp(-r^2/VARIANCE)
 * *cos(-r/WAVELENGTH) to phi on the cells with xy_in != 0 (all cells with TWOSPEEDS);
 * psi is not touched.  Same expression order as the reference. */
void wo_add_circular_wave(const wg_params *p, double init_amp, double factor, double x, double y,
                          double variance, double wavelength, double *phi, const int16_t *xy_in)
{
    for (int i = 0; i < p->nx; i++)
        for (int j = 0; j < p->ny; j++) {
            double xy[2], dist2;
            wo_ij_to_xy(p, i, j, xy);
            dist2 = (xy[0] - x) * (xy[0] - x) + (xy[1] - y) * (xy[1] - y);
            const size_t c = (size_t)i * p->ny + j;
            if ((xy_in[c]) || (p->twospeeds))
                phi[c] += init_amp * factor * exp(-dist2 / variance) * cos(-sqrt(dist2) / wavelength);
        }
}

/* Per sampled cell (i = col*size, j = row*size; arrays [row][col]) of
 * draw_wave_highres_palette (wave_common.c:1750-1848): compute_energy
 * (wave_common.c:453-472), and the velocity |phi - psi| and gradients of
 * compute_energy_flux (wave_common.c:475-511). */
void wo_frame_cells(const wg_params *p, const double *phi, const double *psi, const int16_t *xy_in, int size,
                    double *energy, double *vel, double *gx, double *gy)
{
    const int NX = p->nx, NY = p->ny, w = NX / size, h = NY / size;
    for (int row = 0; row < h; row++)
        for (int col = 0; col < w; col++) {
            const int i = col * size, j = row * size;
            const size_t k = (size_t)row * w + col;
            int iplus = i + 1, iminus = i - 1, jplus = j + 1, jminus = j - 1;
            if (iplus == NX) iplus = NX - 1;
            if (iminus == -1) iminus = 0;
            if (jplus == NY) jplus = NY - 1;
            if (jminus == -1) jminus = 0;
            energy[k] = wo_compute_energy(p, phi, psi, xy_in, i, j);
            vel[k] = fabs(phi[(size_t)i * NY + j] - psi[(size_t)i * NY + j]);
            gx[k] = phi[(size_t)iplus * NY + j] - phi[(size_t)iminus * NY + j];
            gy[k] = phi[(size_t)i * NY + jplus] - phi[(size_t)i * NY + jminus];
        }
}
