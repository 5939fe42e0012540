// wg_device.cuh — device-side parameters and the per-cell rules of the reference's
// stepper (wave_billiard.c:302-610), shared by every stepping kernel.
//
// Arithmetic of the FP64 forms uses __dadd_rn/__dsub_rn/__dmul_rn so that the compiler
// contracts nothing into an FMA and every operation happens in the reference's order:
// the device result is then bit-identical to the CPU reference built without FMA.  The
// only fused operations are the explicit P2_ / L4_ below, whose products are exact.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace wg {

// Scene parameters as the kernels see them (host-precomputed integers included).
struct DevParams {
    int nx, ny;          // grid
    int pitch;           // elements per row in device memory (multiple of 32)
    int wpitch;          // 32-bit mask words per row (pitch / 32)
    int b_cond, twospeeds, osc_left, osc_topbot, sched, floor_clamp, beam;
    int bc_jmin, bc_jmax;          // OSCILLATE_LEFT beam range (wave_billiard.c:320-339)
    int osc_beam_jmax;             // xy_to_ij(0, OSCIL_YMAX)[1] (sub_wave.c:12032)
    int osc_sine_jmax, osc_sine_jmin;  // xy_to_ij(0, OSCIL_YMID +- OSCIL_YMAX)[1]
    int src_on, src_i, src_j;
    int corner2_on;                // the reference's phi_out[0][NX-1] write is in bounds
    // OSCILLATE_TOPBOT: rows i < tb_ilim take the top/bottom oscillation rule (the
    // reference's i < tb_shift, with tb_shift an integer value: an integer comparison, no
    // FP64 conversion on the device)
    int tb_ilim, pad0_;
    double kappa, kappa_sides, kappa_topbot, gamma_sides, gamma_topbot, vmax;
    double c2, c2b, gam, gamb, courant, courantb;   // WG_COEF_MASK coefficients
    double omega, omega_b, amplitude, damping, achirp, yshift, ivar, ishift, wpshift;
    double ymin, ymax;
    double src_amp, src_period;
    double e_scale2, ehalf_c2, ehalf_c2b;  // E_SCALE^2, (0.5*COURANT)*COURANT, (0.5*COURANTB)*COURANTB
};

// ---------------------------------------------------------------------------
// Exactly rounded double operations (never contracted by the compiler).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double A_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double S_(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double M_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double D_(double a, double b) { return __ddiv_rn(a, b); }

// Products by 2 and 4 are exact (a change of exponent) while |x| < DBL_MAX / 4, so one
// fused multiply-add rounds the same exact sum as the separate multiply and add, and
// IEEE 754 gives an exactly zero result the same sign both ways:
//   P2_(x, y)  == A_(-y, M_(2.0, x))       (-y + 2*x)
//   L4_(d, x)  == S_(d, M_(4.0, x))        (d - 4.0*x)
// One FP64 operation instead of two, bit for bit on every field short of overflow.
__device__ __forceinline__ double P2_(double x, double y) { return __fma_rn(2.0, x, -y); }
__device__ __forceinline__ double L4_(double d, double x) { return __fma_rn(-4.0, x, d); }

// -y + 2*x + cc*delta - KAPPA*x - g*(x-y)   (wave_billiard.c:373)
// Z bit 0 (Z_KAPPA): KAPPA = 0.  Bit 1 (Z_GAMMA): g = 0 on every cell.  A zero
// coefficient makes its product a zero, and subtracting a zero changes at most the sign
// of a zero result, never a value; such a term is then left out.
constexpr int Z_KAPPA = 1, Z_GAMMA = 2;
template <int Z = 0>
__device__ __forceinline__ double upd64(double x, double y, double cc, double delta, double kappa, double g)
{
    double r = P2_(x, y);
    r = A_(r, M_(cc, delta));
    if (!(Z & Z_KAPPA)) r = S_(r, M_(kappa, x));
    if (!(Z & Z_GAMMA)) r = S_(r, M_(g, S_(x, y)));
    return r;
}

// x - tc*(x - nb) - K*x - G*(x-y)   (wave_billiard.c:418)
__device__ __forceinline__ double absorb64(double x, double y, double tc, double nb, double k, double g)
{
    double r = S_(x, M_(tc, S_(x, nb)));
    r = S_(r, M_(k, x));
    return S_(r, M_(g, S_(x, y)));
}

// FP32 state: phi and the velocity v = phi(t) - phi(t-1), each stored in FP32 (psi is
// phi - v; conversions in and out are done in FP64).  v kept as its own array carries
// the increment each update applied, to FP32 precision of v itself; recovered from two
// stored levels it would carry the rounding of phi, magnified by |phi|/|v| (16-80 times
// less accurate energies in measurements, more so for small COURANT numbers).  A rule
// returns the cell's new (phi, v).
struct XV {
    float x, v;
};

// Bulk update in increment form: v' = (1-g) v - kappa x + cc delta, x' = x + v', with the
// Laplacian as differences from the centre.  Same mathematics as upd64.  Every rounding
// is spelled out as an operation or a fused multiply-add (nothing left for the compiler
// to contract), so every kernel that applies it rounds each cell the same way.
__device__ __forceinline__ float vel32(float x, float v, float cc, float delta, float kappa, float g)
{
    return fmaf(cc, delta, fmaf(-kappa, x, fmaf(-g, v, v)));
}
__device__ __forceinline__ XV upd32(float x, float v, float cc, float delta, float kappa, float g)
{
    const float vn = vel32(x, v, cc, delta, kappa, g);
    return XV{__fadd_rn(x, vn), vn};
}
// upd32 with KAPPA = 0: the kappa*x term is then an exact zero, so leaving it out changes
// at most the sign of a zero result, never a value.
__device__ __forceinline__ XV upd32_k0(float x, float v, float cc, float delta, float g)
{
    const float vn = fmaf(cc, delta, fmaf(-g, v, v));
    return XV{__fadd_rn(x, vn), vn};
}
// Absorbing edge: x' = x - (tc (x - nb) + k x + g v).
__device__ __forceinline__ XV absorb32(float x, float v, float tc, float nb, float k, float g)
{
    const float t = fmaf(k, x, __fmul_rn(tc, __fsub_rn(x, nb)));
    const float vn = -fmaf(g, v, t);
    return XV{__fadd_rn(x, vn), vn};
}
// A value a rule sets (oscillating edge, FLOOR): the velocity is the change it makes.
__device__ __forceinline__ XV set32(float x, float xn) { return XV{xn, __fsub_rn(xn, x)}; }
// A cell the reference does not write: the in-place two-level form swaps phi and psi
// there, so phi' = psi = x - v and v' = -v.
__device__ __forceinline__ XV keep32(float x, float v) { return XV{__fsub_rn(x, v), -v}; }
// upd32 or keep32 by a flag, as one addition: x - v == x + (-v) exactly (signs of zero
// included), so the unwritten cell's rule is the update's x + v' with v' = -v.
__device__ __forceinline__ XV updkeep32(bool upd, float x, float v, float cc, float delta, float kappa, float g)
{
    const float vn = upd ? vel32(x, v, cc, delta, kappa, g) : -v;
    return XV{__fadd_rn(x, vn), vn};
}
// FLOOR: phi clamped to [-vmax, vmax] by the reference's two comparisons (a NaN passes,
// as there); an unchanged value keeps its velocity.
__device__ __forceinline__ XV clamp32(float x, XV r, float vmax)
{
    if (r.x > vmax) return set32(x, vmax);
    if (r.x < -vmax) return set32(x, -vmax);
    return r;
}
// The point source: its FP64 increment added to the new value and to the velocity (psi
// is not touched), each rounded once.
__device__ __forceinline__ XV source32(XV r, double add)
{
    return XV{(float)A_((double)r.x, add), (float)A_((double)r.v, add)};
}

// oscillating_bc (sub_wave.c:11965-12162) with the reference's constants.
__device__ inline double osc_bc(const DevParams &p, int time, int j)
{
    const double PID = 1.570796327, DPI = 6.283185307;
    const int NY = p.ny;
    const double YSH = p.yshift, OM = p.omega, AMP = p.amplitude, DAMP = p.damping;
    double t, t1, phase, a, env, amp, dist2;
    const double tOM = M_((double)time, OM);
    switch (p.sched) {
    case 0:  // OSC_PERIODIC
        if (YSH > 0.0) t = S_(tOM, D_(M_((double)j, YSH), (double)NY));
        else t = A_(tOM, D_(M_((double)(NY - j), YSH), (double)NY));
        if (t < 0.0) return 0.0;
        return M_(M_(AMP, cos(t)), exp(M_(-t, DAMP)));
    case 1:  // OSC_SLOWING
        a = 0.0025;
        t = tOM;
        if (YSH > 0.0) t = S_(t, D_(M_((double)j, YSH), (double)NY));
        phase = S_(t, M_(M_(a, t), t));
        return M_(M_(AMP, cos(phase)), exp(M_(-phase, DAMP)));
    case 2:   // OSC_WAVE_PACKET
    case 21:  // OSC_WAVE_PACKETS
        t = tOM;
        if (YSH > 0.0) t = S_(t, D_(M_((double)j, YSH), (double)NY));
        t1 = t;
        if (p.sched == 21) t1 = S_(t, M_((double)((int)A_(D_(t, p.wpshift), 0.5)), p.wpshift));
        a = D_(sqrt(p.ivar), OM);
        phase = M_(AMP, cos(t));
        env = M_(exp(D_(M_(-S_(t1, p.ishift), S_(t1, p.ishift)), M_(a, a))), sqrt(D_(DPI, a)));
        return M_(phase, env);
    case 3:  // OSC_CHIRP
        t = tOM;
        if (YSH > 0.0) t = S_(t, D_(M_((double)j, YSH), (double)NY));
        phase = A_(t, M_(M_(p.achirp, t), t));
        return M_(M_(AMP, sin(phase)), exp(M_(-phase, DAMP)));
    case 4:   // OSC_BEAM
    case 5: { // OSC_BEAM_TWOPERIODS
        int jmax = p.osc_beam_jmax, jmin = NY - jmax;
        double h = S_(p.ymax, p.ymin);
        if (j < jmin) dist2 = D_(M_((double)(jmin - 1 - j), h), (double)NY);
        else if (j > jmax) dist2 = D_(M_((double)(j - jmax), h), (double)NY);
        else dist2 = 0.0;
        dist2 = M_(M_(500.0, dist2), dist2);
        t = tOM;
        if (YSH > 0.0) t = S_(t, D_(M_((double)j, YSH), (double)NY));
        if (p.sched == 4) amp = M_(M_(AMP, cos(t)), exp(M_(-t, DAMP)));
        else amp = M_(M_(AMP, A_(M_(0.5, cos(t)), M_(0.5, cos(M_(sqrt(7.0), t))))), exp(M_(-t, DAMP)));
        return M_(amp, exp(D_(-dist2, p.ivar)));
    }
    case 41: {  // OSC_BEAM_GAUSSIAN
        dist2 = D_(M_((double)(j - NY / 2), S_(p.ymax, p.ymin)), (double)NY);
        dist2 = M_(dist2, dist2);
        t = tOM;
        if (YSH > 0.0) t = S_(t, D_(M_((double)j, YSH), (double)NY));
        amp = M_(M_(AMP, cos(t)), exp(M_(-t, DAMP)));
        return M_(amp, exp(D_(-dist2, p.ivar)));
    }
    case 42: case 43: case 44: case 51: {  // beam modulated by a sine in y
        int jmax = p.osc_sine_jmax, jmin = p.osc_sine_jmin, jmid = (jmin + jmax) / 2;
        dist2 = D_((double)(j - jmid), (double)(jmax - jmid));
        if (j > jmax) return 0.0;
        if (j < jmin) return 0.0;
        t = tOM;
        if (YSH > 0.0) t = S_(t, D_(M_((double)j, YSH), (double)NY));
        if (p.sched == 42) {
            amp = M_(M_(AMP, cos(t)), exp(M_(-t, DAMP)));
        } else if (p.sched == 43) {
            a = D_(p.ivar, M_(OM, OM));
            amp = M_(M_(AMP, cos(t)), exp(D_(M_(-S_(t, p.ishift), S_(t, p.ishift)), a)));
        } else if (p.sched == 51) {
            amp = M_(M_(AMP, A_(M_(0.5, cos(t)), M_(0.5, cos(M_(sqrt(7.0), t))))), exp(M_(-t, DAMP)));
        } else {
            phase = A_(t, M_(M_(p.achirp, t), t));
            amp = M_(M_(AMP, sin(phase)), exp(M_(-phase, DAMP)));
        }
        return M_(amp, cos(M_(PID, dist2)));
    }
    case 6:
    case 61:
        t = A_(tOM, D_(M_((double)(NY - j), YSH), (double)NY));
        t1 = A_(tOM, D_(M_((double)j, YSH), (double)NY));
        if (p.sched == 6) amp = (j < NY / 2) ? cos(t) : cos(t1);
        else {
            amp = 0.0;
            if (t > 0.0) amp = A_(amp, cos(t));
            if (t1 > 0.0) amp = A_(amp, cos(t1));
        }
        return M_(AMP, amp);
    case 7:
        if (j > NY / 2) t = A_(tOM, D_(M_((double)(NY - j), YSH), (double)NY));
        else t = A_(M_((double)time, p.omega_b), D_(M_((double)(NY - j), YSH), (double)NY));
        return M_(M_(AMP, cos(t)), exp(M_(-t, DAMP)));
    default:
        return 0.0;
    }
}

__device__ __forceinline__ double point_source(const DevParams &p, long long t)
{
    return M_(p.src_amp, sin(D_(M_(6.283185307179586, (double)t), p.src_period)));
}

__device__ __forceinline__ bool left_bc(const DevParams &p, int j)
{
    return p.osc_left && j < p.ny - 1 && j > p.bc_jmin && j < p.bc_jmax;
}

// FP32 boundary-line cell (rows 0 and nx-1, columns 0 and ny-1) for mirror ("Dirichlet"),
// periodic and absorbing boundaries: edge_cell's rules (below) in the FP32 increment form
// of upd32 / absorb32, the neighbours the reference mirrors replaced by the cell itself.
// x, v: phi and velocity of the cell; n, sv, e, w: phi at i+1, i-1, j+1, j-1 (wrapped
// around the grid for periodic scenes; any value where outside the grid otherwise); ccv,
// tcv, g: the cell's tcc, tc and tgamma; osc(): the oscillating value.  keep32 where the
// reference writes nothing.  CLAMP: FLOOR on written cells with act.  Every FP32 stepper
// (single updates, tiles, skewed passes) uses this rule.
struct Edge32K {
    float kappa, ks, kt, gs, gt, vmax;
};
template <bool CLAMP, class OscF>
__device__ __forceinline__ XV edge32(const DevParams &p, int gi, int gj, float x, float v, float n, float sv, float e,
                                     float w, float ccv, float tcv, float g, bool act, const Edge32K &k, const OscF &osc)
{
    const int NX = p.nx, NY = p.ny;
    const bool bi0 = gi == 0, bi1 = gi == NX - 1, bj0 = gj == 0, bj1 = gj == NY - 1;
    int mode = 0;  // 0 leapfrog with mirrored neighbours, 1 absorbing, 2 oscillating value
    float nb = 0.f, kk = 0.f, gg = 0.f;
    if (bj0 || bj1) {
        if (p.osc_topbot && gi > 0 && gi < NX - 1 && gi < p.tb_ilim) {
            e = x;
            w = x;
        } else if (p.b_cond == WG_BC_DIRICHLET) {
            if (bi1) n = x;
            if (bi0) sv = x;
            if (bj1) e = x; else w = x;
        } else if (p.b_cond == WG_BC_PERIODIC) {
            // the 5-point rule with the wrapped neighbours as given
        } else {
            mode = 1;
            nb = bj1 ? w : e;
            kk = k.kt;
            gg = k.gt;
        }
    } else if (bi0 || bi1) {
        if (bi0 && left_bc(p, gj)) {
            mode = 2;
        } else if (p.b_cond == WG_BC_DIRICHLET) {
            if (bi0) sv = x; else n = x;
        } else if (p.b_cond == WG_BC_PERIODIC) {
            // the 5-point rule with the wrapped neighbours as given
        } else {
            mode = 1;
            nb = bi0 ? n : sv;
            kk = k.ks;
            gg = k.gs;
        }
    }
    if (p.osc_left && !p.beam && bi0 && (bj0 || (p.corner2_on && gj == NX - 1))) mode = 2;
    XV r = keep32(x, v);
    if (mode == 2 || p.twospeeds || act) {
        if (mode == 0) r = upd32(x, v, ccv, ((n - x) + (sv - x)) + ((e - x) + (w - x)), k.kappa, g);
        else if (mode == 1) r = absorb32(x, v, tcv, nb, kk, gg);
        else r = set32(x, osc());
        if (CLAMP && p.floor_clamp && act) r = clamp32(x, r, k.vmax);
    }
    return r;
}

// Any boundary-line cell of the reference (left/right columns, top/bottom rows),
// computed with the reference's rules.  Returns true when the reference writes the
// cell; *out then holds the value (corner oscillation included, FLOOR not).
// Accessors: PHI(i,j), PSI(i,j) field reads; ACT(i,j) -> "xy != 0"; TCC/TC/TG tables.
template <class T, class Phi, class Psi, class Act, class Coef>
__device__ inline bool edge_cell(const DevParams &p, long long time, int i, int j,
                                 const Phi &PHI, const Psi &PSI, const Act &ACT, const Coef &CF,
                                 double *out)
{
    const int NX = p.nx, NY = p.ny;
    bool written = false;
    double v = 0.0;
    if (j == NY - 1 || j == 0) {
        const int jb = j, jn = (j == NY - 1) ? NY - 2 : 1, jw = (j == NY - 1) ? 0 : NY - 1;
        if (p.twospeeds || ACT(i, jb)) {
            double x = (double)PHI(i, jb), y = (double)PSI(i, jb);
            if (p.osc_topbot && i < p.tb_ilim && (i < NX - 1) && (i > 0)) {
                double delta = A_(A_((double)PHI(i + 1, jb), (double)PHI(i - 1, jb)), -M_(2.0, x));
                v = upd64(x, y, CF.tcc(i, jb), delta, p.kappa, CF.tg(i, jb));
            } else {
                int ip, im;
                double delta;
                switch (p.b_cond) {
                case 0:
                    ip = i + 1; if (ip == NX) ip = NX - 1;
                    im = i - 1; if (im == -1) im = 0;
                    delta = S_(A_(A_((double)PHI(ip, jb), (double)PHI(im, jb)), (double)PHI(i, jn)), M_(3.0, x));
                    v = upd64(x, y, CF.tcc(i, jb), delta, p.kappa, CF.tg(i, jb));
                    break;
                case 1:
                    ip = (i + 1) % NX; im = (i - 1) % NX; if (im < 0) im += NX;
                    delta = S_(A_(A_(A_((double)PHI(ip, jb), (double)PHI(im, jb)), (double)PHI(i, jn)), (double)PHI(i, jw)), M_(4.0, x));
                    v = upd64(x, y, CF.tcc(i, jb), delta, p.kappa, CF.tg(i, jb));
                    break;
                case 2:
                    v = absorb64(x, y, CF.tc(i, jb), (double)PHI(i, jn), p.kappa_topbot, p.gamma_topbot);
                    break;
                default:
                    ip = i + 1; if (ip == NX) ip = NX - 1;
                    im = i - 1; if (im == -1) im = 0;
                    if (i == 0) v = absorb64(x, y, CF.tc(0, jb), (double)PHI(1, jb), p.kappa_sides, p.gamma_sides);
                    else {
                        delta = S_(A_(A_(A_((double)PHI(ip, jb), (double)PHI(im, jb)), (double)PHI(i, jn)), (double)PHI(i, jw)), M_(4.0, x));
                        v = upd64(x, y, CF.tcc(i, jb), delta, p.kappa, CF.tg(i, jb));
                    }
                    break;
                }
            }
            written = true;
        }
    } else if (i == 0 || i == NX - 1) {
        const bool left = (i == 0);
        if (left && left_bc(p, j)) {
            v = osc_bc(p, (int)time, j);
            written = true;
        } else if (p.twospeeds || ACT(i, j)) {
            const int in = left ? 1 : NX - 2, iw = left ? NX - 1 : 0;
            double x = (double)PHI(i, j), y = (double)PSI(i, j), delta;
            switch (p.b_cond) {
            case 0:
                delta = S_(A_(A_((double)PHI(in, j), (double)PHI(i, j + 1)), (double)PHI(i, j - 1)), M_(3.0, x));
                v = upd64(x, y, CF.tcc(i, j), delta, p.kappa, CF.tg(i, j));
                break;
            case 1:
                delta = S_(A_(A_(A_((double)PHI(in, j), (double)PHI(iw, j)), (double)PHI(i, j + 1)), (double)PHI(i, j - 1)), M_(4.0, x));
                v = upd64(x, y, CF.tcc(i, j), delta, p.kappa, CF.tg(i, j));
                break;
            default:
                v = absorb64(x, y, CF.tc(i, j), (double)PHI(in, j), p.kappa_sides, p.gamma_sides);
                break;
            }
            written = true;
        }
    }
    // oscillating corners (wave_billiard.c:586-590); the second write of the
    // reference is phi_out[0][NX-1], kept only where that cell exists (NX <= NY).
    if (p.osc_left && !p.beam && i == 0) {
        if (j == 0) { v = osc_bc(p, (int)time, 0); written = true; }
        else if (p.corner2_on && j == NX - 1) { v = osc_bc(p, (int)time, NX - 1); written = true; }
    }
    *out = v;
    return written;
}

__device__ __forceinline__ double floor_clamp(const DevParams &p, double v)
{
    if (v > p.vmax) return p.vmax;
    if (v < -p.vmax) return -p.vmax;
    return v;
}

// compute_energy (wave_common.c:453-472) from double values of the five cells.
__device__ __forceinline__ double cell_energy(const DevParams &p, double x, double psi, double e, double w,
                                              double n, double s, int xy_nonzero)
{
    double v = S_(x, psi);
    double a = S_(e, x), b = S_(x, w);
    double gx2 = A_(M_(a, a), M_(b, b));
    double c = S_(n, x), d = S_(x, s);
    double gy2 = A_(M_(c, c), M_(d, d));
    if (xy_nonzero) return M_(p.e_scale2, A_(M_(v, v), M_(p.ehalf_c2, A_(gx2, gy2))));
    if (p.twospeeds) return M_(p.e_scale2, A_(M_(v, v), M_(p.ehalf_c2b, A_(gx2, gy2))));
    return 0.0;
}

// Neumaier-compensated accumulator (Neumaier's improvement of Kahan summation, 1974):
// s is the running sum, c the sum of the rounding errors of every addition, taken
// from whichever operand was larger in magnitude; the result is s + c.
// An aggregate (no constructor, so it can live in shared memory): start it as {0.0, 0.0}.
struct Neu {
    double s, c;
    __device__ __forceinline__ void add(double x)
    {
        double t = A_(s, x);
        if (fabs(s) >= fabs(x)) c = A_(c, A_(S_(s, t), x));
        else c = A_(c, A_(S_(x, t), s));
        s = t;
    }
    __device__ __forceinline__ void merge(const Neu &o) { add(o.s); c = A_(c, o.c); }
    __device__ __forceinline__ double value() const { return A_(s, c); }
};

}  // namespace wg
