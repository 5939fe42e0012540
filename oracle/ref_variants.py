"""Configurations at which the reference itself is compiled (test infrastructure).

The reference configures everything through compile-time ``#define``s
(wave_billiard.c:46-285, wave_energy.c:46-283).  Each variant below names the macro
values of one headless build; ``oracle/build_ref.py`` patches them into a copy of the
program's define block and compiles it, and the tests build the matching runtime
``wg_params`` with :func:`params_of`.

Kinds:
  ``wb_full``  whole wave_billiard.c (setup functions included)     — benchmark configs
  ``wb_fn``    wave_billiard.c define block + global_pdes.c + the hot-path functions
               extracted verbatim (evolve_wave_half, evolve_wave, oscillating_bc,
               xy_to_ij, compute_energy)                                  — edge cases
  ``we_fn``    the same for wave_energy.c (its evolve_wave_half variant,
               compute_energy_x, compute_energy_tblr)
  ``osc``      only oscillating_bc + xy_to_ij, one build per schedule
"""

# Macro values shared by every small variant (box of the benchmark configs).
SMALL_BASE = dict(
    NX=67, NY=45, XMIN=-2.0, XMAX=2.0, YMIN=-1.125, YMAX=1.125,
    COURANT=0.1, COURANTB=0.05, GAMMA=0.0, GAMMAB=0.0, KAPPA=0.0,
    GAMMA_SIDES=1.0e-4, GAMMA_TOPBOT=1.0e-7, KAPPA_SIDES=5.0e-4, KAPPA_TOPBOT=0.0,
    TWOSPEEDS=0, OSCILLATE_LEFT=0, OSCILLATE_TOPBOT=0, OSCILLATION_SCHEDULE=0,
    B_COND=0, BC_NEUMANN=0, FLOOR=0, VMAX=2.5, E_SCALE=300.0,
    OMEGA=0.05, OMEGA_B=0.03, AMPLITUDE=1.0, DAMPING=0.0, ACHIRP=0.25,
    OSCIL_LEFT_YSHIFT=0.0, OSCIL_YMAX=0.6, OSCIL_YMID=0.1,
    INITIAL_VARIANCE=0.0003, INITIAL_SHIFT=20.0, WAVE_PACKET_SHIFT=200.0,
    INITIAL_AMP=1.0, INITIAL_WAVELENGTH=0.01,
    B_DOMAIN=1, LAMBDA=1.8, NPOLY=6, APOLY=0.0, VARIABLE_IOR=0,
)

# Config 1: plain FP64 ellipse, 1280x720, Dirichlet, COURANT 0.1, GAMMA 0.
C1 = dict(SMALL_BASE, NX=1280, NY=720, B_DOMAIN=1, LAMBDA=1.8, B_COND=0)
# Config 2: 3840x2160, 64 discs (D_CIRCLES) of index 1.5 via TWOSPEEDS, absorbing.
C2 = dict(SMALL_BASE, NX=3840, NY=2160, B_DOMAIN=20, TWOSPEEDS=1, B_COND=2,
          COURANT=0.1, COURANTB=0.1 / 1.5, GAMMA=1.0e-4, GAMMAB=1.0e-4)


def _v(kind, **kw):
    return dict(kind=kind, macros=dict(SMALL_BASE, **kw))


VARIANTS = {
    # full programs
    "c1": dict(kind="wb_full", macros=C1),
    "c2": dict(kind="wb_full", macros=C2),
    # config 2 built with the reference makefile's flags (-O3 -fopenmp, default FP
    # contraction): the timed CPU baseline, not a parity pin
    "c2_stock": dict(kind="wb_full", macros=C2, stock=True),
    "full_neu_ellipse": _v("wb_full", BC_NEUMANN=1, B_DOMAIN=1, LAMBDA=1.8),
    "full_neu_polygon": _v("wb_full", BC_NEUMANN=1, B_DOMAIN=8, LAMBDA=0.9, NPOLY=7, APOLY=0.3),
    "full_stadium": _v("wb_full", B_DOMAIN=2, LAMBDA=1.2, TWOSPEEDS=1, GAMMAB=2e-4),
    # frames: wave_value with the C_ONEDIM scheme and the turbo palette (every plot mode),
    # the frame parameters of wave_billiard.c; a second build with attenuation and the
    # full colour range, a third with two speeds (drawn everywhere, fading by tcc)
    "frame": _v("wb_full", NX=96, NY=64, B_DOMAIN=1, LAMBDA=1.8, COLOR_SCHEME=3, COLOR_PALETTE=10,
                SLOPE=1.0, COLOR_RANGE=0.8, ATTENUATION=0.0, VSHIFT_AMPLITUDE=-0.2, VSCALE_AMPLITUDE=1.0,
                LOG_SCALE=0.75, LOG_SHIFT=0.75, FLUX_SCALE=250.0, AVRG_E_FACTOR=0.95, RESCALE_COLOR_IN_CENTER=0),
    "frame_att": _v("wb_full", NX=96, NY=64, B_DOMAIN=2, LAMBDA=1.2, COLOR_SCHEME=3, COLOR_PALETTE=10,
                    SLOPE=1.5, COLOR_RANGE=1.0, ATTENUATION=0.01, VSHIFT_AMPLITUDE=0.1, VSCALE_AMPLITUDE=2.0,
                    LOG_SCALE=0.5, LOG_SHIFT=1.0, FLUX_SCALE=100.0, AVRG_E_FACTOR=0.9, RESCALE_COLOR_IN_CENTER=0),
    "frame_ts": _v("wb_full", NX=96, NY=64, B_DOMAIN=1, LAMBDA=1.8, TWOSPEEDS=1, COLOR_SCHEME=3, COLOR_PALETTE=10,
                   SLOPE=1.0, COLOR_RANGE=0.8, ATTENUATION=0.0, VSHIFT_AMPLITUDE=-0.2, VSCALE_AMPLITUDE=1.0,
                   LOG_SCALE=0.75, LOG_SHIFT=0.75, FLUX_SCALE=250.0, AVRG_E_FACTOR=0.95, RESCALE_COLOR_IN_CENTER=0),
    # hot path, every boundary rule
    "s_dir": _v("wb_fn", B_COND=0, KAPPA=0.001, FLOOR=1, VMAX=0.3),
    "s_per": _v("wb_fn", B_COND=1, TWOSPEEDS=1),
    "s_abs": _v("wb_fn", B_COND=2, TWOSPEEDS=1),
    "s_abs_mask": _v("wb_fn", B_COND=2, TWOSPEEDS=0, B_DOMAIN=2, LAMBDA=3.0),
    "s_vph": _v("wb_fn", B_COND=3, OSCILLATE_LEFT=1, NX=45, NY=67, OSCIL_LEFT_YSHIFT=5.0),
    "s_vph_beam": _v("wb_fn", B_COND=3, OSCILLATE_LEFT=1, OSCILLATION_SCHEDULE=42),
    "s_topbot": _v("wb_fn", B_COND=0, OSCILLATE_TOPBOT=1, TWOSPEEDS=1),
    "s_neu": _v("wb_fn", B_COND=0, BC_NEUMANN=1),
    "s_neu_ts": _v("wb_fn", B_COND=1, BC_NEUMANN=1, TWOSPEEDS=1, FLOOR=1, VMAX=0.4),
    "s_square": _v("wb_fn", NX=48, NY=48, OSCILLATE_LEFT=1, B_COND=0),
    "s_tiny": _v("wb_fn", NX=3, NY=3, B_COND=1, TWOSPEEDS=1),
    # wave_energy's variant
    "e_dir": _v("we_fn", NX=67, NY=90, B_COND=0),
    "e_per_osc": _v("we_fn", NX=67, NY=90, B_COND=1, TWOSPEEDS=1, OSCILLATE_LEFT=1),
    "e_vph": _v("we_fn", NX=67, NY=90, B_COND=3, TWOSPEEDS=1, FLOOR=1, VMAX=0.3),
    "e_abs": _v("we_fn", NX=67, NY=90, B_COND=2, E_SCALE=20.0),
}

# oscillating_bc: one tiny build per schedule (and a negative y-shift for the
# branches that test its sign).
OSC_SCHEDULES = [0, 1, 2, 21, 3, 4, 41, 42, 43, 44, 5, 51, 6, 61, 7]
for _s in OSC_SCHEDULES:
    VARIANTS[f"osc_{_s}"] = _v("osc", OSCILLATION_SCHEDULE=_s, OSCIL_LEFT_YSHIFT=3.0,
                               DAMPING=0.001, OMEGA=0.02, INITIAL_SHIFT=2.0,
                               WAVE_PACKET_SHIFT=5.0)
VARIANTS["osc_0_neg"] = _v("osc", OSCILLATION_SCHEDULE=0, OSCIL_LEFT_YSHIFT=-3.0)
VARIANTS["osc_7_neg"] = _v("osc", OSCILLATION_SCHEDULE=7, OSCIL_LEFT_YSHIFT=-3.0)

# wg_params field <- macro
_PARAM_OF_MACRO = dict(
    nx="NX", ny="NY", b_cond="B_COND", twospeeds="TWOSPEEDS", bc_neumann="BC_NEUMANN",
    oscillate_left="OSCILLATE_LEFT", oscillate_topbot="OSCILLATE_TOPBOT",
    oscillation_schedule="OSCILLATION_SCHEDULE", floor_clamp="FLOOR",
    xmin="XMIN", xmax="XMAX", ymin="YMIN", ymax="YMAX",
    courant="COURANT", courantb="COURANTB", gamma="GAMMA", gammab="GAMMAB",
    kappa="KAPPA", kappa_sides="KAPPA_SIDES", kappa_topbot="KAPPA_TOPBOT",
    gamma_sides="GAMMA_SIDES", gamma_topbot="GAMMA_TOPBOT",
    omega="OMEGA", omega_b="OMEGA_B", amplitude="AMPLITUDE", damping="DAMPING",
    achirp="ACHIRP", oscil_ymax="OSCIL_YMAX", oscil_ymid="OSCIL_YMID",
    oscil_left_yshift="OSCIL_LEFT_YSHIFT", initial_variance="INITIAL_VARIANCE",
    initial_shift="INITIAL_SHIFT", wave_packet_shift="WAVE_PACKET_SHIFT",
    vmax="VMAX", e_scale="E_SCALE",
)


def params_dict(name):
    """wg_params field values (as a dict) of a variant."""
    m = VARIANTS[name]["macros"]
    return {f: m[mac] for f, mac in _PARAM_OF_MACRO.items()}


def macro_text(value):
    """C literal for a macro value (doubles printed round-trip exact)."""
    if isinstance(value, bool):
        return str(int(value))
    if isinstance(value, int):
        return str(value)
    return repr(float(value))

# The reference with its stepper replaced by the GPU drop-in (include/wavegpu_dropin.h).
for _n in ["s_dir", "s_per", "s_abs", "s_vph", "s_vph_beam", "s_topbot", "s_neu", "s_neu_ts", "s_square"]:
    VARIANTS[_n + "__dropin"] = dict(VARIANTS[_n], dropin=True)
