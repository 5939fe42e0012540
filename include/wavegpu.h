/*
 * wavegpu.h — C ABI of libwavegpu.so, the sm_103a (GB300) implementation of the
 * explicit leapfrog wave-equation stepper of nilsberglund-orleans/YouTube-simulations
 * (`wave_billiard`) and the energy diagnostics of `wave_energy`.
 *
 * Plain C types only: pointers, sizes, int32 status codes.  No CUDA or torch type
 * appears in a signature; a CUDA stream is passed as `void *` (cudaStream_t).
 *
 * Two surfaces:
 *   1. Drop-in: the reference's own functions with the reference's argument meaning,
 *      row-pointer field layout (`double *phi[NX]`, each row NY values, j contiguous)
 *      and compile-time configuration turned into a runtime wg_params.  The header
 *      wavegpu_dropin.h builds that wg_params from the reference's macros.
 *   2. Native handle API: scenes resident in HBM, FP64 or FP32, runtime sizes,
 *      batches of uneven scenes, and a serving loop.
 *
 * Every function returns WG_OK (0) or a negative wg_status; wg_last_error() gives a
 * thread-local message for the last failure of the calling thread.
 */
#ifndef WAVEGPU_H
#define WAVEGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------- */
/* Status codes                                                               */
/* ------------------------------------------------------------------------- */
typedef int32_t wg_status;
enum {
    WG_OK = 0,
    WG_ERR_INVALID = -1,   /* bad argument or size */
    WG_ERR_CUDA = -2,      /* a CUDA runtime call failed */
    WG_ERR_NOMEM = -3,     /* device or pinned allocation failed */
    WG_ERR_BUDGET = -4,    /* admission refused: HBM budget exceeded */
    WG_ERR_STATE = -5,     /* call not valid in the object's current state */
    WG_ERR_TIMEOUT = -6,   /* a bounded device/host wait gave up */
    WG_ERR_NONFINITE = -7, /* a field holds NaN/Inf (blow-up detector) */
    WG_ERR_NOTFOUND = -8   /* unknown scene/request id */
};

/* ------------------------------------------------------------------------- */
/* Configuration: the reference's compile-time macros as a runtime struct.    */
/* Names follow the macros of wave_billiard.c:46-285 and global_pdes.c.       */
/* ------------------------------------------------------------------------- */
enum { WG_BC_DIRICHLET = 0, WG_BC_PERIODIC = 1, WG_BC_ABSORBING = 2, WG_BC_VPER_HABS = 3 };

/* OSCILLATION_SCHEDULE values (global_pdes.c:282-296) */
enum {
    WG_OSC_PERIODIC = 0, WG_OSC_SLOWING = 1, WG_OSC_WAVE_PACKET = 2, WG_OSC_WAVE_PACKETS = 21,
    WG_OSC_CHIRP = 3, WG_OSC_BEAM = 4, WG_OSC_BEAM_GAUSSIAN = 41, WG_OSC_BEAM_SINE = 42,
    WG_OSC_BEAM_SINE_DECREASING = 43, WG_OSC_BEAM_SINE_CHIRP = 44, WG_OSC_BEAM_TWOPERIODS = 5,
    WG_OSC_BEAM_SINE_TWOPERIODS = 51, WG_OSC_TWO_WAVES = 6, WG_OSC_TWO_WAVES_ADDED = 61,
    WG_OSC_TWOFREQ_TOPBOT = 7
};

enum { WG_FP64 = 0, WG_FP32 = 1 };

/* Coefficient storage of a native scene.
 *  WG_COEF_MASK : tcc/tgamma/tc follow the mask bit exactly as init_ior_2d's constant
 *                 branch builds them (sub_wave.c:12983-13002): inside COURANT^2/GAMMA/
 *                 COURANT, outside (TWOSPEEDS) COURANTB^2/GAMMAB/COURANTB.  0 bytes/cell.
 *  WG_COEF_TABLE: a spatially varying tcc table is kept on the device (S bytes/cell);
 *                 tgamma is a table too unless it is uniform; tc is kept for the four
 *                 boundary lines only (it is read nowhere else). */
enum { WG_COEF_MASK = 0, WG_COEF_TABLE = 1 };

typedef struct wg_params {
    int32_t nx, ny;                 /* NX, NY: grid size, field[i][j], j contiguous */
    int32_t b_cond;                 /* B_COND (WG_BC_*) */
    int32_t twospeeds;              /* TWOSPEEDS */
    int32_t bc_neumann;             /* BC_NEUMANN */
    int32_t oscillate_left;         /* OSCILLATE_LEFT */
    int32_t oscillate_topbot;       /* OSCILLATE_TOPBOT */
    int32_t oscillation_schedule;   /* OSCILLATION_SCHEDULE (WG_OSC_*) */
    int32_t floor_clamp;            /* FLOOR */
    int32_t src_on;                 /* project point source on/off (see src_*) */
    int32_t src_i, src_j;           /* point-source cell */
    double xmin, xmax, ymin, ymax;  /* XMIN, XMAX, YMIN, YMAX */
    double courant, courantb;       /* COURANT, COURANTB */
    double gamma, gammab;           /* GAMMA, GAMMAB (used by WG_COEF_MASK) */
    double kappa, kappa_sides, kappa_topbot;  /* KAPPA, KAPPA_SIDES, KAPPA_TOPBOT */
    double gamma_sides, gamma_topbot;         /* GAMMA_SIDES, GAMMA_TOPBOT */
    double omega, omega_b, amplitude, damping, achirp;       /* OMEGA, OMEGA_B, AMPLITUDE, DAMPING, ACHIRP */
    double oscil_ymax, oscil_ymid, oscil_left_yshift;        /* OSCIL_YMAX, OSCIL_YMID, OSCIL_LEFT_YSHIFT */
    double initial_variance, initial_shift, wave_packet_shift; /* INITIAL_VARIANCE, INITIAL_SHIFT, WAVE_PACKET_SHIFT */
    double vmax;                    /* VMAX (FLOOR clamp) */
    double e_scale;                 /* E_SCALE (energy) */
    /* Point source of the project (not in the reference): after update number t
     * (t counts from 1), phi_out[src_i][src_j] += src_amp * sin(2*pi*t/src_period). */
    double src_amp, src_period;
} wg_params;

/* Neumann boundary record, binary-identical to t_neumann_bc (global_pdes.c:518-528). */
typedef struct wg_neumann_bc {
    double nx, ny;
    int16_t signx1, signy1;
    int16_t signx2, signy2;
    int32_t nbi1, nbj1, nbk1;
    int32_t nbi2, nbj2, nbk2;
    int32_t i, j, k;
    int16_t top;
    int16_t active;
} wg_neumann_bc;

/* Fills *p with the macro values of wave_billiard.c:46-285 for the fields it shares
 * with wg_params, sized nx x ny, box [-2,2]x[-1.125,1.125]. */
void wg_params_default(wg_params *p, int32_t nx, int32_t ny);

const char *wg_last_error(void);
const char *wg_status_string(wg_status s);
int32_t wg_abi_version(void);

/* ------------------------------------------------------------------------- */
/* 1. Drop-in surface (row-pointer layout, FP64, reference semantics)          */
/* ------------------------------------------------------------------------- */

/* Sets NX, NY and the macros used by the drop-in calls below.  Replaces the
 * compile-time #defines of wave_billiard.c:46-285; wavegpu_dropin.h calls it. */
wg_status wg_dropin_configure(const wg_params *p);

/* Drop-in transfer modes.
 *  WG_DROPIN_STRICT  : every call copies the fields in, steps on the GPU and copies
 *                      them back, so host arrays are current after each call.
 *  WG_DROPIN_RESIDENT: fields stay in HBM between calls (matched by the row-pointer
 *                      arrays' identity); wg_dropin_sync() copies them back and
 *                      wg_dropin_invalidate() forces a fresh upload after host edits. */
enum { WG_DROPIN_STRICT = 0, WG_DROPIN_RESIDENT = 1 };
wg_status wg_dropin_set_mode(int32_t mode);
wg_status wg_dropin_sync(void);
wg_status wg_dropin_invalidate(void);
/* How the drop-in moves rows between the caller's row arrays and the GPU.
 *  WG_ROWS_AUTO  : in place where the GPU can address the host's pageable memory
 *                  (cudaDevAttrPageableMemoryAccess, e.g. a Grace host): kernels read
 *                  and write the rows over the host link, with no host-side packing;
 *                  elsewhere as WG_ROWS_PACKED.  The default.
 *  WG_ROWS_PACKED: host threads pack the rows into a page-locked stage, one copy.
 * Either way each call waits for its reads of the caller's rows before it returns. */
enum { WG_ROWS_AUTO = 0, WG_ROWS_PACKED = 1 };
wg_status wg_dropin_set_rows(int32_t rows_mode);
/* Step counter of the drop-in (the reference's `static long time`, wave_billiard.c:310). */
wg_status wg_dropin_get_time(int64_t *t);
wg_status wg_dropin_set_time(int64_t t);

/* Replaces evolve_wave_half (wave_billiard.c:302-610): one leapfrog update,
 * phi_out <- F(phi_in, psi_in).  Arrays are NX row pointers of NY values each. */
wg_status wg_evolve_wave_half(double **phi_in, double **psi_in, double **phi_out,
                              int16_t **xy_in, double **tcc, double **tc, double **tgamma,
                              const wg_neumann_bc *neumann_bc, int32_t n_neumann);

/* Replaces evolve_wave (wave_billiard.c:613-631): three updates with the
 * phi -> tmp -> psi -> phi buffer rotation. */
wg_status wg_evolve_wave(double **phi, double **psi, double **tmp,
                         int16_t **xy_in, double **tcc, double **tc, double **tgamma,
                         const wg_neumann_bc *neumann_bc, int32_t n_neumann);

/* Replaces the wave_energy variant (wave_energy.c:662-925): the stepper on the half
 * domain j < NY/2 with coefficient tables built from the mask and the macros. */
wg_status wg_evolve_wave_half_energy(double **phi_in, double **psi_in, double **phi_out,
                                     int16_t **xy_in);
wg_status wg_evolve_wave_energy(double **phi, double **psi, double **tmp, int16_t **xy_in);

/* compute_energy (wave_common.c:453-472) for one cell. */
wg_status wg_compute_energy(double **phi, double **psi, int16_t **xy_in,
                            int32_t i, int32_t j, double *out);
/* compute_energy_x for every column i (wave_energy.c:292-302): out[i] = sum_{j<NY/2} E(i,j). */
wg_status wg_compute_energy_x_all(double **phi, double **psi, int16_t **xy_in, double *out);
/* compute_energy_tblr (sub_wave_comp.c:1752-1858) with the box limits given. */
wg_status wg_compute_energy_tblr(double **phi, double **psi, int16_t **xy_in,
                                 int32_t ileft, int32_t iright, double energies[6]);

/* add_circular_wave (wave_common.c:337-351): phi += init_amp*factor*exp(-r^2/variance)
 * *cos(-r/wavelength) on the cells with xy_in != 0 (every cell with TWOSPEEDS), r the
 * distance of the cell centre (ij_to_xy, sub_wave.c:469-476) from (x, y); psi is not
 * touched.  init_amp, variance, wavelength are the reference's INITIAL_AMP,
 * INITIAL_VARIANCE, INITIAL_WAVELENGTH.  Strict mode: the caller's phi rows are
 * updated; resident mode: the device copy of phi (wg_dropin_sync before reading it). */
wg_status wg_dropin_add_circular_wave(double init_amp, double factor, double x, double y, double variance,
                                      double wavelength, double **phi, double **psi, int16_t **xy_in);

/* phi[i][j] as the drop-in holds it: the resident device copy when `phi` is one of the
 * resident arrays (one 8-byte read, no full sync; SAVE_TIME_SERIES sampling in
 * animation(), wave_billiard.c:900-908), else the caller's own row. */
wg_status wg_dropin_cell(double **phi, int32_t i, int32_t j, double *out);

/* Energy diagnostics over device fields the caller owns, without any allocation.
 * No counterpart in the reference: it is for callers that cannot allocate device
 * memory at the time they need the diagnostics, e.g. a host program that carves all
 * of its device memory out of its own arena at start-up, or a service that must not
 * call cudaMalloc (which can block on device-wide synchronisation) while it serves.
 * phi, psi: FP64 fields [nx][pitch] in device memory; xy: int16 mask [nx][pitch] in
 * device memory (pitch >= ny, in elements); out: nx + 7 doubles in device memory that
 * receive out[0] = total, out[1..6] = the six compute_energy_tblr boxes for
 * ileft/iright, out[7 + i] = compute_energy_x(i).  The work is enqueued on `stream`
 * (cudaStream_t; NULL = the default stream) and the call returns without waiting.
 * Per-column partial sums go to a fixed scratch array in the library's device memory
 * (WG_NOALLOC_MAX_NX columns at most; larger nx is refused with WG_ERR_INVALID).
 * The first call on a device looks up that array's address; make it before any
 * stream capture.  All calls share the array: calls that overlap on the GPU race. */
#define WG_NOALLOC_MAX_NX 16384
wg_status wg_compute_energy_device_noalloc(const wg_params *p, const double *phi, const double *psi,
                                           const int16_t *xy, int32_t pitch, int32_t ileft, int32_t iright,
                                           double *out, void *stream);

/* ------------------------------------------------------------------------- */
/* 2. Native handle API: resident scenes                                       */
/* ------------------------------------------------------------------------- */
/* No counterpart in the reference's interface, which is one compile-time grid per
 * program stepped through host arrays (wave_billiard.c:613-631 from animation(),
 * :897-899).  A scene holds one such grid on the device with runtime sizes: upload
 * replaces the set-up of phi/psi/xy_in and the tables (init_ior_2d, sub_wave.c:12983-
 * 13002), step replaces the evolve_wave loop, energy replaces compute_energy /
 * compute_energy_x / compute_energy_tblr, frames replace draw_wave_highres_palette
 * (wave_common.c:1750-1848) without GL. */
typedef struct wg_scene wg_scene;

/* Creates a scene with device buffers for phi/psi, the packed mask and coefficients.
 * precision: WG_FP64 or WG_FP32.  coef_mode: WG_COEF_MASK or WG_COEF_TABLE.
 * An FP32 scene stores phi and the velocity phi - psi (each rounded once from FP64
 * values), in two pairs of fields: every update writes the other pair.
 * stream: cudaStream_t to run on (NULL = a stream owned by the scene).
 * FP64 scenes give the values of the reference's stepper (evolve_wave_half,
 * wave_billiard.c:302-610).  Where KAPPA = 0, or GAMMA is 0 on every cell, the zero
 * term is left out of the update, so a zero result may differ in sign only; with
 * every term present the fields are bit-identical.  The drop-in keeps every term. */
wg_status wg_scene_create(const wg_params *p, int32_t precision, int32_t coef_mode,
                          void *stream, wg_scene **out);
wg_status wg_scene_destroy(wg_scene *s);
/* Device bytes the scene holds (fields, mask, tables, scratch). */
wg_status wg_scene_bytes(const wg_params *p, int32_t precision, int32_t coef_mode, size_t *bytes);

/* Uploads flat [nx][ny] FP64 host arrays (j contiguous).  xy_in is the reference's
 * short mask.  tcc/tc/tgamma may be NULL in WG_COEF_MASK mode.  Values are rounded
 * to the scene precision on the device (FP32: phi and the FP64 difference phi - psi). */
wg_status wg_scene_upload(wg_scene *s, const double *phi, const double *psi, const int16_t *xy_in,
                          const double *tcc, const double *tc, const double *tgamma);
/* Uploads only phi/psi (the state), from FP64 or from the scene's own precision.  From
 * arrays in an FP32 scene's own precision the call returns without waiting: page-locked
 * arrays are read by the device in stream order (leave them unchanged until a call that
 * waits: energy, download, sync), pageable arrays are copied before the call returns.
 * Page-locked host arrays (cudaHostAlloc, cudaHostRegister) of FP32 scenes are read and
 * written by the device in place, over the host link, with no staging copy. */
wg_status wg_scene_upload_state(wg_scene *s, const void *phi, const void *psi, int32_t host_precision);
wg_status wg_scene_set_neumann(wg_scene *s, const wg_neumann_bc *recs, int32_t n);
/* Advances nsteps leapfrog updates (one kernel pass per temporal block). */
wg_status wg_scene_step(wg_scene *s, int32_t nsteps);
/* Copies phi (time t) and psi (time t-1) to flat host arrays in FP64 or the scene's
 * precision.  Either pointer may be NULL.  FP32 scenes return psi = phi - v computed in
 * FP64 (rounded to FP32 for an FP32 host array). */
wg_status wg_scene_download(wg_scene *s, void *phi, void *psi, int32_t host_precision);
/* Energy diagnostics (compute_energy per cell, wave_common.c:453-472) with compensated
 * sums: FP64 Neumaier accumulators for FP64 fields; for FP32 fields (cell energies in
 * FP32) an error-free FP32 double-word accumulator converted exactly to FP64 per column;
 * columns, boxes and the total merged in FP64 Neumaier sums.
 *  total   : sum of compute_energy over all cells (may be NULL)
 *  columns : nx values, sum over j < ny/2 (compute_energy_x), may be NULL
 *  boxes   : 6 values (compute_energy_tblr) for ileft/iright, may be NULL */
wg_status wg_scene_energy(wg_scene *s, double *total, double *columns,
                          int32_t ileft, int32_t iright, double *boxes);
wg_status wg_scene_get_time(wg_scene *s, int64_t *t);
wg_status wg_scene_set_time(wg_scene *s, int64_t t);
wg_status wg_scene_sync(wg_scene *s);
/* Temporal-block depth (updates per kernel pass) and tile shape; 0 = autotuned. */
wg_status wg_scene_set_blocking(wg_scene *s, int32_t k, int32_t tile_i, int32_t tile_j);
wg_status wg_scene_get_blocking(wg_scene *s, int32_t *k, int32_t *tile_i, int32_t *tile_j);
/* Number of kernel launches this library issued for the scene so far. */
wg_status wg_scene_launch_count(wg_scene *s, int64_t *n);
/* Blow-up detector: *bad = number of non-finite phi values (0 = healthy). */
wg_status wg_scene_check_finite(wg_scene *s, int64_t *bad);

/* Colour-mapped frame of draw_wave_highres_palette (wave_common.c:1053-1162,
 * 1750-1848; colors_waves.c:3-16,161-218; colormaps.c:2449-2482) at every size-th
 * cell, as an RGB8 image of (ny/size) rows x (nx/size) columns, row r = j/size from
 * the bottom (GL's origin), column = i/size, for the C_ONEDIM colour scheme with the
 * caller's 256x3 byte palette `lut` (e.g. the reference's turbo_srgb_bytes).
 * Per sampled cell, `plot` selects the value (wave_value, wave_common.c:1053-1162):
 *   WG_P_AMPLITUDE  VSHIFT + VSCALE*phi;  WG_P_ENERGY  compute_energy;  WG_P_MIXED
 *   phi above NY/2, energy below;  WG_P_MEAN_ENERGY  running sum of energy / (time+1);
 *   WG_P_LOG_ENERGY / _LOG_MEAN_ENERGY  LOG_SHIFT + LOG_SCALE*log(...);  WG_P_ENERGY_FLUX
 *   FLUX_SCALE*|phi-psi|*|grad phi|;  WG_P_TOTAL_ENERGY_FLUX  direction of the decaying
 *   (x0.99 per frame) sum of the flux on a wrapped linear scale, dimmed by
 *   tanh(FLUX_SCALE*|sum|);  WG_P_AVERAGE_ENERGY / _LOG_AVERAGE_ENERGY  exponential
 *   average with AVRG_E_FACTOR.
 * amplitude = COLOR_RANGE*tanh(SLOPE*value/scale)*exp(-time*ATTENUATION); palette entry
 * (int)(256*h), clamped to 0..255, with h = 0.5*(1 + amplitude), or h = amplitude for
 * the energy and flux modes (color_scheme_asym_palette).  Drawn cells (TWOSPEEDS or
 * xy != 0) take that entry times the optional fades, rounded; other cells are black.
 * The running sums (mean, average, total flux) live in the scene at frame resolution
 * and are updated on every sampled cell by each call; they restart at zero on
 * wg_scene_frame_reset or when `plot` or `size` changes.
 * rgb_host and/or rgb_device receive the image (either may be NULL). */
enum { WG_P_AMPLITUDE = 0, WG_P_ENERGY = 1, WG_P_MIXED = 2, WG_P_MEAN_ENERGY = 3, WG_P_LOG_ENERGY = 4,
       WG_P_LOG_MEAN_ENERGY = 5, WG_P_ENERGY_FLUX = 6, WG_P_TOTAL_ENERGY_FLUX = 7, WG_P_AVERAGE_ENERGY = 8,
       WG_P_LOG_AVERAGE_ENERGY = 9 };  /* P_* of global_pdes.c:318-327 */
typedef struct wg_frame_params {
    int32_t size;            /* downsampling (draw_wave_highres_palette's size=2) */
    int32_t fade;            /* apply fade_value */
    double vshift, vscale;   /* VSHIFT_AMPLITUDE, VSCALE_AMPLITUDE */
    double slope, color_range, scale; /* SLOPE, COLOR_RANGE, scale */
    double fade_value;
    int32_t fade_in_obstacle; /* FADE_IN_OBSTACLE: times (tcc/COURANT^2)^0.1 (wave_common.c:1739-1748) */
    int32_t plot;            /* WG_P_* */
    double log_shift, log_scale;  /* LOG_SHIFT, LOG_SCALE */
    double flux_scale;       /* FLUX_SCALE */
    double avrg_e_factor;    /* AVRG_E_FACTOR */
    double attenuation;      /* ATTENUATION */
    int32_t time;            /* the frame counter `time` of draw_wave_highres_palette */
    int32_t reserved;
} wg_frame_params;
wg_status wg_scene_frame_rgb8(wg_scene *s, const wg_frame_params *fp, const uint8_t *lut,
                              uint8_t *rgb_host, void *rgb_device);
/* Restart the frame's running sums (the reference's total_energy, average_energy and
 * total_flux arrays) at zero. */
wg_status wg_scene_frame_reset(wg_scene *s);
/* Mask and tables built on the device instead of wg_scene_upload's host arrays:
 * xy_in_billiard_single_domain (sub_wave.c:5712-6252) at every cell centre for domain
 * 0 rectangle, 1 ellipse, 2 stadium, 8 polygon (npoly, apoly), 20 discs, 201 discs in a
 * rectangle (circles: ncircles x (xc, yc, radius), the reference's circles[]), and for
 * WG_COEF_TABLE scenes the tables of init_ior_2d (sub_wave.c:12983-13002).  Then
 * wg_scene_upload_state sets phi and psi.  Masks are 0/1.  A Neumann scene (BC_NEUMANN,
 * WG_COEF_TABLE, domain 1 or 8) also gets the set-up of init_neumann_bc
 * (sub_wave.c:13720-13947) on the device after its tables: ghost cells (outside, a
 * 4-neighbour inside) marked -1, one record each in the reference's row-major order, with
 * test_neumann_data's deactivation.  The polygon's cos/sin (and its normal's atan) are
 * CUDA's: a cell within rounding of an edge may fall on the other side. */
wg_status wg_scene_build_domain(wg_scene *s, int32_t domain, double lambda, int32_t npoly, double apoly,
                                const double *circles, int32_t ncircles);
/* The scene's mask, [nx][ny]: 1 inside, 0 outside, -1 for Neumann ghost cells. */
wg_status wg_scene_download_mask(wg_scene *s, int16_t *xy);
/* The Neumann records wg_scene_build_domain made on the device (the reference's
 * t_neumann_bc, global_pdes.c:518-528): *count = their number; out (room for capacity
 * records) may be NULL to ask the count only.  WG_ERR_STATE for records set from the
 * host. */
wg_status wg_scene_neumann_records(wg_scene *s, wg_neumann_bc *out, int32_t capacity, int32_t *count);
/* RGB8 frame (row 0 at the bottom, width x height pixels) to a file: the uncompressed
 * baseline TIFF of writetiff (sub_wave.c:62-122: 8-bit RGB, one row per strip,
 * ORIENTATION_BOTLEFT, `description` as ImageDescription, scanline s = row
 * height-1-s), or a binary PPM (P6, top row first).  Host-only; no GPU needed. */
wg_status wg_write_tiff(const char *path, const char *description, const uint8_t *rgb, int32_t width,
                        int32_t height);
wg_status wg_write_ppm(const char *path, const uint8_t *rgb, int32_t width, int32_t height);
/* SAVE_TIME_SERIES (wave_billiard.c:667-672, 900-908): record phi at n cells (i[k], j[k])
 * after every update, room for `capacity` updates (n = 0 removes the probes).  While
 * probes are set the scene takes single updates (no temporal blocking).  A step that
 * would overflow the buffer is refused (WG_ERR_STATE) until the samples are read.
 * wg_scene_read_probes copies the oldest min(count, max_updates) updates x n values
 * (update-major) to `out` and drops them from the buffer. */
wg_status wg_scene_set_probes(wg_scene *s, int32_t n, const int32_t *i, const int32_t *j, int32_t capacity);
wg_status wg_scene_read_probes(wg_scene *s, double *out, int32_t max_updates, int32_t *count);
/* add_circular_wave (wave_common.c:337-351) on the scene's phi (level t): the pulse of
 * wg_dropin_add_circular_wave, with the scene's mask and TWOSPEEDS.  Only the cells where
 * exp(-r^2/variance) is nonzero in double precision are visited. */
wg_status wg_scene_add_circular_wave(wg_scene *s, double init_amp, double factor, double x, double y,
                                     double variance, double wavelength);

/* ------------------------------------------------------------------------- */
/* 3. Batches of uneven scenes: one persistent launch over a tile work queue   */
/* ------------------------------------------------------------------------- */
/* No counterpart in the reference (one grid per process): many scenes of different
 * sizes and parameters stepped together, each by the reference's rules. */
typedef struct wg_batch wg_batch;
wg_status wg_batch_create(int32_t precision, void *stream, wg_batch **out);
wg_status wg_batch_destroy(wg_batch *b);
/* Adds a scene (WG_COEF_MASK only) to the batch; *slot gets its index. */
wg_status wg_batch_add(wg_batch *b, const wg_params *p, const double *phi, const double *psi,
                       const int16_t *xy_in, int32_t *slot);
/* Removes a scene; its device memory is returned to the batch's pool. */
wg_status wg_batch_remove(wg_batch *b, int32_t slot);
/* Advances every active scene by nsteps updates, the launches of a frame recorded
 * once as a CUDA graph.  Scenes take single updates (one persistent kernel per update
 * over a tile work queue) or, for FP32 scenes with mirror or absorbing boundaries and
 * nsteps >= 2, skewed passes of 2..6 updates at the depth of their size class; both
 * give the same fields bit for bit. */
wg_status wg_batch_step(wg_batch *b, int32_t nsteps);
/* Skewed passes: mode -1 (default) tunes a depth and a row chunk per size class
 * (floor(log2(cells)) - 10, 16 classes) at the first frame that needs it; 0 turns them
 * off; 2..6 fixes the depth. */
wg_status wg_batch_set_skew(wg_batch *b, int32_t mode);
/* depths[16]: the depth of each size class (0: not tuned / none); chunk_rows[16]
 * (optional): the tuned rows of a task's row chunk (0: sized from the whole list's work);
 * ms_per_update[16*8] (optional): the autotuner's best time per update of class c at
 * depth K, [c*8 + K]. */
wg_status wg_batch_skew_depths(wg_batch *b, int32_t *depths, int32_t *chunk_rows, double *ms_per_update);
wg_status wg_batch_download(wg_batch *b, int32_t slot, double *phi, double *psi);
wg_status wg_batch_energy(wg_batch *b, int32_t slot, double *total);
wg_status wg_batch_count(wg_batch *b, int32_t *n_active, int64_t *cells);
wg_status wg_batch_launch_count(wg_batch *b, int64_t *n);

/* ------------------------------------------------------------------------- */
/* 4. Serving loop: continuous batching of scene requests under an HBM budget  */
/* ------------------------------------------------------------------------- */
/* No counterpart in the reference: requests admitted into a running batch, each frame
 * colour-mapped as the reference's P_AMPLITUDE drawing does (wave_common.c:1053-1065). */
typedef struct wg_server wg_server;
typedef struct wg_server_config {
    int32_t precision;        /* WG_FP32 or WG_FP64 */
    int32_t steps_per_frame;  /* leapfrog updates per returned frame */
    int32_t max_scenes;       /* resident scenes at most */
    int32_t pipeline;         /* 0: a tick returns with its frames in host memory;
                                 1: pipelined ticks (see wg_server_tick) */
    uint64_t hbm_budget;      /* device bytes the resident scenes may hold */
    wg_frame_params frame;    /* colour map of the returned frames */
    uint8_t lut[768];         /* 256x3 palette bytes (the reference's turbo_srgb_bytes) */
} wg_server_config;
typedef struct wg_server_stats {
    int64_t submitted, admitted, completed, queued, resident, frames, ticks;
    double cell_updates;                  /* cell updates performed */
    double busy_seconds;                  /* wall time inside wg_server_tick / wg_server_drain */
    /* per frame: from the host's enqueue of the tick that renders it to the host seeing
     * the frame in host memory (with pipelined ticks this includes waiting behind the
     * previous tick's device work) */
    double frame_latency_p50_ms, frame_latency_p99_ms, frame_latency_max_ms;
    double first_frame_p50_ms, first_frame_p99_ms;  /* submit -> first frame on the host */
    uint64_t bytes_resident, bytes_peak;
    /* per tick: device time from the tick's first kernel to its frames in host memory */
    double tick_device_p50_ms, tick_device_p99_ms;
    int64_t cancelled;
} wg_server_stats;
enum { WG_REQ_QUEUED = 0, WG_REQ_RESIDENT = 1, WG_REQ_DONE = 2, WG_REQ_CANCELLED = 3 };

wg_status wg_server_create(const wg_server_config *cfg, void *stream, wg_server **out);
wg_status wg_server_destroy(wg_server *s);
/* Queues a scene request (mask values 0/1; the arrays are copied).  It is admitted at a
 * later tick, first come first served, as soon as its device bytes fit the budget. */
wg_status wg_server_submit(wg_server *s, const wg_params *p, const double *phi, const double *psi,
                           const int16_t *xy, int32_t frames, int32_t keep_result, int64_t *request_id);
/* One tick: retire requests whose frames are all rendered and cancelled ones, admit
 * what fits, advance every resident scene by one frame (one CUDA-graph launch for all of
 * them), render every scene's frame and copy them to host memory.
 * pipeline = 0: the tick waits for its own frames; *frames_out = frames produced.
 * pipeline = 1: the tick enqueues its work on the device, then waits only for the
 * previous tick's frames (two frame buffers alternate), so the device works on tick t
 * while the host handles tick t-1; *frames_out = frames of the previous tick that are
 * now in host memory.  wg_server_drain completes the last enqueued tick. */
wg_status wg_server_tick(wg_server *s, int32_t *frames_out);
/* Pipelined servers: waits for the enqueued tick and makes its frames readable
 * (*frames_out = their number; 0 when no tick was pending).  No-op otherwise. */
wg_status wg_server_drain(wg_server *s, int32_t *frames_out);
/* Cancels a request: a queued one leaves the queue now; a resident one leaves the batch
 * (and returns its bytes to the budget) at the next tick, before that tick's frame.
 * Its state becomes WG_REQ_CANCELLED.  A finished request gives WG_ERR_STATE. */
wg_status wg_server_cancel(wg_server *s, int64_t request_id);
/* The latest frame of a request in host memory.  Valid until the next call that makes
 * newer frames readable (the next tick, or drain); after it the call returns
 * WG_ERR_STATE. */
wg_status wg_server_frame(wg_server *s, int64_t request_id, uint8_t *rgb, int32_t *frame_index,
                          int32_t *width, int32_t *height);
/* Final phi/psi of a finished request submitted with keep_result. */
wg_status wg_server_result(wg_server *s, int64_t request_id, double *phi, double *psi);
wg_status wg_server_request_state(wg_server *s, int64_t request_id, int32_t *state, int32_t *frames_done);
wg_status wg_server_get_stats(wg_server *s, wg_server_stats *out);
/* Device bytes a request of these parameters holds while resident (what admission
 * charges against the budget). */
wg_status wg_server_request_bytes(wg_server *s, const wg_params *p, uint64_t *bytes);

#ifdef __cplusplus
}
#endif
#endif /* WAVEGPU_H */
