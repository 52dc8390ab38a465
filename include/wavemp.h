/*
 * wavemp.h -- C ABI of the GB300 (sm_103a) implementation of the per-stage right-hand side of the
 * 2-D five-equation stiffened-gas solver of aschamarthi/Wave-Multiphase.
 *
 * The reference (sainath_SC_it_works.py "SC", Sainath_M10.py "M10") has no library interface; its
 * RHS is a set of Warp kernels driven by closures inside main() (SC:1894-1995). Each entry point
 * below replaces one of those closures with the same argument meaning and the same array layout,
 * so a host loop written like the reference's time loop (SC:2009-2082) can call them in the same
 * order. The fused entry points (wm_rhs_stage, wm_step) run the same sequence with fewer passes
 * over memory.
 *
 * Conventions (as in the reference):
 *  - Every field is a double array of (nx + 2g) rows by (ny + 2g) columns: x index i is the row,
 *    y index j is contiguous; row i starts at ptr + i * pitch (pitch >= ny + 2g, in elements).
 *    Interior cells are i in [g, g+nx), j in [g, g+ny). g >= 4 (the reference uses g = 5).
 *  - The caller owns every field array. The handle owns (or is given) the workspace: face fluxes,
 *    limiter factors, per-cell sensors and the time-step accumulator.
 *  - All device work is enqueued on the caller's stream (a cudaStream_t passed as void*; NULL is
 *    the legacy default stream) and returns without waiting, except where a host value is
 *    requested (wm_get_dt, and wm_step with dt_next != NULL).
 *  - Return codes: WM_OK (0) or a negative WM_ERR_*; no exception crosses the ABI. One handle per
 *    stream at a time: a handle is not safe for concurrent use from several streams or threads.
 */
#ifndef WAVEMP_H
#define WAVEMP_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WM_OK 0
#define WM_ERR_INVALID (-1) /* bad argument: null pointer, size, enum, pitch, alignment */
#define WM_ERR_CUDA (-2)    /* a CUDA runtime call failed; see wm_last_error() */
#define WM_ERR_NOMEM (-3)   /* device allocation failed or caller workspace too small */
#define WM_ERR_STATE (-4)   /* call out of order (e.g. limit_fluxes before compute_fluxes) */

/* Scheme variant: which reference script's face kernel (fx_kernel / gy_kernel) is followed. */
#define WM_VARIANT_SC 0  /* SC:966-1301: Ducros-gated central shear, THINC under the indicator */
#define WM_VARIANT_M10 1 /* M10:868-1222: THINC always on the interface field, Wong staged limiter
                            on reconstructed states and a pressure floor */

/* Reconstruction of the characteristic fields. */
#define WM_RECON_SHIPPED 0 /* MUSCL kappa=1/3 (SC:430-446), central-4 shear (SC:1076-1082) */
#define WM_RECON_MP5C6 1   /* MP5 (SC:353-405) where the shipped code uses MUSCL, central-6
                              (SC:407-412) where it uses central-4 */

/* Ghost-cell rule per side (bc_x_kernel / bc_y_kernel, SC:1616-1682). */
#define WM_BC_TRANSMISSIVE 0 /* copy the nearest interior cell */
#define WM_BC_SLIP 1         /* copy it and negate the wall-normal momentum and velocity */

/* Arithmetic of the face sweeps. */
#define WM_PREC_FP64 0 /* plain form: everything in binary64 */
#define WM_PREC_FP32 1 /* precision form: reconstruction and fluxes in binary32; pressure and
                          sound-speed recovery, the limiter's bound solves and the conserved-state
                          accumulation in binary64 */

typedef struct wm_params {
    double gamma1, pinf1; /* stiffened gas of fluid 1 (alpha1 = its volume fraction) */
    double gamma2, pinf2; /* fluid 2 */
    double dx, dy;        /* uniform cell sizes */
    double cfl;           /* CFL number of get_dt (SC:33) */
    int variant;          /* WM_VARIANT_* */
    int recon;            /* WM_RECON_* */
    int bc[4];            /* x-low, x-high, y-low, y-high: WM_BC_* */
    int emergency_repair; /* USE_EMERGENCY_REPAIR (SC:37): run enforce_admissible every stage */
    int precision;        /* WM_PREC_* */
    int fp64_switches;    /* WM_PREC_FP32 only: the scheme's two discontinuous switches -- the THINC
                             smoothness indicator (SC:1028-1032) and the Ducros shear sensor
                             (SC:1035-1036) -- from binary64 entropies and primitives, so that the
                             binary32 sweep takes the binary64 decisions (costs one binary64 pow a
                             cell); 0: binary32 sensors */
} wm_params;

/* The reference's ten per-cell arrays (SC:1839-1841): conserved state, primitives, al_prim. */
typedef struct wm_fields {
    double *ar1, *ar2; /* partial densities alpha1*rho1, alpha2*rho2 */
    double *ru, *rv;   /* momenta */
    double *E;         /* total energy */
    double *al;        /* alpha1 (conserved copy, clamped by update_prims) */
    double *u_p, *v_p, *p_p; /* primitives written by update_prims */
    double *al_prim;   /* alpha1 snapshot used by the non-conservative source */
    long long pitch;   /* elements between consecutive x rows */
} wm_fields;

/* Counters read back by wm_status (device-side, cumulative since wm_create or wm_reset_status). */
typedef struct wm_stats {
    long long repaired_cells;   /* cells whose energy enforce_admissible reset */
    long long nonfinite_cells;  /* cells with a NaN partial density, momentum or energy before
                                   repair */
    long long limited_cells;    /* interior cells with a limiter factor theta < 1 in any pass */
    long long steps;            /* SSP-RK3 steps run through wm_step */
} wm_stats;

typedef struct wm_handle wm_handle;

/* Library version string and the last CUDA error message seen by any entry point. */
const char *wm_version(void);
const char *wm_last_error(void);

/* Bytes of device workspace a handle needs for this grid and parameter set. */
size_t wm_workspace_bytes(const wm_params *p, int nx, int ny, int g);

/* Create a handle. With workspace == NULL the library allocates the workspace (cudaMalloc on the
 * current device); otherwise it uses the caller's device buffer of workspace_bytes >=
 * wm_workspace_bytes(), 256-byte aligned, which must outlive the handle. Replaces the buffer
 * allocations of main() (SC:1843-1866). */
int wm_create(const wm_params *p, int nx, int ny, int g, void *workspace, size_t workspace_bytes,
              wm_handle **out);
void wm_destroy(wm_handle *h);

/* ---- the reference's closures (SC:1894-1995), one call each ------------------------------- */
/* apply_bc() SC:1899-1905: fill the g ghost layers of the nine cell arrays (not al_prim). */
int wm_apply_bc(wm_handle *h, const wm_fields *q, void *stream);
/* compute_fluxes() SC:1919-1935: Ducros sensor (SC only) and the high-order x and y face fluxes
 * with the interface velocities, into the handle's workspace. */
int wm_compute_fluxes(wm_handle *h, const wm_fields *q, void *stream);
/* compute_low_fluxes() SC:1937-1947: first-order HLLC face fluxes into the workspace. */
int wm_compute_low_fluxes(wm_handle *h, const wm_fields *q, void *stream);
/* limit_fluxes(dt) SC:1949-1972: three Wong limiter passes blending the high-order fluxes toward
 * the first-order ones in place. */
int wm_limit_fluxes(wm_handle *h, const wm_fields *q, double dt, void *stream);
/* rk3_update(alpha, beta, dt) SC:1974-1984: q = alpha*q_old + beta*(q - dt*R) on interior cells. */
int wm_rk3_update(wm_handle *h, const wm_fields *q, const wm_fields *q_old, double alpha,
                  double beta, double dt, void *stream);
/* enforce_admissible() SC:1907-1911 (a no-op when emergency_repair is 0). */
int wm_enforce_admissible(wm_handle *h, const wm_fields *q, void *stream);
/* update_prims() SC:1913-1917: clamp alpha1, recover u, v, p, copy al_prim <- al. */
int wm_update_prims(wm_handle *h, const wm_fields *q, void *stream);
/* copy_old() SC:1894-1897: q_old <- q for the six conserved arrays (whole padded arrays). */
int wm_copy_old(wm_handle *h, const wm_fields *q, const wm_fields *q_old, void *stream);
/* get_dt() SC:1986-1995: CFL * min over interior cells of the acoustic time step. Blocks until
 * the value is on the host, as the reference does. */
int wm_get_dt(wm_handle *h, const wm_fields *q, double *dt, void *stream);

/* ---- fused forms ---------------------------------------------------------------------------- */
/* One SSP-RK3 stage: apply_bc, compute_fluxes, compute_low_fluxes, limit_fluxes(dt),
 * rk3_update(alpha, beta, dt), enforce_admissible, update_prims -- the body of SC:2030-2055.
 * q_old may be NULL when alpha == 0. In the binary64 form with blends in place (the default) the
 * first-order fluxes are formed where the limiter reads them and are not stored: the WM_WS_FXL /
 * WM_WS_GYL arrays are left as they were, and wm_limit_fluxes after this call returns WM_ERR_STATE
 * until wm_compute_low_fluxes has run. */
int wm_rhs_stage(wm_handle *h, const wm_fields *q, const wm_fields *q_old, double dt, double alpha,
                 double beta, void *stream);
/* One SSP-RK3 step (SC:2033-2059): copy_old, three stages with (alpha, beta) = (0,1), (3/4,1/4),
 * (1/3,2/3), then get_dt. If dt > 0 it is the step's dt; if dt <= 0 the step uses the dt the
 * handle computed at the end of the previous wm_step (or by wm_get_dt / wm_init_dt). The next dt
 * stays on the device; if dt_next != NULL the call also waits for it and stores it there. */
int wm_step(wm_handle *h, const wm_fields *q, const wm_fields *q_old, double dt, double *dt_next,
            void *stream);
/* Compute the time step of the current state on the device (no host wait) for the next wm_step
 * with dt <= 0. */
int wm_init_dt(wm_handle *h, const wm_fields *q, void *stream);

/* Limiter form of the fused stage (wm_rhs_stage, wm_step, wm_run). in_place = 1: the reference's
 * in-place blend sweeps (pp_blend_x/y_flux_kernel, SC:1479-1548) between the passes. in_place = 0:
 * no blend sweeps -- each limiter pass and the combine rebuild the blended face fluxes in registers
 * from the high- and first-order fluxes and the passes' cell factors, bit-identical. The second
 * moves less memory but adds blend arithmetic: the default is in place for WM_PREC_FP64 (whose
 * binary64 pipe is the bound) and rebuilt for WM_PREC_FP32 (blends in binary32); the batched form
 * does the same (in place for binary64, rebuilt for binary32). After a fused stage the workspace's
 * high-order arrays hold the limited fluxes in place form, the unlimited ones otherwise; the closures
 * always blend in place. A face at theta = 1 whose first-order values are all finite keeps its
 * high-order values in every form (the blend's exact value there). */
int wm_set_limiter_sweeps(wm_handle *h, int in_place);

/* Binary32 pre-checks that let cells skip binary64 tests whose outcome they prove -- the limiter's
 * bound solves (the plain form's from binary32 roundings of its binary64 state and fluxes, with a
 * margin covering those roundings), the combine's clamp / floor / NaN / repair tests, and the THINC
 * switch of the binary64 sensors (cator2 of the cell entropies against 0.35, SC:318-325, 1028-1032:
 * binary32 entropies with an error bound, then where that does not settle it the stencil's
 * entropy ratios from binary64 differences of pressure, density and mixture gamma with an error
 * bound, the binary64 pow only where neither settles it) -- on (1, default) or off (0). Results are
 * the same bits either way; off exists to show that. */
int wm_set_prechecks(wm_handle *h, int on);
/* Diagnostic of the THINC switch pre-checks on state q (binary64, any form): for every cell and
 * direction with a full five-cell stencil, the pre-checks (binary32 entropies, then entropy
 * ratios) and the binary64 decision are evaluated from q. *checked counts the stencils, *decided
 * those a pre-check settled, *disagreed those settled differently from the binary64 decision (0
 * when the error bounds hold). No counterpart in the reference. */
int wm_verify_switch_precheck(wm_handle *h, const wm_fields *q, long long *checked, long long *decided,
                              long long *disagreed, void *stream);
/* Diagnostic of the Ducros sensor pre-check on state q (binary64, any form; variant SC's sensor):
 * for both directions of every cell with a full stencil, the binary32 pre-check (from the binary32
 * roundings of u, v, p) and the binary64 decision sigma < 0.01 are evaluated from q. Counts as
 * wm_verify_switch_precheck. No counterpart in the reference. */
int wm_verify_ducros_precheck(wm_handle *h, const wm_fields *q, long long *checked, long long *decided,
                              long long *disagreed, void *stream);
/* Diagnostic of the limiter pre-check (after wm_compute_fluxes and wm_compute_low_fluxes, like
 * wm_limit_fluxes, whose work it does): every bound pass evaluates both the binary32 pre-check that
 * lets cells skip the binary64 bound solve and the solve itself; *decided counts cells the
 * pre-check decided, *disagreed cells where the solve did not return 1 for them (0 when the
 * pre-check's margins hold). No counterpart in the reference. */
int wm_verify_limiter_precheck(wm_handle *h, const wm_fields *q, double dt, long long *decided,
                               long long *disagreed, void *stream);

/* ---- the time loop on the device -------------------------------------------------------------
 * wm_run runs the reference's time loop (SC:2009-2073) for one solve: per step, clamp dt to every
 * save time not yet written and to t_end (SC:2021-2026), one SSP-RK3 step, t += dt, step += 1,
 * dt = the CFL dt of the new state, and a save time ts counts as reached when |t - ts| < dt/2
 * (SC:2066-2073). The steps run inside one CUDA graph (a conditional while node: the step kernels
 * plus two single-thread kernels for the clamps and the loop test) until a save time is reached
 * (sched->hit = its index; the caller writes its output and calls again), t >= t_end - 1e-14
 * (sched->finished), or max_steps steps; one host wait per call. Before the first call set t,
 * t_end, step, the save times and saved[k] = (t >= save_times[k] - 1e-14) (SC:2013). The first
 * call allocates a small device block for the loop state. Not for a stream in capture. */
#define WM_MAX_SAVES 32
typedef struct wm_schedule {
    double t, t_end;
    long long step;
    int nsaves;
    int hit;       /* out: first save index reached by the call's last step, or -1 */
    int finished;  /* out: the loop condition t < t_end - 1e-14 failed */
    double dt;     /* out: the CFL dt of the current state */
    double save_times[WM_MAX_SAVES];
    int saved[WM_MAX_SAVES];
} wm_schedule;
int wm_run(wm_handle *h, const wm_fields *q, const wm_fields *q_old, wm_schedule *sched, long long max_steps,
           void *stream);
/* 1 when wm_run's last call ran as a graph (0: the same kernels, one host wait per step). */
int wm_run_uses_graph(wm_handle *h);

/* ---- batched form: many independent solves, one persistent launch per call -------------------
 * A batch holds up to `capacity` solves in slots. Each solve has its own grid size, cell sizes,
 * equation of state, boundary rules, end time and step budget, and its own cell arrays and
 * workspace (caller-owned device memory of wm_solve_workspace_bytes); all solves of a batch share
 * the scheme (variant, reconstruction, precision, repair, ghost width, CFL). wm_batch_run advances
 * every unfinished solve by up to nsteps SSP-RK3 steps in ONE persistent cooperative kernel launch
 * (replayed from a CUDA graph captured on first use), each with its own device-resident dt
 * (CFL 0.4 of its own state, clamped to its end time). Slots can be filled and cleared between
 * runs (continuous batching). The batched counterpart of the reference's time loop, SC:2009-2059. */
typedef struct wm_batch wm_batch;
typedef struct wm_batch_params {
    int variant, recon, precision, emergency_repair; /* as in wm_params */
    int g;                                           /* ghost layers of every solve */
    double cfl;
    int tile_shape; /* -1: per grid-size class (wm_batch_tile_shape; 32-wide tiles by default),
                       0..3: every grid in tiles of 1x128, 2x64, 4x32 or 8x16 cells */
    int fp64_switches; /* as in wm_params */
    long long spin_limit; /* waits (64 ns naps) a block spends at a grid barrier before the run gives
                             up and sets the batch's error flag; <= 0: 2^26 (about 4 s) */
} wm_batch_params;
typedef struct wm_solve_desc {
    int nx, ny;
    double dx, dy;
    double gamma1, pinf1, gamma2, pinf2;
    int bc[4];
    double t_end;         /* > 0: stop at this time (the last dt is clamped to reach it) */
    long long max_steps;  /* > 0: stop after this many steps */
    wm_fields q, q_old;   /* the solve's ten cell arrays and six step-start arrays */
} wm_solve_desc;
typedef struct wm_solve_status {
    int used, done;
    double t, dt;         /* elapsed time, dt of the next step */
    long long steps;
} wm_solve_status;
size_t wm_solve_workspace_bytes(const wm_batch_params *p, int nx, int ny);
int wm_batch_create(const wm_batch_params *p, int capacity, wm_batch **out);
void wm_batch_destroy(wm_batch *b);
/* Occupy `slot` with a solve whose state is already initialised (the start-up sequence of the
 * reference, SC:1998-2007, e.g. with wm_create + the closures). Time and step count start at 0. */
int wm_batch_set(wm_batch *b, int slot, const wm_solve_desc *d, void *workspace, size_t bytes);
int wm_batch_clear(wm_batch *b, int slot);
/* dt of the slot's first step from its current state (get_dt), on the device. */
int wm_batch_init_dt(wm_batch *b, int slot, void *stream);
int wm_batch_run(wm_batch *b, int nsteps, void *stream);
/* Waits for the stream and copies every slot's status (capacity entries); WM_ERR_STATE if a grid
 * barrier of a run since the last query timed out. Such a run stopped its solves part-way through a
 * phase; the query clears the flag and the barrier counters, so the batch runs again once the
 * caller has put its solves back in a known state (e.g. restored their arrays and scalars). */
int wm_batch_query(wm_batch *b, wm_solve_status *out, void *stream);
/* Barrier wait limit of later runs (as wm_batch_params.spin_limit; <= 0: the default). */
int wm_batch_spin_limit(wm_batch *b, long long limit);
/* Tile shape (0..3) for the grids whose cell count has floor(log2(nx*ny)) == size_class. */
int wm_batch_tile_shape(wm_batch *b, int size_class, int shape);
/* Copy the per-slot scalars (dt accumulator, dt, t, steps, done; 40 bytes per slot) to (write=0)
 * or from (write=1) host memory -- snapshot and restore for measuring runs. */
int wm_batch_scalars(wm_batch *b, void *host, int write, void *stream);
int wm_batch_info(wm_batch *b, int *ntiles, int *grid, int *graph);
/* Per-step dt record (mode 1: log[k] = the dt of the slot's step k) or replay (mode 2: step k
 * uses log[k] instead of its own CFL dt, the end-time clamp still applies; the slot's first dt is
 * log[0] when wm_batch_init_dt runs after this call), for len steps; mode 0 turns it off. `log` is
 * caller-owned device memory of len doubles. Lets two forms of the same solves run on one dt
 * sequence, so that their difference is the arithmetic's alone. */
int wm_batch_dt_log(wm_batch *b, int slot, double *log, long long len, int mode);
/* Phase timing of later runs (enable=1) or none (0). WM_BATCH_PHASES device-time sums in ms (the
 * phases of a stage: ghost fill x, ghost fill y, preparation, sensors, face sweeps, the three
 * limiter passes, combine; then the end-of-step dt phase), summed over stages and steps. */
#define WM_BATCH_PHASES 10
int wm_batch_profile(wm_batch *b, int enable);
int wm_batch_profile_read(wm_batch *b, double *ms, int reset, void *stream);

/* ---- post-processing ------------------------------------------------------------------------ */
/* Schlieren field of the reference's figure (save_png SC:1728-1771, without a plotting library):
 * grad[i*ny + j] = |grad(ar1 + ar2)| over the interior by numpy.gradient's rule on the cell
 * centres (bit-identical to it). xh / yh: the nx-1 / ny-1 device spacings of the interior
 * coordinates, or NULL when every spacing equals x_h0 / y_h0 (numpy's uniform branch).
 * rho_scratch: nx*ny doubles. rgb (optional, ny x 2nx x 3 bytes): the schlieren panel (blue ramp
 * over [1, 2400], alpha1 = 0.5 level in red) beside alpha1 in inverted grey. Needs 2 <= nx <= 65535,
 * ny >= 2. */
int wm_schlieren(const wm_fields *q, int nx, int ny, int g, const double *xh, const double *yh,
                 double x_h0, double y_h0, double *rho_scratch, double *grad, unsigned char *rgb,
                 void *stream);

/* Copy `bytes` from src to dst with the SMs instead of a copy engine: the caller's host <-> device
 * state transfers, which the reference makes with wp.copy of wp.array(host) (SC:1877-1886) and
 * .numpy() (SC:2004-2007). Each side is memory of the current device, managed memory, or
 * page-locked host memory (cudaHostAlloc / cudaHostRegister; torch's pin_memory), read or written
 * in place through its mapped address. Both addresses 16-byte aligned and bytes a multiple of 16.
 * Refused before any launch (WM_ERR_INVALID): a first or last byte of a range that is not in such
 * memory, or not in memory of one kind; a range that runs past its allocation into an adjacent one
 * is the caller's error, as for cudaMemcpyAsync. WM_ERR_CUDA without a usable device.
 * Asynchronous on `stream`. No counterpart in the reference's kernels. */
int wm_copy_state(void *dst, const void *src, long long bytes, void *stream);

/* ---- diagnostics ---------------------------------------------------------------------------- */
/* The integer-pipe binary64 -> binary32 and binary32 -> binary64 conversions and binary64
 * compares / min / max / sign against the hardware ones on n device bit patterns (each read as a
 * binary64, paired with the next one for the compares, and by its low 32 bits as a binary32): the
 * numbers of results that differ (0 expected; NaN counts as equal to NaN). *bad_f32 also counts
 * binary32 pairs hi + lo of the switch pre-check whose lo is not the hardware rounding of x - hi
 * (for |x| in [2^-74, 2^128)) or not 0 (elsewhere). No counterpart in the reference. */
int wm_check_conversions(const unsigned long long *bits, long long n, long long *bad_f32,
                         long long *bad_f64, long long *bad_cmp, void *stream);
/* The binary64 face sweep's reciprocal, quotient and square root (a binary32 seed refined by fused
 * multiply-adds) against IEEE 1/y, x/y and sqrt(x), and its integer-pipe minmods, halving and
 * sign selection against the reference's products on the hardware operations, on n device bit
 * patterns (y: each pattern, x, z, w: the next three; sqrt of |y|, mm2(y, x), mm4(y, x, z, w),
 * y / 2, 0.5 (1 + s) y + 0.5 (1 - s) x for s = +-1). counts[0..2]: results of rcp, div, sqrt
 * that differ from IEEE by more than one unit in the last place, or that are not bit-identical
 * where either result is zero, infinite, subnormal or NaN (0 expected); counts[3..5]: results one
 * unit away; counts[6..9]: mm2, mm4, halving, selection results that are not bit-identical (NaN
 * equal to NaN; 0 expected); counts[10]: pairs of quotients x / y, w / z from one shared reciprocal
 * that are more than four units from IEEE or not bit-identical at special values (0 expected). No
 * counterpart in the reference. */
int wm_check_sweep_arith(const unsigned long long *bits, long long n, long long counts[11], void *stream);
/* Copy workspace array `which` (WM_WS_*) of the padded grid into the caller's device buffer dst
 * (same padded shape, contiguous rows of ny + 2g). */
#define WM_WS_FX 0      /* 7 arrays: high-order x fluxes 0..5 and srcx (after limit_fluxes: blended) */
#define WM_WS_GY 7      /* 7 arrays: y fluxes and srcy */
#define WM_WS_FXL 14    /* 7 arrays: first-order x fluxes and srcxl (written by wm_compute_low_fluxes) */
#define WM_WS_GYL 21    /* 7 arrays: first-order y fluxes and srcyl */
#define WM_WS_THETA 28  /* 3 arrays: cell limiter factor of pass 0, 1, 2 */
#define WM_WS_SIGMA_X 31
#define WM_WS_SIGMA_Y 32
#define WM_WS_COUNT 33
int wm_read_workspace(wm_handle *h, int which, double *dst, void *stream);
/* Read (and optionally reset) the device counters; blocks on the stream. */
int wm_status(wm_handle *h, wm_stats *out, int reset, void *stream);

/* Kernel-group timing with CUDA events recorded on the launching stream around each group of
 * launches (ghost fill, per-cell preparation, face sweeps, limiter, combine). Off by default;
 * while on, every stage records two events per group. wm_profile_read waits for the recorded
 * events and returns, per group, the summed milliseconds and the number of kernel launches. */
#define WM_PROF_BC 0
#define WM_PROF_PREP 1
#define WM_PROF_FACES 2
#define WM_PROF_LIMITER 3
#define WM_PROF_FINAL 4
#define WM_PROF_GROUPS 5
int wm_profile(wm_handle *h, int enable);
int wm_profile_read(wm_handle *h, double ms[WM_PROF_GROUPS], long long launches[WM_PROF_GROUPS],
                    int reset);

/* ---- no-allocation form (no counterpart in the reference) ------------------------------------
 * For callers that cannot allocate device memory -- e.g. a host application that serves all
 * device memory from its own pool and does not let libraries call cudaMalloc, or a loop that must
 * never wait on the allocator. Runs the same stage as wm_rhs_stage in the plain binary64 form
 * (same kernels, same arithmetic, so the same bits), without a handle: the workspace is a device
 * array inside the library, sized for grids of at most WM_STATIC_MAX_CELLS padded cells,
 * (nx + 2g) * (ny + 2g) <= 32768 (about 11.3 MiB, held by every GPU that loads the library until
 * the process exits). Larger grids, and the binary32 precision form (p->precision ==
 * WM_PREC_FP32, whose workspace has another layout), are rejected with WM_ERR_INVALID and a
 * message in wm_last_error(). Calls no cudaMalloc or cudaFree. The first call on a device (and the
 * first after a cudaDeviceReset of it) looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture. All calls on a device
 * share the array and it keeps the last call's contents; calls that overlap on the GPU (other
 * streams or threads) race on it. */
#define WM_STATIC_MAX_CELLS 32768
int wm_rhs_stage_static(const wm_params *p, int nx, int ny, int g, const wm_fields *q,
                        const wm_fields *q_old, double dt, double alpha, double beta, void *stream);

/* Measured FP64 FMA throughput of the current device in FLOP/s (a short on-device loop). */
int wm_probe_fp64_flops(double *flops, void *stream);

#ifdef __cplusplus
}
#endif
#endif
