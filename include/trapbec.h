/*
 * trapbec.h -- C ABI of the GB300 time-stepping engine for the TrapBEC
 * Gross-Pitaevskii solver.
 *
 * The reference program (Fortran 90 + MPI) has no library interface: its hot
 * path is a set of argument-less module procedures acting on module globals
 * (get_rhs, ghost_comm, Psi_norm, Psi_info) and inline loops in `program run`.
 * Each entry point below replaces one of those pieces; the comment on each
 * names the reference lines it stands in for (paths relative to the
 * reference project root).
 *
 * Conventions
 *  - Every function returns an int status: 0 (TRAPBEC_OK) on success, a
 *    positive TRAPBEC_ERR_* code otherwise.  Nothing throws or exits across
 *    the ABI.  trapbec_strerror() maps a code to text; trapbec_last_error()
 *    gives the detail of the last failure on the calling thread.
 *  - Host arrays are owned by the caller and copied at set/get time.  Device
 *    buffers are owned by the context.
 *  - Complex arrays are interleaved (re, im) pairs, layout-compatible with
 *    Fortran complex(c_float_complex) / complex(c_double_complex) and C99
 *    float _Complex / double _Complex.  Their element type is the context's
 *    precision (TRAPBEC_FP32 -> float pairs, TRAPBEC_FP64 -> double pairs).
 *  - Array order is the reference's Psi(k,j,i): z fastest, then y, then x.
 *  - One host thread per context; each context owns one CUDA stream and all
 *    of its calls are ordered on it.  get/diag calls synchronise.  The
 *    overlapped host copies (trapbec_set_psi_async, trapbec_get_psi_async)
 *    run on two more streams of the context, ordered against it by events.
 *  - All quantities are in the reference's units (healing-length units with
 *    g = mu = 1/2 folded into the equation, finite_diff.f90:23-27,128-132).
 */
#ifndef TRAPBEC_H
#define TRAPBEC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TRAPBEC_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum trapbec_status {
  TRAPBEC_OK = 0,
  TRAPBEC_ERR_ARG = 1,         /* bad argument / parameter combination      */
  TRAPBEC_ERR_CUDA = 2,        /* a CUDA runtime or driver call failed      */
  TRAPBEC_ERR_NOMEM = 3,       /* device or host allocation failed          */
  TRAPBEC_ERR_STATE = 4,       /* call not valid in the current state       */
  TRAPBEC_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up        */
  TRAPBEC_ERR_NONFINITE = 6,   /* NaN/Inf detected in psi by a reduction    */
  TRAPBEC_ERR_IO = 7,          /* file could not be read or written         */
  TRAPBEC_ERR_UNSUPPORTED = 8, /* option not built for this configuration   */
  TRAPBEC_ERR_PARSE = 9,       /* cparam.local text could not be parsed     */
  TRAPBEC_ERR_NODEVICE = 10    /* no CUDA device / driver available         */
};

/* ---- enumerations mirroring the cparam.local string parameters ---------- */
enum trapbec_boundaries {      /* cparam.local `boundaries`, ghost.f90:53-60 */
  TRAPBEC_BC_ZERO = 0,
  TRAPBEC_BC_SOLID = 1,
  TRAPBEC_BC_PERIODIC = 2
};

enum trapbec_potential {       /* cparam.local `potential`, finite_diff.f90:29-124 */
  TRAPBEC_POT_ZERO = 0,
  TRAPBEC_POT_HARMONIC = 1,
  TRAPBEC_POT_HARMONIC_RING = 2,
  TRAPBEC_POT_HARMONIC_RING2 = 3,
  TRAPBEC_POT_BARRIER = 4,
  TRAPBEC_POT_BOX_TRAP = 5,
  TRAPBEC_POT_CHANNEL = 6,
  TRAPBEC_POT_QUARTIC = 7,
  TRAPBEC_POT_SPHERE = 8,
  TRAPBEC_POT_MOBIUS = 9,      /* reads the Trap array (built as mesh_init builds it, or trapbec_set_trap) + marker */
  TRAPBEC_POT_ARRAY = 10       /* plain Trap array, no marker (new)            */
};

enum trapbec_precision { TRAPBEC_FP32 = 0, TRAPBEC_FP64 = 1 };

enum trapbec_layout {
  TRAPBEC_LAYOUT_INTERIOR = 0, /* Psi(1:nz,1:ny,1:nx)                         */
  TRAPBEC_LAYOUT_GHOSTED = 1   /* Psi(-2:nz+3,-2:ny+3,-2:nx+3), initial.f90:16 */
};

enum trapbec_field {           /* output-time diagnostic fields               */
  TRAPBEC_FIELD_VELOCITY = 0,  /* vel of get_phase, diagnostic.f90:27-48       */
  TRAPBEC_FIELD_QPRESSURE = 1  /* qpressure of get_qpressure, diagnostic.f90:50-84 */
};

enum trapbec_imag_variant {
  TRAPBEC_IMAG_REF_EULER = 0,  /* Psi = Psi + dt*0.5*rhs, no renorm, run.f90:19-35 */
  TRAPBEC_IMAG_RK3_RENORM = 1  /* low-storage RK3 in imaginary time + FP64
                                  renormalisation + |dE| stop (new)           */
};

enum trapbec_scalar {          /* run-time changeable scalars (trapbec_set_scalar) */
  TRAPBEC_SCALAR_OMEGA_Z = 0,
  TRAPBEC_SCALAR_DT_RE = 1,
  TRAPBEC_SCALAR_DT_IM = 2,
  TRAPBEC_SCALAR_GAMMA = 3,
  TRAPBEC_SCALAR_T = 4,
  TRAPBEC_SCALAR_ADVECTIVE_VX = 5,
  TRAPBEC_SCALAR_NORM_TARGET = 6
};

/* ---- parameters: the hot-path subset of cparam.local ------------------- */
/* cparam.local:2-44 and mpi_var.f90:147-156.  Field names follow the
 * Fortran parameter names.  nprocx/nprocy do not split the device domain
 * (one GPU holds the whole grid); they only reproduce the coordinate
 * arithmetic of an MPI run on an nprocx x nprocy process grid
 * (initial.f90:34-42), so results can be compared with such a run.        */
typedef struct trapbec_params {
  int32_t nx, ny, nz;          /* Nx, Ny, Nz: global grid                     */
  int32_t nprocx, nprocy;      /* virtual process grid (default 1,1)          */
  int32_t precision;           /* trapbec_precision                           */
  int32_t boundaries;          /* trapbec_boundaries                          */
  int32_t periodicz;           /* logical periodicz                           */
  int32_t two_dim;             /* logical two_dim                             */
  int32_t potential;           /* trapbec_potential                           */
  int32_t lbeam;               /* logical lbeam                               */
  int32_t winding_number;      /* integer winding_number                      */
  double lx, ly, lz;           /* Lx, Ly, Lz                                  */
  double dt_re, dt_im;         /* complex dt                                  */
  double gamma;                /* dissipation, applied as dt*(1-i*gamma)      */
  double harm_wx, harm_wy, harm_wz;
  double potential_off;        /* pot = 0 once t > potential_off              */
  double wbeam;                /* laser width                                 */
  double advective_vx;         /* moving frame velocity                       */
  double omega_z;              /* rotating frame angular velocity             */
  double t_spindown;           /* rotation switched off once t >= t_spindown  */
  double ring_rad;             /* vortex ring radius (initial states)         */
  int32_t vor_ring_count;      /* number of random rings (initial states)     */
  int32_t reserved[7];         /* zero                                        */
} trapbec_params;

/* Fill *p with the defaults of the shipped cparam.local (cparam.local:2-44)
 * but precision FP64, 64^3, 'zero' boundaries, 'harmonic' potential.       */
int trapbec_params_default(trapbec_params* p);

/* Parse cparam.local text (Fortran declarations `type :: name=value, ...`)
 * into *p, starting from the current contents of *p.  Unknown names that
 * the hot path needs are errors; names the hot path ignores are accepted.
 * errbuf (may be NULL) receives a one-line message on failure.
 * Replaces the compile-time include of cparam.local (cdata.f90:3).        */
int trapbec_params_parse(const char* text, trapbec_params* p, char* errbuf, size_t errlen);

/* ---- context ------------------------------------------------------------ */
typedef struct trapbec_ctx trapbec_ctx;

/* Allocate device state for one grid on the current CUDA device.
 * Replaces mpi_setup + mesh_init's allocations and coordinates
 * (mpi_var.f90:14-43, initial.f90:16-42) and ghost_init (ghost.f90:16-26). */
int trapbec_create(const trapbec_params* p, trapbec_ctx** out);
void trapbec_destroy(trapbec_ctx* ctx);

/* Copy psi host->device / device->host.  layout: trapbec_layout.  For the
 * GHOSTED layout only the interior is read on set; on get the ghost cells
 * are filled the way ghost_comm leaves them (ghost.f90:27-192).            */
int trapbec_set_psi(trapbec_ctx* ctx, const void* psi, int layout);
int trapbec_get_psi(trapbec_ctx* ctx, void* psi, int layout);

/* Set the Trap(1:nz,1:ny,1:nx) array (cdata.f90:10) used by the 'mobius' and
 * 'array' potentials; values are FP64 and converted to the context precision.
 * For 'mobius' without a call to this function, the first step builds the
 * Trap on the device as mesh_init does (initial.f90:159-198: a clamped sum of
 * 200 x 200 Gaussians of the strip table per cell, inverted about the maximum
 * over the grid); 'array' needs this call.                                  */
int trapbec_set_trap(trapbec_ctx* ctx, const double* trap);

/* Fill psi with one of the reference's initial states (initial.f90:58-157
 * and the helpers :202-870), evaluated on the device.  Random draws use a
 * seeded counter-based generator instead of the clock-seeded Fortran RNG
 * (mpi_var.f90:183-209).  Also accepts the states of the workload set:
 * "tf_vortex_line", "tf_vortex_ring" (see trapbec_init_args).              */
typedef struct trapbec_init_args {
  uint64_t seed;               /* RNG seed                                    */
  double amp;                  /* overall amplitude (new states)              */
  double r_tf2[3];             /* TF inverse radii^2 per axis (new states)    */
  double ring_radius;          /* ring radius (tf_vortex_ring)                */
  double core2;                /* Pade core parameter (rho^2 + core2)         */
  double noise_amp;            /* phase-noise amplitude (tf_vortex_ring)      */
  double reserved[4];
} trapbec_init_args;
int trapbec_init_state(trapbec_ctx* ctx, const char* init_cond, const trapbec_init_args* args);

/* Evaluate rhs = get_rhs(psi) for the current psi without stepping and copy
 * it to host memory (interior layout).  Replaces finite_diff.f90:8-136.    */
int trapbec_get_rhs(trapbec_ctx* ctx, void* rhs_out);

/* Advance nsteps real-time low-storage RK3 steps with dt*(1-i*gamma).
 * *t_inout is the simulation time t (cdata.f90:18), advanced by Re(dt) per
 * step.  Replaces run.f90:42-57 (one call per `shots` block).            */
int trapbec_step_rt(trapbec_ctx* ctx, int nsteps, double* t_inout);

/* Overlapped host copies: the state of the next `shots` block goes up and
 * the last block's result comes back while the GPU steps, the way run.f90
 * would overlap its restart read and its var####.dat output (run.f90:45-66,
 * output.f90:64-75) with the next block if the copies were asynchronous.
 * Interior layout only; the host arrays should be pinned for the copies to
 * run concurrently with the steps.
 *  trapbec_set_psi_async : queue `psi`: it is copied to the device at once on
 *      a copy stream and becomes the state at the start of the next
 *      time-stepping call (trapbec_step_rt / _async, trapbec_step_imag);
 *      until then the current state is unchanged and may still be read.
 *      trapbec_set_psi, trapbec_init_state and trapbec_read_restart replace a
 *      queued state.  `psi` must stay unchanged until trapbec_synchronize.
 *  trapbec_get_psi_async : snapshot the current state on the device (after
 *      all queued steps) and copy the snapshot to `psi` on a copy stream;
 *      `psi` holds it after trapbec_wait_psi or trapbec_synchronize.
 *  trapbec_step_rt_async : trapbec_step_rt that returns once the steps are
 *      queued (*t_inout advanced already); their kernel time and a timed-out
 *      device wait are reported by trapbec_synchronize or by the next call
 *      that waits (trapbec_diag, trapbec_get_psi, trapbec_step_rt, ...).
 *  trapbec_wait_psi      : wait for the copy of the last trapbec_get_psi_async.
 *  trapbec_synchronize   : wait for all queued steps and copies.
 *  trapbec_diag_async    : queue trapbec_diag's reduction of the current state
 *      (after all queued steps) without waiting, so that the next block of
 *      steps can be queued behind it; trapbec_diag_wait returns its values
 *      (TRAPBEC_ERR_STATE if none is pending, TRAPBEC_ERR_TIMEOUT if a
 *      device wait of the steps before it timed out).                    */
int trapbec_set_psi_async(trapbec_ctx* ctx, const void* psi, int layout);
int trapbec_get_psi_async(trapbec_ctx* ctx, void* psi, int layout);
int trapbec_step_rt_async(trapbec_ctx* ctx, int nsteps, double* t_inout);
int trapbec_wait_psi(trapbec_ctx* ctx);
int trapbec_synchronize(trapbec_ctx* ctx);

/* Imaginary-time relaxation.
 *  REF_EULER : nsteps of Psi = Psi + dt*0.5*rhs (run.f90:19-35); *stat_out
 *              receives the last norm ratio intPsi2/intPsi2_old (run.f90:23).
 *  RK3_RENORM: up to nsteps RK3 steps with real step Re(dt); after each step
 *              psi is renormalised to the norm target (FP64) and the FP64
 *              energy is formed; stops when |E_n - E_{n-1}| <= tol*|E_n|
 *              (or on the absolute test of trapbec_set_imag_stop).
 *              *stat_out receives the last |dE|/|E| (absolute test: the last
 *              |dE| times the energy scale).  Every energy the test compares
 *              comes from the same fused evaluation (the incoming state's
 *              energy reduced in stage 1), including the final state's.
 * *steps_done receives the number of steps taken.                          */
int trapbec_step_imag(trapbec_ctx* ctx, int nsteps, int variant, double tol,
                      int* steps_done, double* stat_out);

/* Stop test of the RK3_RENORM relaxation (new; the reference relaxes a fixed
 * number of steps, run.f90:20-33).
 *  TRAPBEC_STOP_REL (default):  |E_n - E_{n-1}| <= tol * |E_n|
 *  TRAPBEC_STOP_ABS:            |E_n - E_{n-1}| * energy_scale < tol
 *  TRAPBEC_STOP_ABS_PER_NORM:   |E_n - E_{n-1}| / N * energy_scale < tol
 * E is the energy trapbec_diag reports and N the norm target (reference
 * units); energy_scale > 0 converts into the unit the tolerance is stated
 * in.  For a trap-units problem (x = a x', t = a^2 t', phi = sqrt(mu/g) psi,
 * a = 1/sqrt(2 mu)) the total energy takes (mu/g) a^3 2 mu and the energy
 * per particle (ABS_PER_NORM) takes 2 mu.  Applies to later
 * trapbec_step_imag calls.                                                  */
enum trapbec_imag_stop { TRAPBEC_STOP_REL = 0, TRAPBEC_STOP_ABS = 1, TRAPBEC_STOP_ABS_PER_NORM = 2 };
int trapbec_set_imag_stop(trapbec_ctx* ctx, int mode, double energy_scale);

/* Diagnostics of the current psi.  intpsi2/maxpsi/minpsi/meanpsi follow
 * Psi_norm and Psi_info (diagnostic.f90:7-25) but are summed in FP64 with
 * compensation.  The rest are new (FP64): energy, chemical potential and
 * their pieces, in reference units with the cell volume dV = hx*hy*hz.     */
typedef struct trapbec_diag_out {
  double intpsi2;              /* sum |psi|^2 (no dV), Psi_norm               */
  double maxpsi, minpsi, meanpsi; /* Psi_info                                 */
  double norm;                 /* dV * sum |psi|^2                            */
  double energy;               /* dV * sum[-1/2 Re psi* lap + 1/2 pot|psi|^2
                                         + 1/4 |psi|^4 - 1/2 Re psi* rot]     */
  double mu;                   /* <psi|H|psi>/<psi|psi> without the -1/2 shift */
  double kinetic, potential, interaction, rotation; /* raw sums (no dV)       */
  int32_t nonfinite;           /* 1 if any NaN/Inf was seen                    */
  int32_t reserved;
} trapbec_diag_out;
int trapbec_diag(trapbec_ctx* ctx, trapbec_diag_out* out);
/* trapbec_diag queued without waiting, and its result (see the overlapped
 * host copies above).                                                      */
int trapbec_diag_async(trapbec_ctx* ctx);
int trapbec_diag_wait(trapbec_ctx* ctx, trapbec_diag_out* out);

/* Bounded waits of the tiled stage kernels (no counterpart in the reference).
 * Every wait of a launch for its TMA data gives up after `limit`
 * microseconds (0 = the default, 2 s), records TRAPBEC_ERR_TIMEOUT, lets the copies in
 * flight land and returns; the call then returns TRAPBEC_ERR_TIMEOUT and the
 * context stays usable (psi is not meaningful after it).  inject = 1 is a
 * test hook: every wait then waits for an mbarrier phase that nothing
 * completes, so the timeout path runs without any fault.                   */
int trapbec_set_wait_limit(trapbec_ctx* ctx, uint32_t limit, int inject);

/* Forcing (force_random_points, force.f90:12-54): multiply psi by a Pade
 * vortex sqrt(r^2 (c1 + c2 r^2) / (1 + c3 r^2 + c2 r^4)) e^{i dir theta},
 * straight along z through (x0, y0); dir = +1 or -1.
 * trapbec_force_vortex takes the position and sign; trapbec_force_random_points
 * draws them as the reference does (x0 ~ U[-Lx/4, Lx/4], y0 ~ U[-Ly/4, Ly/4],
 * dir = -1 if U[0,1] < 0.5 else +1) from a counter-based stream: draw number
 * `draw` of `seed` is reproducible on its own (the reference's draws come from
 * gfortran's random_number and cannot be reproduced).  drawn[3] (optional)
 * receives (x0, y0, dir).                                                   */
int trapbec_force_vortex(trapbec_ctx* ctx, double x0, double y0, double dir);
int trapbec_force_random_points(trapbec_ctx* ctx, uint64_t seed, uint64_t draw, double drawn[3]);

/* Output-time diagnostics of the current psi, written to host memory as
 * 3 x (nx*ny*nz) reals of the context precision, component-major
 * ([3][nx][ny][nz], i.e. Fortran vel(k,j,i,c)):
 *  velocity : 6th-order first derivative of atan2(Im, Re) along x, y, z
 *             (get_phase, diagnostic.f90:27-48; no phase unwrapping)
 *  qpressure: 2nd-order gradient of the 4th-order Laplacian of |psi|
 *             (get_qpressure, diagnostic.f90:50-84)
 * Both read the ghosted state as ghost_comm leaves it (edges/corners 0).   */
int trapbec_get_velocity(trapbec_ctx* ctx, void* vel_out);
int trapbec_get_qpressure(trapbec_ctx* ctx, void* qp_out);

/* Change a scalar between calls (trapbec_scalar), e.g. an Omega ramp.     */
int trapbec_set_scalar(trapbec_ctx* ctx, int which, double value);
int trapbec_get_scalar(trapbec_ctx* ctx, int which, double* value);

/* Select the stage kernel: 0 = automatic (tiled TMA kernel where the grid
 * allows it), 1 = simple per-cell kernel, 2 = tiled kernel (error if the
 * grid does not allow it).  tile_z/tile_y pick a built tile shape for every
 * launch (tile_z = -(i+1): built shape number i); 0, 0 restores the defaults:
 * the first built shape that fits the grid (shape 0, 128 x 8 tiles in FP32,
 * where it does) for reductions and imaginary time, the real-time shape
 * (64 x 32 tiles in FP32) for the plain real-time stages where it fits.     */
int trapbec_set_kernel(trapbec_ctx* ctx, int kind, int tile_z, int tile_y);

/* Tile shape the tiled kernel runs with: of the plain real-time stages
 * (real_time = 1) or of every other launch (real_time = 0).  0, 0 when those
 * launches use the per-cell kernel.                                         */
int trapbec_get_tile_shape(trapbec_ctx* ctx, int real_time, int* tile_z, int* tile_y);

/* Work order of the tiled kernel (0 = automatic).  chunk > 0: each CTA takes
 * a contiguous range of work units in (z-tile, x-chunk, y-tile, x) order with
 * chunks of `chunk` x-planes (nx: tile-major).  chunk < 0: the strided order,
 * segments of -chunk x-planes in (x-chunk, z-tile, y-tile) order dealt
 * round-robin over the CTAs, so neighbouring tiles are streamed over the same
 * x-range at the same time and their shared ghost rows are served from L2 on
 * grids of many more tiles than CTAs.  trapbec_autotune reports either.     */
int trapbec_set_chunk(trapbec_ctx* ctx, int chunk);

/* Form of the real-time RK3 step (run.f90:42-57) on the tiled kernel.
 * TRAPBEC_RK3_THREE_STAGE (default): three full stages, each storing w and psi.
 * TRAPBEC_RK3_COMPENSATED (FP32 contexts): the three stages with a
 *   compensated state.  Each stage's update psi' = psi + B w is formed as an
 *   exact two-term sum psi' + lo' = psi + (B w + lo), where lo is a second
 *   complex FP32 array (allocated by this call) holding the rounding
 *   remainder of the previous update.  Increments below half an FP32 ulp of
 *   psi, which the plain FP32 update loses (a nearly stationary state drifts
 *   in norm by ~1e-6-1e-5 over 1000 steps), accumulate in lo instead.  The
 *   stencil reads psi alone; get_psi and trapbec_diag report psi.  Costs 48
 *   more bytes of HBM traffic per grid point and step (128 instead of 80).
 *   Runs on two-row tile shapes with harmonic or no potential and a rotating
 *   or no frame; other set-ups make trapbec_step_rt return
 *   TRAPBEC_ERR_UNSUPPORTED.  lo restarts from zero whenever psi is changed
 *   by anything other than a compensated step (set_psi, init_state,
 *   imaginary time, forcing, another form).
 * TRAPBEC_RK3_DEFERRED: stage 1 stores w1 only and stage 2 forms
 *   psi1 = psi0 + w1/3 from ghosted boxes of psi0 and w1 with the same FMA,
 *   writing w2 to a second w buffer (allocated by this call): 72 instead of
 *   80 bytes of HBM traffic per grid point and step, bit-identical results.
 *   It applies on tile shapes whose shared memory holds both boxes and where
 *   the plain stage variant runs (harmonic or no potential, rotation or no
 *   frame term); elsewhere the step keeps three stages.  On GB300 it measured
 *   slower than three stages on the best tile shape.
 * TRAPBEC_RK3_PSI_DIFF (FP32 and FP64 contexts): no w array is stored.  The
 *   two psi arrays hold the last two stage values, and each stage recovers
 *   the w of the stage before it from their difference: stage 1 stores psi1
 *   only, stage 2 takes w1 = 3 (psi1 - psi0) and writes psi2 over psi0,
 *   stage 3 takes w2 = psi2 - psi1 and writes psi3 over psi1.  The same RK3
 *   scheme, with w rounded differently: the recovered w carries the rounding
 *   of the psi update it came from, so results agree with three stages to
 *   the rounding of a few ulps per step (FP64: 1e-12 relative after hundreds
 *   of steps), not bit for bit.  64 instead of 80 bytes of HBM traffic per
 *   grid point and step.  It applies where the plain stage variant runs on
 *   the tiled kernel (harmonic or no potential, rotation or no frame term);
 *   elsewhere the step keeps three stages.
 * trapbec_get_stage_form: *form = the form the next trapbec_step_rt takes
 * (THREE_STAGE where a requested deferred or psi-difference form cannot run). */
enum trapbec_rk3_form {
  TRAPBEC_RK3_THREE_STAGE = 0,
  TRAPBEC_RK3_DEFERRED = 1,
  TRAPBEC_RK3_COMPENSATED = 2,
  TRAPBEC_RK3_PSI_DIFF = 3
};
int trapbec_set_stage_form(trapbec_ctx* ctx, int form);
int trapbec_get_stage_form(trapbec_ctx* ctx, int* form);

/* Autotune the tiled kernel of the real-time stages for this grid: time every
 * built tile shape and a few chunk lengths over `steps` RK3 steps each on the
 * current state (which is saved and restored), keep the fastest for the plain
 * real-time stages (reductions and imaginary time keep their shape).
 * *tile_z, *tile_y, *chunk (may be NULL) receive the choice, *ms_per_step its
 * time.  Results are cached per process for identical grids.               */
int trapbec_autotune(trapbec_ctx* ctx, int steps, int* tile_z, int* tile_y, int* chunk, double* ms_per_step);

/* Kernels launched by this context since creation (for launch accounting). */
int trapbec_launch_count(trapbec_ctx* ctx, int64_t* count);

/* Device time of the stage kernels of the last trapbec_step_* call, ms,
 * measured with events on the context stream around the kernels.          */
int trapbec_last_kernel_ms(trapbec_ctx* ctx, double* ms);

/* ---- output / restart layout (output.f90:48-118, initial.f90:796-818) --- */
/* Write data/proc000/var####.dat (one unformatted record: coords(2) int32,
 * Lx, Ly, Lz, t, Psi interior) or imag_var####.dat, and the 3-record restart
 * file var.dat (itime+1, t, Psi).  Real kind follows the precision.        */
int trapbec_write_var(trapbec_ctx* ctx, const char* datadir, int itime, int shots,
                      double t, int imaginary);
int trapbec_write_restart(trapbec_ctx* ctx, const char* datadir, int itime, double t);
/* The same two files for a state already in host memory (interior layout,
 * the precision of *p), e.g. one read back by trapbec_get_psi_async, so that
 * the files are written while the next steps run.                         */
int trapbec_write_var_host(const trapbec_params* p, const char* datadir, int itime, int shots, double t,
                           int imaginary, const void* psi);
int trapbec_write_restart_host(const trapbec_params* p, const char* datadir, int itime, double t, const void* psi);
/* Page-locked host memory for the overlapped copies (cudaMallocHost).      */
int trapbec_host_alloc(size_t bytes, void** out);
void trapbec_host_free(void* p);
/* Write data/proc000/vel##.dat or qpress##.dat (one record: coords(2) int32,
 * the field as vel(1:nz,1:ny,1:nx,3)), as var_print does when vel_print /
 * qpress_print are set (output.f90:80-91); ## is itime/shots in i2.2.      */
int trapbec_write_field(trapbec_ctx* ctx, const char* datadir, int itime, int shots, int which);
/* Read var.dat (proc000, or proc00 as the reference reader expects).        */
int trapbec_read_restart(trapbec_ctx* ctx, const char* datadir, int* nstart, double* t);
int trapbec_write_dims(const trapbec_params* p, const char* datadir);
int trapbec_write_timing(const trapbec_params* p, const char* datadir,
                         double time_per_timestep, double tot_comm_time);

/* ---- statistics of a device-resident psi without allocating ------------ */
/* This entry point has no counterpart in the reference.  It returns, for a
 * psi the caller already holds in device memory, the four values trapbec_diag
 * reports as intpsi2, maxpsi, minpsi and meanpsi (Psi_norm and Psi_info), and
 * it allocates nothing: no cudaMalloc, cudaFree or allocating library call.
 * It is meant for callers that cannot let a library allocate device memory,
 * such as hosts that reserve a GPU's memory up front in their own pool and
 * must not have memory taken behind the pool's back or their streams stalled
 * by the device synchronisation an allocation may cause.
 *  psi       device pointer to ncells complex values of `precision`, aligned
 *            to one complex value (8 bytes FP32, 16 bytes FP64)
 *  ncells    1 .. 268435456 (16384 blocks x 16384 cells; larger counts are
 *            rejected with TRAPBEC_ERR_ARG because the fixed scratch would
 *            not hold their partial sums)
 *  stats     device pointer to 4 doubles (8-byte aligned): intpsi2, maxpsi,
 *            minpsi, meanpsi
 *  stream    cudaStream_t to launch on (NULL: the legacy default stream)
 * Null or misaligned pointers, an unknown precision and out-of-range counts
 * return TRAPBEC_ERR_ARG before anything touches the GPU.
 * The work is queued on `stream`; read `stats` after synchronising with it.
 * Scratch space is a 512 KiB array in the library's device memory, present on
 * every GPU that loads the library until the process exits.  The driver maps
 * it when the library's device code is loaded into a context: by default at
 * the first call of this function on a device (at library load under
 * CUDA_MODULE_LOADING=EAGER), which may also synchronise the device.  A host
 * that reserves nearly all of a GPU's memory for its own pool should make one
 * call before reserving it.  The first call on a device (and the first after
 * the device's context was reset or re-created) looks up that array's address
 * in the current context; make that call before starting any stream capture.
 * All calls on a device share the one array, so calls that overlap on the GPU
 * (different streams, or different host threads) race and must be serialised
 * by the caller.                                                            */
int trapbec_psi_stats_noalloc(const void* psi, int64_t ncells, int precision, double* stats, void* stream);

/* ---- batched imaginary-time ground states (new) ------------------------- */
/* Many independent instances (own grid size, trap, g via units, Omega) are
 * relaxed together: each RK3 stage is one persistent launch over the work
 * of all unconverged instances; the step loop is captured in a CUDA graph. */
typedef struct trapbec_batch trapbec_batch;
int trapbec_batch_create(int ninst, const trapbec_params* params, trapbec_batch** out);
void trapbec_batch_destroy(trapbec_batch* b);
int trapbec_batch_set_psi(trapbec_batch* b, int inst, const void* psi);
int trapbec_batch_get_psi(trapbec_batch* b, int inst, void* psi);
/* Relax all instances: up to max_steps steps each, convergence when
 * |dE|/|E| <= tol (or the absolute test of trapbec_batch_set_imag_stop).
 * check_every = steps per graph replay between host checks.
 * steps_out[ninst], energy_out[ninst], mu_out[ninst] (may be NULL).        */
int trapbec_batch_solve_imag(trapbec_batch* b, int max_steps, double tol, int check_every,
                             int* steps_out, double* energy_out, double* mu_out);
/* Stop test of later solves (trapbec_imag_stop, as trapbec_set_imag_stop):
 * TRAPBEC_STOP_ABS stops instance i when |E_n - E_{n-1}| * energy_scale[i]
 * < tol, TRAPBEC_STOP_ABS_PER_NORM when |E_n - E_{n-1}| / N_i *
 * energy_scale[i] < tol; energy_scale may be NULL (a scale of 1 for every
 * instance), and TRAPBEC_STOP_REL ignores it.                              */
int trapbec_batch_set_imag_stop(trapbec_batch* b, int mode, const double* energy_scale);
/* Fill instance `inst` with a Thomas-Fermi state ("thomas_fermi", from the
 * instance's harm_w*) or a workload state ("tf_noise", "tf_vortex_line",
 * "tf_vortex_ring"; see trapbec_init_state).                                */
int trapbec_batch_init_state(trapbec_batch* b, int inst, const char* init_cond, const trapbec_init_args* args);
/* Device time of the last solve (ms, events around the whole loop), the tile
 * shape the autotuner chose, and the kernels launched so far.               */
int trapbec_batch_stats(trapbec_batch* b, double* solve_ms, int* tile_z, int* tile_y, int64_t* launches);
/* Status of instance `inst` after a solve: out[0..9] = renormalisation factor
 * pending, previous energy, last |dE|/|E|, energy, chemical potential, norm
 * before renormalisation, norm target, steps, converged flag, non-finite flag. */
int trapbec_batch_status(trapbec_batch* b, int inst, double* out10);

/* ---- measurement helper (no counterpart in the reference) -------------- */
/* The rate (instructions per second) at which the current GPU retires FP64
 * fused multiply-adds: independent FMA chains on every SM, one timed launch
 * after a warm-up, CUDA events.  The compute roofline of the FP64 stage
 * kernels, which GB300's FP64 pipe bounds before HBM does.  Allocates and
 * frees a small output buffer; synchronises the device.                    */
int trapbec_fp64_fma_rate(double* ops_per_second);

/* ---- errors ------------------------------------------------------------- */
const char* trapbec_strerror(int code);
const char* trapbec_last_error(void);
int trapbec_abi_version(void);
/* sizeof of the ABI structs (0: trapbec_params, 1: trapbec_diag_out,
 * 2: trapbec_init_args), so bindings can check their mirrors.            */
int trapbec_abi_struct_size(int which);

#ifdef __cplusplus
}
#endif
#endif /* TRAPBEC_H */
