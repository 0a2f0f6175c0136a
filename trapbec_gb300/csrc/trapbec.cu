// trapbec.cu -- context, orchestration and the C ABI of libtrapbec.
//
// One context = one grid on one GPU, one CUDA stream.  Device layout: psi,
// w and the potential are interior-only arrays in the reference's order
// Psi(k,j,i) (z fastest); the ghost planes of the reference (initial.f90:16,
// ghost.f90) are not stored: the stage kernels produce ghost values by index
// mapping (per-cell kernel) or by TMA out-of-bounds fill plus a fix-up of
// the boundary tiles (tiled kernel).  psi is double-buffered because a fused
// stage reads neighbours of psi while writing the updated psi.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/trapbec.h"
#include "common.cuh"
#include "host_util.h"
#include "host_coords.h"
#include "kernels_init.cuh"
#include "kernels_simple.cuh"
#include "tiled_api.h"
#include "imag_ctrl.cuh"
#include "kernels_diag.cuh"

using namespace tb;

// ---------------------------------------------------------------- errors --
namespace tbh {
static thread_local std::string g_err;
void set_error(const std::string& m) { g_err = m; }
const char* get_error() { return g_err.c_str(); }
}  // namespace tbh
using tbh::set_error;

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                      \
      return (e_ == cudaErrorNoDevice || e_ == cudaErrorInsufficientDriver)               \
                 ? TRAPBEC_ERR_NODEVICE                                                   \
                 : (e_ == cudaErrorMemoryAllocation ? TRAPBEC_ERR_NOMEM : TRAPBEC_ERR_CUDA); \
    }                                                                                     \
  } while (0)

#define CKL()                                                                             \
  do {                                                                                    \
    cudaError_t e_ = cudaGetLastError();                                                  \
    if (e_ != cudaSuccess) {                                                              \
      set_error(std::string("kernel launch: ") + cudaGetErrorString(e_));                 \
      return TRAPBEC_ERR_CUDA;                                                            \
    }                                                                                     \
  } while (0)

// ---------------------------------------------------------------- context --
struct AsyncDiag {       // what trapbec_diag_async leaves in host memory
  double red[NRED];      // the reduction's NRED values
  int err;               // the tiled kernel's error flag at that point of the stream
};

// Store the finalised reduction and the error flag straight into the
// page-locked slot (mapped into the device's address space): a copy-engine
// transfer on the context stream would queue behind a large read-back on the
// copy stream in the same direction and hold the next steps back.
__global__ void publish_diag_kernel(const double* __restrict__ red_out, const int* __restrict__ d_err,
                                    AsyncDiag* __restrict__ dst) {
  const int i = threadIdx.x;
  if (i < NRED) dst->red[i] = red_out[i];
  if (i == NRED) dst->err = *d_err;
  __threadfence_system();
}

struct trapbec_ctx {
  trapbec_params p;
  int prec = TRAPBEC_FP64;
  size_t n = 0, esz = 0, rsz = 0;   // cells, complex and real element sizes
  int dev = 0, nsm = 0;
  cudaStream_t st = nullptr;
  void* psi[2] = {nullptr, nullptr};
  int cur = 0;
  void* w = nullptr;
  void* w2 = nullptr;                  // second w buffer of the deferred real-time form (allocated on request)
  double force_args[3] = {0.0, 0.0, 1.0};   // (x0, y0, dir) of the next forced vortex
  void *xx = nullptr, *yy = nullptr, *zz = nullptr, *px = nullptr, *py = nullptr, *pz = nullptr;
  void* trap_user = nullptr;   // Trap array set by the caller (context precision)
  void* trap_eff = nullptr;    // evaluated potential (POT_ARR)
  bool pot_valid = false;
  double pot_t = -1.0;
  double* red = nullptr;       // [NRED][red_cap] block partials
  int red_cap = 0;
  double* red_out = nullptr;   // NRED finalised values
  double* host_red = nullptr;  // pinned NRED
  ImagCtrl* ctrl = nullptr;    // device control block of the imaginary-time loop
  ImagCtrl* host_ctrl = nullptr;
  double t = 0.0;
  double dt_re = 0, dt_im = 0, gamma = 0, omega = 0, vx = 0;
  double norm_target = -1.0;
  bool norm_user = false;              // norm_target set by the caller (else derived per state)
  double intpsi2_old = 1.0;    // run.f90:23 ratio state
  bool ctrl_init = false;
  int kernel_kind = 0, tile_z = 0, tile_y = 0;
  int64_t launches = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double last_ms = 0.0;
  std::vector<double> hxx, hyy, hzz;   // coordinates as double (exact copies of T values)
  TiledPlan plan;                      // tiled-kernel plan (tensor maps, tile shape) of every launch ...
  bool plan_valid = false;
  int shape = 0;                       // tiled-kernel shape index
  TiledPlan plan_rt;                   // ... but the plain real-time stages, which run this one
  bool plan_rt_valid = false;
  int shape_rt = -1;
  int* d_err = nullptr;                // device error flag of the tiled kernel
  uint32_t wait_us = 2000000;          // bounded-wait limit of the tiled kernel (microseconds)
  int inject_wait = 0;                 // test hook of the bounded waits
  int* h_err = nullptr;                // pinned copy
  int chunk_user = 0;                  // x-chunk requested by the caller (0 = automatic)
  int stage_form = TRAPBEC_RK3_THREE_STAGE;   // real-time RK3 form (trapbec_rk3_form)
  int imag_stop = TRAPBEC_STOP_REL;    // stop test of RK3_RENORM (trapbec_imag_stop)
  double imag_escale = 0.0;            // its energy scale (absolute modes)
  void* lo = nullptr;                  // rounding remainder of psi (compensated form, allocated on request)
  bool lo_valid = false;               // lo belongs to the current psi (else it is cleared before use)
  // Overlapped host copies (trapbec_set_psi_async / trapbec_get_psi_async /
  // trapbec_step_rt_async), created on first use.  A queued state goes host ->
  // `stage` on cs_in while earlier steps run and is copied into psi on the
  // context stream at the next time-stepping call; a read-back copies psi into
  // `snap` on the context stream and snap -> host on cs_out while later steps
  // run.  The events order the two device buffers between the streams.
  cudaStream_t cs_in = nullptr, cs_out = nullptr;
  void* stage = nullptr;
  void* snap = nullptr;
  cudaEvent_t ev_staged = nullptr;      // cs_in: the queued state has landed in stage
  cudaEvent_t ev_stage_free = nullptr;  // st: stage was copied into psi (may be overwritten)
  cudaEvent_t ev_snap_ready = nullptr;  // st: snap holds the state to read back
  cudaEvent_t ev_snap_drained = nullptr;   // cs_out: snap reached the host (may be overwritten)
  bool stage_free_rec = false, snap_drained_rec = false;   // those two events have been recorded
  bool staged_pending = false;         // a queued state replaces psi at the next time-stepping call
  bool out_pending = false;            // a read-back is in flight
  bool step_async = false;             // do_step_rt returns after queueing (trapbec_step_rt_async)
  bool steps_pending = false;          // queued steps not yet waited for (timing and error flag unread)
  AsyncDiag* adiag = nullptr;          // page-locked result slot of trapbec_diag_async
  AsyncDiag* adiag_dev = nullptr;      // its device-side address
  cudaEvent_t ev_diag = nullptr;       // st: that slot is filled
  bool diag_pending = false;
};

namespace {

int g_nsm_cache = 0;

// psi was changed by something other than a compensated real-time step: the
// remainder array no longer belongs to it and is cleared before its next use.
inline void psi_changed(trapbec_ctx* c) { c->lo_valid = false; }

template <typename T> T eps_of() { return std::numeric_limits<T>::epsilon(); }

template <typename T> int setup_tables(trapbec_ctx* c) {
  const trapbec_params& p = c->p;
  std::vector<T> xx, yy, zz, px, py, pz;
  tbh::make_coords<T>(p, xx, yy, zz);
  tbh::make_harm_tables<T>(p, xx, yy, zz, px, py, pz);
  CK(cudaMemcpyAsync(c->xx, xx.data(), sizeof(T) * p.nx, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->yy, yy.data(), sizeof(T) * p.ny, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->zz, zz.data(), sizeof(T) * p.nz, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->px, px.data(), sizeof(T) * p.nx, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->py, py.data(), sizeof(T) * p.ny, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->pz, pz.data(), sizeof(T) * p.nz, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->hxx.assign(xx.begin(), xx.end());
  c->hyy.assign(yy.begin(), yy.end());
  c->hzz.assign(zz.begin(), zz.end());
  return TRAPBEC_OK;
}

int simple_grid(const trapbec_ctx* c) {
  size_t want = (c->n + SIMPLE_THREADS - 1) / SIMPLE_THREADS;
  size_t cap = (size_t)std::max(1, c->nsm) * 8;
  return (int)std::max<size_t>(1, std::min(want, cap));
}

bool pot_time_dependent(int kind) {
  return kind == TRAPBEC_POT_HARMONIC_RING || kind == TRAPBEC_POT_HARMONIC_RING2 ||
         kind == TRAPBEC_POT_BARRIER || kind == TRAPBEC_POT_BOX_TRAP;
}

// Which potential path the stage kernels use at time t.
template <typename T> int pot_mode_at(trapbec_ctx* c, double t) {
  const trapbec_params& p = c->p;
  if ((T)t > (T)p.potential_off) return POT_NONE;  // finite_diff.f90:124
  if (!p.lbeam && p.potential == TRAPBEC_POT_ZERO) return POT_NONE;
  if (!p.lbeam && p.potential == TRAPBEC_POT_HARMONIC) return POT_HARM;
  return POT_ARR;
}

// The 'mobius' potential's Trap array, built once on the device as mesh_init
// builds it (initial.f90:159-198): the 200 x 200 strip table is formed here
// in the context precision with the reference's expressions (pi =
// 3.14159265359 as in cdata.f90:13), the sums and the inversion by
// mobius_trap_kernel / mobius_invert_kernel.  It becomes the context's Trap
// (a later trapbec_set_trap replaces it).
template <typename T> int build_mobius_trap(trapbec_ctx* c) {
  const int N = MOBIUS_N;
  std::vector<T> tab((size_t)3 * N * N);
  const T pi = (T)3.14159265359;
  for (int i = 1; i <= N; ++i)
    for (int j = 1; j <= N; ++j) {
      const T r = (T)(i - 1) * (T)2 / (T)200 - (T)1;          // r=real(i-1)*2./200-1
      const T theta = (T)(j - 1) * (T)2 * pi / (T)200;       // theta=real(j-1)*2.*pi/200
      const T h = theta / (T)2;
      const T ring = (T)25 + (T)5 * r * std::cos(h);         // (25.+5*r*cos(theta/2))
      const size_t q = (size_t)(j - 1) * N + (i - 1);
      tab[q] = ring * std::cos(theta);
      tab[(size_t)N * N + q] = ring * std::sin(theta);
      tab[(size_t)2 * N * N + q] = (T)5 * r * std::sin(h);   // 5*r*sin(theta/2)
    }
  void* d_tab = nullptr;
  unsigned long long* d_max = nullptr;
  CK(cudaMalloc(&d_tab, tab.size() * sizeof(T)));
  CK(cudaMalloc(&d_max, sizeof(unsigned long long)));
  if (!c->trap_user) CK(cudaMalloc(&c->trap_user, c->n * sizeof(T)));
  CK(cudaMemcpyAsync(d_tab, tab.data(), tab.size() * sizeof(T), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemsetAsync(d_max, 0, sizeof(unsigned long long), c->st));
  const trapbec_params& p = c->p;
  mobius_trap_kernel<T><<<simple_grid(c), SIMPLE_THREADS, 0, c->st>>>(
      (const T*)d_tab, (const T*)c->xx, (const T*)c->yy, (const T*)c->zz, p.nx, p.ny, p.nz, (T*)c->trap_user, d_max);
  CKL();
  mobius_invert_kernel<T><<<simple_grid(c), SIMPLE_THREADS, 0, c->st>>>((T*)c->trap_user, c->n, d_max);
  CKL();
  c->launches += 2;
  CK(cudaStreamSynchronize(c->st));
  cudaFree(d_tab);
  cudaFree(d_max);
  c->pot_valid = false;
  return TRAPBEC_OK;
}

template <typename T> int ensure_potential(trapbec_ctx* c, double t) {
  if (pot_mode_at<T>(c, t) != POT_ARR) return TRAPBEC_OK;
  const trapbec_params& p = c->p;
  bool tdep = pot_time_dependent(p.potential);
  if (c->pot_valid && (!tdep || c->pot_t == t)) return TRAPBEC_OK;
  if (p.potential == TRAPBEC_POT_MOBIUS && !c->trap_user) {
    int rc = build_mobius_trap<T>(c);   // mesh_init's Trap of the 'mobius' potential
    if (rc) return rc;
  }
  if (p.potential == TRAPBEC_POT_ARRAY && !c->trap_user) {
    set_error("potential needs a Trap array: call trapbec_set_trap first");
    return TRAPBEC_ERR_STATE;
  }
  if (!c->trap_eff) CK(cudaMalloc(&c->trap_eff, c->n * sizeof(T)));
  PotArgs<T> a;
  a.trap_out = (T*)c->trap_eff;
  a.trap_in = (const T*)c->trap_user;
  a.xx = (const T*)c->xx; a.yy = (const T*)c->yy; a.zz = (const T*)c->zz;
  a.nx = p.nx; a.ny = p.ny; a.nz = p.nz;
  a.kind = p.potential;
  a.lbeam = p.lbeam;
  a.Lx = (T)p.lx; a.Ly = (T)p.ly; a.Lz = (T)p.lz; a.t = (T)t;
  a.harm_wx = (T)p.harm_wx; a.harm_wy = (T)p.harm_wy; a.harm_wz = (T)p.harm_wz; a.wbeam = (T)p.wbeam;
  fill_potential_kernel<T><<<simple_grid(c), SIMPLE_THREADS, 0, c->st>>>(a);
  CKL();
  c->launches++;
  c->pot_valid = true;
  c->pot_t = t;
  return TRAPBEC_OK;
}

// Fill the parts of StageArgs that do not depend on the stage.
template <typename T> StageArgs<T> base_args(trapbec_ctx* c, double t) {
  const trapbec_params& p = c->p;
  StageArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.xx = (const T*)c->xx; a.yy = (const T*)c->yy; a.zz = (const T*)c->zz;
  a.px = (const T*)c->px; a.py = (const T*)c->py; a.pz = (const T*)c->pz;
  a.trap = (const T*)c->trap_eff;
  a.nx = p.nx; a.ny = p.ny; a.nz = p.nz;
  a.bc = p.boundaries;
  a.zper =(p.periodicz || p.boundaries == TRAPBEC_BC_PERIODIC) ? 1 : 0;
  a.two_dim = p.two_dim ? 1 : 0;
  a.pot_mode = pot_mode_at<T>(c, t);
  T hx = (T)p.lx / (T)p.nx, hy = (T)p.ly / (T)p.ny, hz = (T)p.lz / (T)p.nz;  // initial.f90:26
  a.ix2 = (T)1 / ((T)180 * (hx * hx));
  a.iy2 = (T)1 / ((T)180 * (hy * hy));
  a.iz2 = (T)1 / ((T)180 * (hz * hz));
  a.ix1 = (T)1 / ((T)60 * hx);
  a.iy1 = (T)1 / ((T)60 * hy);
  // finite_diff.f90:126-131: advective term takes precedence over rotation.
  if (std::fabs((T)c->vx) > eps_of<T>()) {
    a.frame_mode = FRAME_ADV;
    a.omega = (T)2 * (T)c->vx;
  } else if (std::fabs((T)c->omega) > eps_of<T>() && (T)t < (T)p.t_spindown) {
    a.frame_mode = FRAME_ROT;
    a.omega = (T)c->omega;
  } else {
    a.frame_mode = FRAME_NONE;
    a.omega = 0;
  }
  a.scale = (T)1;
  return a;
}

// Default x-chunk of the work order (the autotuner may pick another).
int auto_chunk(const trapbec_ctx* c) {
  if (c->chunk_user > 0) return std::min(c->chunk_user, c->p.nx);
  if (c->chunk_user < 0) return -std::min(-c->chunk_user, c->p.nx);   // the strided order
  return c->p.nx;   // tile-major: measured fastest at 512^3; the autotuner tries other orders
}

template <typename T> bool use_tiled(trapbec_ctx* c) {
  if (c->kernel_kind == 1) return false;
  return c->plan_valid;
}

// Stage kinds of the real-time step that take the real-time plan when plain.
inline bool rt_kind(int kind) {
  return kind == ST_S1 || kind == ST_S2 || kind == ST_S3 || kind == ST_S1W || kind == ST_S2D || kind == ST_S1P ||
         kind == ST_S2P || kind == ST_S3P;
}

// The two tiled plans: `plan` (shape index `shape`; shape < 0: the first
// built shape that plans for this grid, in index order) for every launch and
// `plan_rt` for the plain real-time stages (shape_rt < 0: the default
// real-time shape where it plans; otherwise, or if it does not plan, the
// general plan).  Chunk lengths follow auto_chunk.
template <typename T> void make_plans(trapbec_ctx* c, int shape, int shape_rt) {
  if (shape >= 0) {
    c->plan_valid = (plan_tiled<T>(c->p, c->psi, c->w, c->w2, c->nsm, shape, c->d_err, &c->plan) == 0);
  } else {
    c->plan_valid = false;
    shape = 0;
    for (int i = 0; i < tiled_nshapes<T>() && !c->plan_valid; ++i)
      if (plan_tiled<T>(c->p, c->psi, c->w, c->w2, c->nsm, i, c->d_err, &c->plan) == 0) {
        c->plan_valid = true;
        shape = i;
      }
  }
  c->shape = shape;
  if (shape_rt < 0) shape_rt = tiled_rt_shape<T>();
  c->plan_rt_valid = false;
  if (shape_rt != shape)
    c->plan_rt_valid = (plan_tiled<T>(c->p, c->psi, c->w, c->w2, c->nsm, shape_rt, c->d_err, &c->plan_rt) == 0);
  if (!c->plan_rt_valid && c->plan_valid) {
    c->plan_rt = c->plan;
    c->plan_rt_valid = true;
  }
  c->shape_rt = c->plan_rt_valid ? c->plan_rt.shape : -1;
  if (c->plan_valid) c->plan.chunk = auto_chunk(c);
  if (c->plan_rt_valid) c->plan_rt.chunk = auto_chunk(c);
}

// Read and clear the device error flag of the tiled kernel.
int check_device_error(trapbec_ctx* c) {
  CK(cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (*c->h_err != 0) {
    int code = *c->h_err;
    *c->h_err = 0;
    CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->st));
    CK(cudaStreamSynchronize(c->st));
    set_error("device-side wait timed out in the tiled stage kernel (code " + std::to_string(code) + ")");
    return TRAPBEC_ERR_TIMEOUT;
  }
  return TRAPBEC_OK;
}

// Wait for steps queued by trapbec_step_rt_async: their kernel time and the
// tiled kernel's error flag.
int finish_steps(trapbec_ctx* c) {
  if (!c->steps_pending) return TRAPBEC_OK;
  c->steps_pending = false;
  CK(cudaEventSynchronize(c->e1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->e0, c->e1));
  c->last_ms = ms;
  return check_device_error(c);
}

// Copy streams, events and the staging buffer of the overlapped host copies.
int ensure_async(trapbec_ctx* c, bool stage, bool snap) {
  if (!c->cs_in) {
    CK(cudaStreamCreateWithFlags(&c->cs_in, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->cs_out, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&c->ev_staged, &c->ev_stage_free, &c->ev_snap_ready, &c->ev_snap_drained})
      CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  }
  if (stage && !c->stage) CK(cudaMalloc(&c->stage, c->n * c->esz));
  if (snap && !c->snap) CK(cudaMalloc(&c->snap, c->n * c->esz));
  return TRAPBEC_OK;
}

// dst = src (one state array) on the context stream.
int copy_state(trapbec_ctx* c, void* dst, const void* src) {
  const size_t bytes = c->n * c->esz;
  copy_state_kernel<<<4 * c->nsm, COPY_THREADS, 0, c->st>>>((const uint4*)src, (uint4*)dst, bytes / 16,
                                                            (int)((bytes % 16) != 0));
  CKL();
  c->launches++;
  return TRAPBEC_OK;
}

// A state queued by trapbec_set_psi_async becomes psi: the context stream
// waits for its host copy, copies it in, and the state's bookkeeping is that
// of trapbec_set_psi.
int apply_staged(trapbec_ctx* c) {
  if (!c->staged_pending) return TRAPBEC_OK;
  c->staged_pending = false;
  CK(cudaStreamWaitEvent(c->st, c->ev_staged, 0));
  int rc = copy_state(c, c->psi[c->cur], c->stage);
  if (rc) return rc;
  CK(cudaEventRecord(c->ev_stage_free, c->st));
  c->stage_free_rec = true;
  psi_changed(c);
  if (!c->norm_user) c->norm_target = -1.0;
  if (c->ctrl_init) {  // a new state cancels any pending renormalisation
    c->host_ctrl->scale = 1.0;
    c->host_ctrl->have_prev = 0;
    CK(cudaMemcpyAsync(c->ctrl, c->host_ctrl, sizeof(ImagCtrl), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  return TRAPBEC_OK;
}

// Launch one stage.  kind: StageKind or 4 (diagnostics).  Returns status.
template <typename T>
int launch_stage(trapbec_ctx* c, int kind, StageArgs<T>& a, int* nblk_out) {
  // plain real-time stages take the real-time plan, unless they carry the
  // compensated state and its shape does not build that variant
  const bool rt = rt_kind(kind) && tiled_plain(a) && !(a.lo && !(c->plan_rt_valid && c->plan_rt.comp_ok));
  TiledPlan& plan = rt ? c->plan_rt : c->plan;
  const bool tiled = c->kernel_kind != 1 && (rt ? c->plan_rt_valid : c->plan_valid);
  if (a.lo && !(tiled && plan.comp_ok)) {
    set_error("the compensated real-time form needs the tiled FP32 kernel on a two-row tile shape");
    return TRAPBEC_ERR_UNSUPPORTED;
  }
  plan.wait_us = c->wait_us;
  plan.inject_wait = c->inject_wait;
  if (!tiled && (kind == ST_S1W || kind == ST_S2D || kind == ST_S1P || kind == ST_S2P || kind == ST_S3P)) {
    set_error("the deferred and psi-difference real-time stages need the tiled kernel");
    return TRAPBEC_ERR_UNSUPPORTED;
  }
  if (tiled) {
    int rc = launch_tiled<T>(plan, kind, a, c->st, c->red_cap, nblk_out);
    if (rc) { set_error("tiled stage launch failed (" + std::to_string(rc) + ")"); return TRAPBEC_ERR_CUDA; }
    CKL();
    c->launches++;
    return TRAPBEC_OK;
  }
  int g = simple_grid(c);
  if (a.red && g > c->red_cap) g = c->red_cap;
  switch (kind) {
    case ST_S1: stage_simple_kernel<T, ST_S1><<<g, SIMPLE_THREADS, 0, c->st>>>(a); break;
    case ST_S2: stage_simple_kernel<T, ST_S2><<<g, SIMPLE_THREADS, 0, c->st>>>(a); break;
    case ST_S3: stage_simple_kernel<T, ST_S3><<<g, SIMPLE_THREADS, 0, c->st>>>(a); break;
    case ST_EU: stage_simple_kernel<T, ST_EU><<<g, SIMPLE_THREADS, 0, c->st>>>(a); break;
    default: stage_simple_kernel<T, 4><<<g, SIMPLE_THREADS, 0, c->st>>>(a); break;
  }
  CKL();
  c->launches++;
  if (nblk_out) *nblk_out = g;
  return TRAPBEC_OK;
}

template <typename T> int apply_pending_scale(trapbec_ctx* c) {
  if (!c->ctrl_init) return TRAPBEC_OK;
  CK(cudaMemcpyAsync(c->host_ctrl, c->ctrl, sizeof(ImagCtrl), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  double s = c->host_ctrl->scale;
  if (s != 1.0) {
    scale_kernel<T><<<simple_grid(c), SIMPLE_THREADS, 0, c->st>>>((c_t<T>*)c->psi[c->cur], c->n, (T)s);
    CKL();
    c->launches++;
    psi_changed(c);
    c->host_ctrl->scale = 1.0;
    CK(cudaMemcpyAsync(c->ctrl, c->host_ctrl, sizeof(ImagCtrl), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  return TRAPBEC_OK;
}

// Diagnostics reduction of the current psi into c->host_red[NRED].
// Queue the diagnostics reduction of the current psi into c->red_out[NRED].
template <typename T> int enqueue_diag(trapbec_ctx* c) {
  int rc = ensure_potential<T>(c, c->t);
  if (rc) return rc;
  StageArgs<T> a = base_args<T>(c, c->t);
  a.psi_in = (const c_t<T>*)c->psi[c->cur];
  a.red = c->red;
  a.reduce = 2;
  int nblk = 0;
  rc = launch_stage<T>(c, 4, a, &nblk);
  if (rc) return rc;
  reduce_finalize_kernel<<<1, FIN_THREADS, 0, c->st>>>(c->red, nblk, c->red_out);
  CKL();
  c->launches++;
  return TRAPBEC_OK;
}

template <typename T> int run_diag(trapbec_ctx* c) {
  int rc = enqueue_diag<T>(c);
  if (rc) return rc;
  CK(cudaMemcpyAsync(c->host_red, c->red_out, sizeof(double) * NRED, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return check_device_error(c);
}

// trapbec_diag_async: the reduction, then its values and the tiled kernel's
// error flag into the context's page-locked slot, with no wait.
template <typename T> int diag_async_impl(trapbec_ctx* c) {
  int rc = apply_pending_scale<T>(c);
  if (rc) return rc;
  if (!c->adiag) {
    CK(cudaHostAlloc(&c->adiag, sizeof(AsyncDiag), cudaHostAllocMapped));
    CK(cudaHostGetDevicePointer((void**)&c->adiag_dev, c->adiag, 0));
  }
  if (!c->ev_diag) CK(cudaEventCreateWithFlags(&c->ev_diag, cudaEventDisableTiming));
  if ((rc = enqueue_diag<T>(c))) return rc;
  publish_diag_kernel<<<1, 32, 0, c->st>>>(c->red_out, c->d_err, c->adiag_dev);
  CKL();
  c->launches++;
  CK(cudaEventRecord(c->ev_diag, c->st));
  c->diag_pending = true;
  return TRAPBEC_OK;
}

template <typename T> double cell_volume(const trapbec_ctx* c) {
  const trapbec_params& p = c->p;
  double hx = (double)((T)p.lx / (T)p.nx), hy = (double)((T)p.ly / (T)p.ny), hz = (double)((T)p.lz / (T)p.nz);
  return hx * hy * (p.two_dim ? 1.0 : hz);
}

template <typename T> void fill_diag(trapbec_ctx* c, const double* r, trapbec_diag_out* o) {
  const trapbec_params& p = c->p;
  double dV = cell_volume<T>(c);
  o->intpsi2 = r[0];
  o->maxpsi = r[6];
  o->minpsi = r[7];
  o->meanpsi = r[5] / ((double)p.nx * p.ny * p.nz);
  o->norm = dV * r[0];
  o->kinetic = r[1];
  o->potential = r[2];
  o->interaction = r[3];
  o->rotation = r[4];
  o->energy = dV * (-0.5 * r[1] + 0.5 * r[2] + 0.25 * r[3] - 0.5 * r[4]);
  o->mu = (-0.5 * r[1] + 0.5 * r[2] + 0.5 * r[3] - 0.5 * r[4]) / r[0];
  o->nonfinite = r[8] != 0.0 ? 1 : 0;
  o->reserved = 0;
}

// ---------------------------------------------------------------- steps --
template <typename T> int do_step_rt(trapbec_ctx* c, int nsteps) {
  int rc = apply_pending_scale<T>(c);
  if (rc) return rc;
  // run.f90:42: dt = dt*(1 - i*gamma), formed in the reference precision
  T dr = (T)c->dt_re, di = (T)c->dt_im, g = (T)c->gamma;
  T dcr = dr * (T)1 - di * (-g);
  T dci = dr * (-g) + di * (T)1;
  // eye*0.5*dt = (0, 0.5)*dt = (-0.5*Im dt, 0.5*Re dt)  (run.f90:47)
  T cre = -(T)0.5 * dci, cim = (T)0.5 * dcr;
  const T a2 = (T)(-2.) / (T)3.;
  const bool comp = c->stage_form == TRAPBEC_RK3_COMPENSATED;
  if (comp) {
    if (!c->lo) { set_error("compensated form: remainder array missing"); return TRAPBEC_ERR_STATE; }
    if (!c->lo_valid) CK(cudaMemsetAsync(c->lo, 0, c->n * c->esz, c->st));   // a new state: no remainder yet
  }
  if (nsteps > 0) psi_changed(c);
  CK(cudaEventRecord(c->e0, c->st));
  for (int s = 0; s < nsteps; ++s) {
    rc = ensure_potential<T>(c, c->t);
    if (rc) return rc;
    StageArgs<T> a = base_args<T>(c, c->t);
    a.c_re = cre; a.c_im = cim;
    a.w = (c_t<T>*)c->w;
    if (comp) {
      if (!tiled_plain(a)) {
        set_error("the compensated real-time form covers harmonic or no potential and a rotating or no frame");
        return TRAPBEC_ERR_UNSUPPORTED;
      }
      a.lo = (c_t<T>*)c->lo;
    }
    if (c->stage_form == TRAPBEC_RK3_DEFERRED && c->kernel_kind != 1 && c->plan_rt_valid && c->plan_rt.defer_ok &&
        tiled_plain(a)) {
      // deferred form: stage 1 stores w1 only; stage 2 forms psi1 = psi0 + w1/3
      // from psi0 and w1 with the FMA stage 1 would have used, and writes w2
      // to the second w buffer; stage 3 writes psi3 over psi0.  Same values.
      a.psi_in = (const c_t<T>*)c->psi[c->cur]; a.psi_out = nullptr;
      a.A = 0; a.B = (T)1 / (T)3;
      if ((rc = launch_stage<T>(c, ST_S1W, a, nullptr))) return rc;
      a.w_in = (const c_t<T>*)c->w; a.w = (c_t<T>*)c->w2;
      a.B1 = (T)1 / (T)3;
      a.psi_out = (c_t<T>*)c->psi[c->cur ^ 1];
      a.A = a2; a.B = (T)1;
      if ((rc = launch_stage<T>(c, ST_S2D, a, nullptr))) return rc;
      a.w_in = nullptr;
      a.psi_in = (const c_t<T>*)c->psi[c->cur ^ 1]; a.psi_out = (c_t<T>*)c->psi[c->cur];
      a.A = (T)(-1); a.B = (T)0.5;
      if ((rc = launch_stage<T>(c, ST_S3, a, nullptr))) return rc;
      c->t = (double)((T)c->t + dcr);   // run.f90:55, t real
      continue;
    }
    if (c->stage_form == TRAPBEC_RK3_PSI_DIFF && c->kernel_kind != 1 && c->plan_rt_valid && c->plan_rt.pdiff_ok &&
        tiled_plain(a)) {
      // psi-difference form: no w array.  Stage 1 stores psi1 only; stage 2
      // takes w1 = 3 (psi1 - psi0) and writes psi2 over psi0; stage 3 takes
      // w2 = psi2 - psi1 and writes psi3 over psi1.  Same scheme, w rounded
      // differently (the recovered w includes the rounding of the psi update).
      c_t<T>* p0 = (c_t<T>*)c->psi[c->cur];
      c_t<T>* p1 = (c_t<T>*)c->psi[c->cur ^ 1];
      a.w = nullptr;
      a.psi_in = p0; a.psi_out = p1;
      a.A = 0; a.B = (T)1 / (T)3;
      if ((rc = launch_stage<T>(c, ST_S1P, a, nullptr))) return rc;
      a.psi_in = p1; a.w_in = p0; a.psi_out = p0;
      a.A = a2; a.B = (T)1; a.rB = (T)3;
      if ((rc = launch_stage<T>(c, ST_S2P, a, nullptr))) return rc;
      a.psi_in = p0; a.w_in = p1; a.psi_out = p1;
      a.A = (T)(-1); a.B = (T)0.5; a.rB = (T)1;
      if ((rc = launch_stage<T>(c, ST_S3P, a, nullptr))) return rc;
      c->cur ^= 1;
      c->t = (double)((T)c->t + dcr);   // run.f90:55, t real
      continue;
    }
    // stage 1: w = c rhs; psi += w/3
    a.psi_in = (const c_t<T>*)c->psi[c->cur]; a.psi_out = (c_t<T>*)c->psi[c->cur ^ 1];
    a.A = 0; a.B = (T)1 / (T)3;
    if ((rc = launch_stage<T>(c, ST_S1, a, nullptr))) return rc;
    // stage 2: w = -2/3 w + c rhs; psi += w
    a.psi_in = (const c_t<T>*)c->psi[c->cur ^ 1]; a.psi_out = (c_t<T>*)c->psi[c->cur];
    a.A = a2; a.B = (T)1;
    if ((rc = launch_stage<T>(c, ST_S2, a, nullptr))) return rc;
    // stage 3: w = -w + c rhs; psi += w/2
    a.psi_in = (const c_t<T>*)c->psi[c->cur]; a.psi_out = (c_t<T>*)c->psi[c->cur ^ 1];
    a.A = (T)(-1); a.B = (T)0.5;
    if ((rc = launch_stage<T>(c, ST_S3, a, nullptr))) return rc;
    c->cur ^= 1;
    c->t = (double)((T)c->t + dcr);   // run.f90:55, t real
  }
  CK(cudaEventRecord(c->e1, c->st));
  if (comp) c->lo_valid = true;
  if (c->step_async) {   // trapbec_step_rt_async: the steps are queued; finish_steps reads the rest
    c->steps_pending = true;
    return TRAPBEC_OK;
  }
  c->steps_pending = false;
  CK(cudaEventSynchronize(c->e1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->e0, c->e1));
  c->last_ms = ms;
  return check_device_error(c);
}

template <typename T> int do_imag_euler(trapbec_ctx* c, int nsteps, int* steps_done, double* ratio) {
  int rc = apply_pending_scale<T>(c);
  if (rc) return rc;
  // run.f90:22: Psi = Psi + dt*0.5*rhs, with dt before the damping of run.f90:42
  T cre = (T)c->dt_re * (T)0.5, cim = (T)c->dt_im * (T)0.5;
  psi_changed(c);
  double r = 0.0;
  for (int s = 0; s < nsteps; ++s) {
    if ((rc = ensure_potential<T>(c, c->t))) return rc;
    StageArgs<T> a = base_args<T>(c, c->t);
    a.c_re = cre; a.c_im = cim;
    a.psi_in = (const c_t<T>*)c->psi[c->cur]; a.psi_out = (c_t<T>*)c->psi[c->cur ^ 1];
    if ((rc = launch_stage<T>(c, ST_EU, a, nullptr))) return rc;
    c->cur ^= 1;
    if ((rc = run_diag<T>(c))) return rc;   // Psi_norm (run.f90:23)
    double nrm = c->host_red[0];
    r = nrm / c->intpsi2_old;
    c->intpsi2_old = nrm;
  }
  *steps_done = nsteps;
  *ratio = r;
  return TRAPBEC_OK;
}

template <typename T> int do_imag_rk3(trapbec_ctx* c, int nsteps, double tol, int* steps_done, double* rel_out) {
  int rc = apply_pending_scale<T>(c);
  if (rc) return rc;
  double dV = cell_volume<T>(c);
  if (!(c->norm_target > 0.0)) {   // unset (or derived from a non-finite state)
    if ((rc = run_diag<T>(c))) return rc;
    c->norm_target = dV * c->host_red[0];
  }
  if (!c->ctrl_init) {
    std::memset(c->host_ctrl, 0, sizeof(ImagCtrl));
    c->host_ctrl->scale = 1.0;
    c->ctrl_init = true;
  } else {
    CK(cudaMemcpyAsync(c->host_ctrl, c->ctrl, sizeof(ImagCtrl), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  c->host_ctrl->n0 = c->norm_target;
  c->host_ctrl->tol = tol;
  c->host_ctrl->dV = dV;
  c->host_ctrl->escale = c->imag_escale;
  c->host_ctrl->stop_mode = c->imag_stop;
  c->host_ctrl->converged = 0;
  c->host_ctrl->step = 0;
  c->host_ctrl->nonfinite = 0;
  c->host_ctrl->have_prev = 0;   // the first comparison is after the first step
  CK(cudaMemcpyAsync(c->ctrl, c->host_ctrl, sizeof(ImagCtrl), cudaMemcpyHostToDevice, c->st));
  const T cf = (T)0.5 * (T)c->dt_re;
  const T a2 = (T)(-2.) / (T)3.;
  const int start_cur = c->cur;
  psi_changed(c);
  CK(cudaEventRecord(c->e0, c->st));
  int nblk = 0;
  // stage 1 of the step from buffer `par`, with the energy of the incoming
  // (renormalised) state reduced and handed to the energy finaliser
  auto stage1_energy = [&](int par) -> int {
    int r2 = ensure_potential<T>(c, c->t);
    if (r2) return r2;
    StageArgs<T> a = base_args<T>(c, c->t);
    a.c_re = cf; a.c_im = 0;
    a.w = (c_t<T>*)c->w;
    a.ctrl = c->ctrl;
    a.psi_in = (const c_t<T>*)c->psi[par]; a.psi_out = (c_t<T>*)c->psi[par ^ 1];
    a.A = 0; a.B = (T)1 / (T)3;
    a.red = c->red; a.reduce = 2; a.use_ctrl_scale = 1;
    if ((r2 = launch_stage<T>(c, ST_S1, a, &nblk))) return r2;
    imag_fin_energy_kernel<<<1, FIN_THREADS, 0, c->st>>>(c->red, nblk, c->ctrl);
    CKL();
    c->launches++;
    return TRAPBEC_OK;
  };
  for (int s = 0; s < nsteps; ++s) {
    int par = (start_cur + s) & 1;
    if ((rc = stage1_energy(par))) return rc;
    StageArgs<T> a = base_args<T>(c, c->t);
    a.c_re = cf; a.c_im = 0;
    a.w = (c_t<T>*)c->w;
    a.ctrl = c->ctrl;
    a.reduce = 0; a.red = nullptr; a.use_ctrl_scale = 0;
    a.psi_in = (const c_t<T>*)c->psi[par ^ 1]; a.psi_out = (c_t<T>*)c->psi[par];
    a.A = a2; a.B = (T)1;
    if ((rc = launch_stage<T>(c, ST_S2, a, nullptr))) return rc;
    a.psi_in = (const c_t<T>*)c->psi[par]; a.psi_out = (c_t<T>*)c->psi[par ^ 1];
    a.A = (T)(-1); a.B = (T)0.5;
    a.red = c->red; a.reduce = 1;
    if ((rc = launch_stage<T>(c, ST_S3, a, &nblk))) return rc;
    imag_fin_norm_kernel<<<1, FIN_THREADS, 0, c->st>>>(c->red, nblk, c->ctrl);
    CKL();
    c->launches++;
    if ((s + 1) % 64 == 0 || s + 1 == nsteps) {
      CK(cudaMemcpyAsync(c->host_ctrl, c->ctrl, sizeof(ImagCtrl), cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      if (c->host_ctrl->converged || c->host_ctrl->nonfinite) break;
    }
  }
  CK(cudaEventRecord(c->e1, c->st));
  CK(cudaMemcpyAsync(c->host_ctrl, c->ctrl, sizeof(ImagCtrl), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->e0, c->e1));
  c->last_ms = ms;
  ImagCtrl& h = *c->host_ctrl;
  int done = h.step;
  c->cur = (start_cur + done) & 1;
  if ((rc = check_device_error(c))) {   // a bounded wait gave up: the sums are not meaningful
    *steps_done = done;
    *rel_out = NAN;
    return rc;
  }
  if (h.nonfinite) {
    *steps_done = done;
    *rel_out = NAN;
    set_error("non-finite norm in imaginary-time relaxation");
    return TRAPBEC_ERR_NONFINITE;
  }
  if (!h.converged) {
    // Energy of the final state, which the loop forms in the next step's
    // stage 1: run that stage-1 evaluation once more (its psi and w outputs go
    // to the spare buffers and are discarded; the state stays in c->cur with
    // its renormalisation pending), so the last |dE| compares two energies of
    // the same evaluation.  It may meet the stop test; no step is counted.
    if ((rc = stage1_energy(c->cur))) return rc;
    CK(cudaMemcpyAsync(c->host_ctrl, c->ctrl, sizeof(ImagCtrl), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    if ((rc = check_device_error(c))) { *steps_done = done; *rel_out = NAN; return rc; }
    if (h.nonfinite) {
      *steps_done = done;
      *rel_out = NAN;
      set_error("non-finite energy in imaginary-time relaxation");
      return TRAPBEC_ERR_NONFINITE;
    }
    if (done == 0) h.rel = INFINITY;   // nothing to compare with
  }
  if ((rc = apply_pending_scale<T>(c))) return rc;
  *steps_done = done;
  *rel_out = h.rel;
  return TRAPBEC_OK;
}

template <typename T> int init_state_impl(trapbec_ctx* c, const char* name, const trapbec_init_args* ia) {
  const trapbec_params& p = c->p;
  psi_changed(c);
  std::string nm(name);
  InitArgsDev<T> a;
  std::memset(&a, 0, sizeof(a));
  a.psi = (c_t<T>*)c->psi[c->cur];
  a.xx = (const T*)c->xx; a.yy = (const T*)c->yy; a.zz = (const T*)c->zz;
  a.nx = p.nx; a.ny = p.ny; a.nz = p.nz;
  a.wn = p.winding_number;
  a.Lx = (T)p.lx; a.Ly = (T)p.ly; a.Lz = (T)p.lz;
  a.pi = (T)3.14159265359;   // cdata.f90:13
  a.harm_wx = (T)p.harm_wx; a.harm_wy = (T)p.harm_wy; a.harm_wz = (T)p.harm_wz;
  tbh::Rng rng{ia ? ia->seed : 0};
  auto runif = [&](T lo, T hi) { T u = (T)rng.next(); return lo + u * (hi - lo); };
  auto go = [&](int kind) -> int {
    a.kind = kind;
    init_state_kernel<T><<<simple_grid(c), SIMPLE_THREADS, 0, c->st>>>(a);
    CKL();
    c->launches++;
    return TRAPBEC_OK;
  };
  int rc = TRAPBEC_OK;
  const T pi = a.pi;
  if (nm == "constant") {
    a.v[0] = a.v[1] = (T)1 / std::sqrt((T)2);
    rc = go(IK_CONST);
  } else if (nm == "thomas_fermi") {
    rc = go(IK_TF);
  } else if (nm == "soliton") {
    if (!(rc = go(IK_TF))) rc = go(IK_SOLITON_PHASE);
  } else if (nm == "single_vortex") {
    rc = go(IK_SINGLE);
  } else if (nm == "sausage") {
    rc = go(IK_SAUSAGE);
  } else if (nm == "crow") {
    rc = go(IK_CROW);
  } else if (nm == "random_points" || nm == "leap_frog") {
    a.v[0] = a.v[1] = (T)0.7071;
    if ((rc = go(IK_SET))) return rc;
    int nv = nm == "random_points" ? 20 : 4;
    for (int v = 1; v <= nv; ++v) {
      T vx, vy, dir;
      if (nm == "random_points") {
        vx = runif(-(T)p.lx / (T)5, (T)p.lx / (T)5);
        vy = runif(-(T)p.ly / (T)5, (T)p.ly / (T)5);
        dir = runif((T)0.9, (T)1);
        dir = dir < (T)0.5 ? (T)(-1) : (T)1;
      } else {
        const T sh = 3, s1 = 3, s2 = 12;
        if (v == 1) { vx = -sh; vy = s1; dir = 1; }
        else if (v == 2) { vx = sh; vy = s2; dir = 1; }
        else if (v == 3) { vx = -sh; vy = -s1; dir = -1; }
        else { vx = sh; vy = -s2; dir = -1; }
      }
      a.v[0] = vx; a.v[1] = vy; a.v[2] = dir; a.v[3] = 0;
      if ((rc = go(IK_VORTEX_MUL))) return rc;
    }
  } else if (nm == "lattice") {  // initial.f90:377-420 (ramp = 0: straight lines)
    a.v[0] = 1; a.v[1] = 1;
    if ((rc = go(IK_SET))) return rc;
    for (int v1 = 1; v1 <= 10; ++v1)
      for (int v2 = 1; v2 <= 10; ++v2) {
        (void)runif(0, (T)2 * pi);   // rphase
        (void)runif(0, 1);           // rdir
        a.v[0] = (T)v1 * ((T)p.lx / (T)16) - (T)p.lx / (T)3;
        a.v[1] = (T)v2 * ((T)p.ly / (T)16) - (T)p.ly / (T)3;
        a.v[2] = 1; a.v[3] = 0;
        if ((rc = go(IK_VORTEX_MUL))) return rc;
      }
  } else if (nm == "lattice2" || nm == "bundle") {  // initial.f90:422-539
    if ((rc = go(IK_TF))) return rc;
    if (nm == "lattice2") {
      for (int pl = 0; pl < 2; ++pl)
        for (int v1 = 1; v1 <= 3; ++v1)
          for (int v2 = 1; v2 <= 3; ++v2) {
            if (pl == 0) {
              a.v[0] = (T)v1 * ((T)p.lx / (T)4) - (T)p.lx / (T)2;
              a.v[1] = (T)v2 * ((T)p.ly / (T)4) - (T)p.ly / (T)2;
            } else {
              a.v[0] = (T)v1 * ((T)p.lx / (T)4) + (T)10 - (T)p.lx / (T)2;
              a.v[1] = (T)v2 * ((T)p.lz / (T)4) + (T)10 - (T)p.lz / (T)2;
            }
            a.v[2] = 1; a.v[3] = (T)pl;
            if ((rc = go(IK_VORTEX_MUL))) return rc;
          }
    } else {
      for (int pl = 0; pl < 3; ++pl)
        for (int v1 = 1; v1 <= 7; ++v1) {
          T rpos = v1 == 1 ? (T)0 : (T)10;
          T tpos = v1 == 1 ? (T)0 : (T)(v1 - 2) * (T)2 * pi / (T)6;
          T c1 = rpos * std::cos(tpos), c2 = rpos * std::sin(tpos);
          if (pl == 0 || pl == 2) c1 = c1 - (T)30; else c2 = c2 - (T)30;
          a.v[0] = c1; a.v[1] = c2; a.v[2] = 1; a.v[3] = (T)pl;
          if ((rc = go(IK_VORTEX_MUL))) return rc;
        }
    }
  } else if (nm == "line_of_lines") {  // initial.f90:541-585
    a.v[0] = a.v[1] = (T)1 / std::sqrt((T)2);
    if ((rc = go(IK_SET))) return rc;
    a.v[0] = 0; a.v[1] = 0; a.v[2] = 0; a.v[3] = (T)p.ring_rad; a.v[4] = 0;
    rc = go(IK_RINGPAIR_MUL);
  } else if (nm == "linked_rings") {  // initial.f90:587-626
    a.v[0] = 0; a.v[1] = 0; a.v[2] = 0; a.v[3] = (T)p.ring_rad; a.v[4] = 1;
    if ((rc = go(IK_RINGPAIR_MUL))) return rc;
    a.v[0] = 1; a.v[1] = 0; a.v[2] = (T)p.ring_rad * (T)1.2; a.v[3] = (T)p.ring_rad; a.v[4] = 0;
    rc = go(IK_RINGPAIR_MUL);
  } else if (nm == "random_phase") {  // setup_quench, initial.f90:346-375
    a.v[0] = 0; a.v[1] = 0;
    if ((rc = go(IK_SET))) return rc;
    a.wn = p.two_dim ? 1 : 0;
    for (int kk = 1; kk <= 20; ++kk) {
      a.v[0] = std::floor(runif(-20, 20));
      a.v[1] = std::floor(runif(-20, 20));
      a.v[2] = std::floor(runif(-20, 20));
      a.v[3] = runif((T)(-0.1), (T)0.1);
      a.v[4] = runif((T)(-0.1), (T)0.1);
      if ((rc = go(IK_QUENCH_ADD))) return rc;
    }
    a.wn = p.winding_number;
    rc = go(IK_TF_MUL);
  } else if (nm == "vortex_rings") {
    a.v[0] = 1; a.v[1] = 0;
    if ((rc = go(IK_SET))) return rc;
    for (int v = 1; v <= p.vor_ring_count; ++v) {
      T ax = runif(0, 0), ay = runif(0, (T)2 * pi), az = runif(0, (T)2 * pi);
      T tu = runif(-1, 1), tth = runif(0, (T)2 * pi), tr = runif(0, (T)p.lx / (T)6);
      T tx = tr * std::sqrt((T)1 - tu * tu) * std::cos(tth);
      T ty = tr * std::sqrt((T)1 - tu * tu) * std::sin(tth);
      T tz = tr * tu;
      a.v[0] = ax; a.v[1] = ay; a.v[2] = az; a.v[3] = tx; a.v[4] = ty; a.v[5] = tz; a.v[6] = (T)p.ring_rad;
      if ((rc = go(IK_RING_MUL))) return rc;
    }
  } else if (nm == "tf_vortex_line" || nm == "tf_vortex_ring" || nm == "tf_noise") {
    if (!ia) { set_error("init_state: workload states need trapbec_init_args"); return TRAPBEC_ERR_ARG; }
    a.d[0] = ia->amp; a.d[1] = ia->r_tf2[0]; a.d[2] = ia->r_tf2[1]; a.d[3] = ia->r_tf2[2];
    a.d[4] = ia->ring_radius; a.d[5] = ia->core2; a.d[6] = ia->noise_amp;
    a.seed = ia->seed;
    rc = go(nm == "tf_vortex_line" ? IK_TF_LINE : (nm == "tf_vortex_ring" ? IK_TF_RING : IK_TF_NOISE));
  } else if (nm == "add_noise") {  // helpers applied to the current state
    a.seed = ia ? ia->seed : 0;
    rc = go(IK_NOISE_ADD);
  } else if (nm == "add_ring") {  // setup_add_ring option 1, initial.f90:759-794
    a.v[0] = 0; a.v[1] = (T)(-0.25) * (T)p.lx; a.v[2] = 0; a.v[3] = (T)p.ring_rad; a.v[4] = 0;
    rc = go(IK_RINGPAIR_MUL);
  } else if (nm == "add_dipole") {  // setup_add_dipole, initial.f90:839-870
    for (int v = 1; v <= 2; ++v) {
      a.v[0] = -20; a.v[1] = v == 1 ? (T)5 : (T)(-5); a.v[2] = v == 1 ? (T)1 : (T)(-1); a.v[3] = 0;
      if ((rc = go(IK_VORTEX_MUL))) return rc;
    }
  } else if (nm == "phase_imprint") {  // initial.f90:820-836
    rc = go(IK_PHASE_IMPRINT);
  } else if (nm == "add_pcurrent") {  // setup_pcurrent, initial.f90:669-739
    a.v[0] = (T)p.potential;
    rc = go(IK_PCURRENT);
  } else if (nm == "force_vortex") {  // force.f90:33-44 at (x0, y0) with dir, from force_args
    a.v[0] = (T)c->force_args[0]; a.v[1] = (T)c->force_args[1]; a.v[2] = (T)c->force_args[2];
    rc = go(IK_FORCE_VORTEX);
  } else {
    set_error("unknown initial state: " + nm);   // initial.f90:155-156
    return TRAPBEC_ERR_ARG;
  }
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->st));
  return TRAPBEC_OK;
}

template <typename T> int create_impl(trapbec_ctx* c) {
  const trapbec_params& p = c->p;
  size_t n = c->n;
  CK(cudaMalloc(&c->psi[0], n * c->esz));
  CK(cudaMalloc(&c->psi[1], n * c->esz));
  CK(cudaMalloc(&c->w, n * c->esz));
  CK(cudaMemsetAsync(c->psi[0], 0, n * c->esz, c->st));
  CK(cudaMemsetAsync(c->psi[1], 0, n * c->esz, c->st));
  CK(cudaMemsetAsync(c->w, 0, n * c->esz, c->st));
  CK(cudaMalloc(&c->xx, sizeof(T) * p.nx));
  CK(cudaMalloc(&c->yy, sizeof(T) * p.ny));
  CK(cudaMalloc(&c->zz, sizeof(T) * p.nz));
  CK(cudaMalloc(&c->px, sizeof(T) * p.nx));
  CK(cudaMalloc(&c->py, sizeof(T) * p.ny));
  CK(cudaMalloc(&c->pz, sizeof(T) * p.nz));
  c->red_cap = std::max(4096, c->nsm * 16);
  CK(cudaMalloc(&c->red, sizeof(double) * NRED * (size_t)c->red_cap));
  CK(cudaMalloc(&c->red_out, sizeof(double) * NRED));
  CK(cudaMallocHost(&c->host_red, sizeof(double) * NRED));
  CK(cudaMalloc(&c->ctrl, sizeof(ImagCtrl)));
  CK(cudaMallocHost(&c->host_ctrl, sizeof(ImagCtrl)));
  CK(cudaMemsetAsync(c->ctrl, 0, sizeof(ImagCtrl), c->st));
  CK(cudaMalloc(&c->d_err, sizeof(int)));
  CK(cudaMallocHost(&c->h_err, sizeof(int)));
  CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->st));
  *c->h_err = 0;
  int rc = setup_tables<T>(c);
  if (rc) return rc;
  make_plans<T>(c, -1, -1);
  return TRAPBEC_OK;
}

void free_ctx(trapbec_ctx* c) {
  if (!c) return;
  if (c->cs_in) cudaStreamSynchronize(c->cs_in);
  if (c->cs_out) cudaStreamSynchronize(c->cs_out);
  void* bufs[] = {c->psi[0], c->psi[1], c->w, c->w2, c->lo, c->xx, c->yy, c->zz, c->px, c->py, c->pz,
                  c->trap_user, c->trap_eff, c->red, c->red_out, c->ctrl, c->d_err, c->stage, c->snap};
  for (void* b : bufs) if (b) cudaFree(b);
  if (c->host_red) cudaFreeHost(c->host_red);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->host_ctrl) cudaFreeHost(c->host_ctrl);
  if (c->adiag) cudaFreeHost(c->adiag);
  for (cudaEvent_t e : {c->e0, c->e1, c->ev_staged, c->ev_stage_free, c->ev_snap_ready, c->ev_snap_drained,
                        c->ev_diag})
    if (e) cudaEventDestroy(e);
  if (c->cs_in) cudaStreamDestroy(c->cs_in);
  if (c->cs_out) cudaStreamDestroy(c->cs_out);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

int validate(const trapbec_params* p) {
  if (!p) { set_error("null params"); return TRAPBEC_ERR_ARG; }
  if (p->nx <= 0 || p->ny <= 0 || p->nz <= 0) { set_error("grid sizes must be positive"); return TRAPBEC_ERR_ARG; }
  if (p->precision != TRAPBEC_FP32 && p->precision != TRAPBEC_FP64) { set_error("bad precision"); return TRAPBEC_ERR_ARG; }
  if (p->boundaries < 0 || p->boundaries > 2) { set_error("wrong boundaries set"); return TRAPBEC_ERR_ARG; }
  if (p->potential < 0 || p->potential > 10) { set_error("error incorrect potential set"); return TRAPBEC_ERR_ARG; }
  int px = p->nprocx > 0 ? p->nprocx : 1, py = p->nprocy > 0 ? p->nprocy : 1;
  if (p->nx % px || p->ny % py) {  // mpi_var.f90:157-160
    set_error("unable to evenly subdivide grid check meshsize and number of processors");
    return TRAPBEC_ERR_ARG;
  }
  // Ghost fills reach 3 cells in: solid and periodic boundaries need n >= 4
  // on every axis whose derivatives are used (ghost.f90 mirrors Psi(2..4)).
  bool needz = !p->two_dim;
  if (p->nx < 4 || p->ny < 4 || (needz && p->nz < 4)) {
    set_error("grid must have at least 4 cells per differentiated axis");
    return TRAPBEC_ERR_ARG;
  }
  if (p->lx <= 0 || p->ly <= 0 || p->lz <= 0) { set_error("box lengths must be positive"); return TRAPBEC_ERR_ARG; }
  return TRAPBEC_OK;
}

#define DISPATCH(ctx, fn, ...) ((ctx)->prec == TRAPBEC_FP64 ? fn<double>(__VA_ARGS__) : fn<float>(__VA_ARGS__))

// Interior <-> ghosted host layouts: Psi(-2:nz+3,-2:ny+3,-2:nx+3).
void to_ghosted(const trapbec_params& p, const char* in, char* out, size_t esz) {
  size_t gz = p.nz + 6, gy = p.ny + 6, gx = p.nx + 6;
  std::memset(out, 0, gz * gy * gx * esz);
  for (int i = 0; i < p.nx; ++i)
    for (int j = 0; j < p.ny; ++j)
      std::memcpy(out + (((size_t)(i + 3) * gy + (j + 3)) * gz + 3) * esz,
                  in + (((size_t)i * p.ny + j) * p.nz) * esz, (size_t)p.nz * esz);
}
void from_ghosted(const trapbec_params& p, const char* in, char* out, size_t esz) {
  size_t gz = p.nz + 6, gy = p.ny + 6;
  for (int i = 0; i < p.nx; ++i)
    for (int j = 0; j < p.ny; ++j)
      std::memcpy(out + (((size_t)i * p.ny + j) * p.nz) * esz,
                  in + (((size_t)(i + 3) * gy + (j + 3)) * gz + 3) * esz, (size_t)p.nz * esz);
}
// Fill the ghost shell the way ghost_comm leaves it on one rank (faces only;
// edges and corners stay zero as the reference never writes them).
void ghost_fill_host(const trapbec_params& p, char* g, size_t esz) {
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  size_t gz = nz + 6, gy = ny + 6;
  auto at = [&](int k, int j, int i) { return g + (((size_t)(i + 2) * gy + (j + 2)) * gz + (k + 2)) * esz; };
  auto cp = [&](char* dst, const char* src) { std::memcpy(dst, src, esz); };
  auto zero = [&](char* dst) { std::memset(dst, 0, esz); };
  // 1-based Fortran indices below (ghost.f90:27-192)
  for (int m = 1; m <= 3; ++m)
    for (int j = 1; j <= ny; ++j)
      for (int k = 1; k <= nz; ++k) {
        char* hi = at(k, j, nx + m); char* lo = at(k, j, 1 - m);
        if (p.boundaries == TRAPBEC_BC_PERIODIC) { cp(hi, at(k, j, m)); cp(lo, at(k, j, nx + 1 - m)); }
        else if (p.boundaries == TRAPBEC_BC_SOLID) { cp(hi, at(k, j, nx - m)); cp(lo, at(k, j, 1 + m)); }
        else { zero(hi); zero(lo); }
      }
  for (int i = 1; i <= nx; ++i)
    for (int m = 1; m <= 3; ++m)
      for (int k = 1; k <= nz; ++k) {
        char* hi = at(k, ny + m, i); char* lo = at(k, 1 - m, i);
        if (p.boundaries == TRAPBEC_BC_PERIODIC) { cp(hi, at(k, m, i)); cp(lo, at(k, ny + 1 - m, i)); }
        else if (p.boundaries == TRAPBEC_BC_SOLID) { cp(hi, at(k, ny - m, i)); cp(lo, at(k, 1 + m, i)); }
        else { zero(hi); zero(lo); }
      }
  bool zper = p.periodicz || p.boundaries == TRAPBEC_BC_PERIODIC;
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j)
      for (int m = 1; m <= 3; ++m) {
        char* hi = at(nz + m, j, i); char* lo = at(1 - m, j, i);
        if (zper) { cp(hi, at(m, j, i)); cp(lo, at(nz + 1 - m, j, i)); }
        else if (p.boundaries == TRAPBEC_BC_SOLID) { cp(hi, at(nz - m, j, i)); cp(lo, at(1 + m, j, i)); }
        else { zero(hi); zero(lo); }
      }
}

}  // namespace

// ================================================================== C ABI ==
extern "C" {

int trapbec_abi_version(void) { return TRAPBEC_ABI_VERSION; }

int trapbec_abi_struct_size(int which) {
  switch (which) {
    case 0: return (int)sizeof(trapbec_params);
    case 1: return (int)sizeof(trapbec_diag_out);
    case 2: return (int)sizeof(trapbec_init_args);
  }
  return -1;
}

const char* trapbec_strerror(int code) {
  switch (code) {
    case TRAPBEC_OK: return "ok";
    case TRAPBEC_ERR_ARG: return "invalid argument";
    case TRAPBEC_ERR_CUDA: return "CUDA error";
    case TRAPBEC_ERR_NOMEM: return "out of memory";
    case TRAPBEC_ERR_STATE: return "invalid state";
    case TRAPBEC_ERR_TIMEOUT: return "device wait timed out";
    case TRAPBEC_ERR_NONFINITE: return "non-finite values in psi";
    case TRAPBEC_ERR_IO: return "I/O error";
    case TRAPBEC_ERR_UNSUPPORTED: return "unsupported";
    case TRAPBEC_ERR_PARSE: return "parse error";
    case TRAPBEC_ERR_NODEVICE: return "no CUDA device";
  }
  return "unknown error";
}

const char* trapbec_last_error(void) { return tbh::get_error(); }

int trapbec_create(const trapbec_params* p, trapbec_ctx** out) {
  if (!out) return TRAPBEC_ERR_ARG;
  *out = nullptr;
  int rc = validate(p);
  if (rc) return rc;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    set_error(std::string("no CUDA device: ") + cudaGetErrorString(e));
    return TRAPBEC_ERR_NODEVICE;
  }
  trapbec_ctx* c = new trapbec_ctx;
  c->p = *p;
  c->prec = p->precision;
  c->n = (size_t)p->nx * p->ny * p->nz;
  c->rsz = p->precision == TRAPBEC_FP64 ? 8 : 4;
  c->esz = 2 * c->rsz;
  c->dt_re = p->dt_re; c->dt_im = p->dt_im; c->gamma = p->gamma;
  c->omega = p->omega_z; c->vx = p->advective_vx;
  cudaGetDevice(&c->dev);
  cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->dev);
  g_nsm_cache = c->nsm;
  auto bail = [&](int code) { free_ctx(c); return code; };
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("cudaStreamCreate failed");
    return bail(TRAPBEC_ERR_CUDA);
  }
  cudaEventCreate(&c->e0);
  cudaEventCreate(&c->e1);
  rc = DISPATCH(c, create_impl, c);
  if (rc) return bail(rc);
  *out = c;
  return TRAPBEC_OK;
}

void trapbec_destroy(trapbec_ctx* c) {
  if (c && c->st) cudaStreamSynchronize(c->st);   // free_ctx also waits for the copy streams
  free_ctx(c);
}

int trapbec_set_psi(trapbec_ctx* c, const void* psi, int layout) {
  if (!c || !psi) return TRAPBEC_ERR_ARG;
  int rc0 = finish_steps(c);
  if (rc0) return rc0;
  c->staged_pending = false;   // this state replaces a queued one
  psi_changed(c);
  if (layout == TRAPBEC_LAYOUT_INTERIOR) {
    CK(cudaMemcpyAsync(c->psi[c->cur], psi, c->n * c->esz, cudaMemcpyHostToDevice, c->st));
  } else if (layout == TRAPBEC_LAYOUT_GHOSTED) {
    std::vector<char> tmp(c->n * c->esz);
    from_ghosted(c->p, (const char*)psi, tmp.data(), c->esz);
    CK(cudaMemcpyAsync(c->psi[c->cur], tmp.data(), c->n * c->esz, cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
  } else {
    set_error("bad layout");
    return TRAPBEC_ERR_ARG;
  }
  if (!c->norm_user) c->norm_target = -1.0;   // the next relaxation keeps this state's norm
  if (c->ctrl_init) {  // a new state cancels any pending renormalisation
    c->host_ctrl->scale = 1.0;
    c->host_ctrl->have_prev = 0;
    CK(cudaMemcpyAsync(c->ctrl, c->host_ctrl, sizeof(ImagCtrl), cudaMemcpyHostToDevice, c->st));
  }
  CK(cudaStreamSynchronize(c->st));
  return TRAPBEC_OK;
}

int trapbec_get_psi(trapbec_ctx* c, void* psi, int layout) {
  if (!c || !psi) return TRAPBEC_ERR_ARG;
  int rc = finish_steps(c);
  if (rc) return rc;
  rc = DISPATCH(c, apply_pending_scale, c);
  if (rc) return rc;
  if (layout == TRAPBEC_LAYOUT_INTERIOR) {
    CK(cudaMemcpyAsync(psi, c->psi[c->cur], c->n * c->esz, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  } else if (layout == TRAPBEC_LAYOUT_GHOSTED) {
    std::vector<char> tmp(c->n * c->esz);
    CK(cudaMemcpyAsync(tmp.data(), c->psi[c->cur], c->n * c->esz, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    to_ghosted(c->p, tmp.data(), (char*)psi, c->esz);
    ghost_fill_host(c->p, (char*)psi, c->esz);
  } else {
    set_error("bad layout");
    return TRAPBEC_ERR_ARG;
  }
  return TRAPBEC_OK;
}

int trapbec_set_trap(trapbec_ctx* c, const double* trap) {
  if (!c || !trap) return TRAPBEC_ERR_ARG;
  if (!c->trap_user) CK(cudaMalloc(&c->trap_user, c->n * c->rsz));
  if (c->prec == TRAPBEC_FP64) {
    CK(cudaMemcpyAsync(c->trap_user, trap, c->n * 8, cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
  } else {
    std::vector<float> f(c->n);
    for (size_t i = 0; i < c->n; ++i) f[i] = (float)trap[i];
    CK(cudaMemcpyAsync(c->trap_user, f.data(), c->n * 4, cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  c->pot_valid = false;
  return TRAPBEC_OK;
}

int trapbec_init_state(trapbec_ctx* c, const char* name, const trapbec_init_args* args) {
  if (!c || !name) return TRAPBEC_ERR_ARG;
  int rc = finish_steps(c);
  if (rc) return rc;
  c->staged_pending = false;   // this state replaces a queued one
  rc = DISPATCH(c, init_state_impl, c, name, args);
  if (rc) return rc;
  if (!c->norm_user) c->norm_target = -1.0;   // the next relaxation keeps the new state's norm
  if (c->ctrl_init) {
    c->host_ctrl->scale = 1.0;
    c->host_ctrl->have_prev = 0;
    CK(cudaMemcpyAsync(c->ctrl, c->host_ctrl, sizeof(ImagCtrl), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  return TRAPBEC_OK;
}

}  // extern "C"
namespace {
template <typename T> int get_rhs_impl(trapbec_ctx* c, void* out) {
  int rc = apply_pending_scale<T>(c);
  if (rc) return rc;
  if ((rc = ensure_potential<T>(c, c->t))) return rc;
  StageArgs<T> a = base_args<T>(c, c->t);
  a.c_re = 1; a.c_im = 0; a.A = 0; a.B = 0;   // w = 1*rhs exactly
  a.w = (c_t<T>*)c->w;
  a.psi_in = (const c_t<T>*)c->psi[c->cur];
  a.psi_out = (c_t<T>*)c->psi[c->cur ^ 1];     // spare buffer, discarded
  if ((rc = launch_stage<T>(c, ST_S1, a, nullptr))) return rc;
  CK(cudaMemcpyAsync(out, c->w, c->n * c->esz, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return TRAPBEC_OK;
}
}  // namespace
extern "C" {

int trapbec_get_rhs(trapbec_ctx* c, void* rhs_out) {
  if (!c || !rhs_out) return TRAPBEC_ERR_ARG;
  return DISPATCH(c, get_rhs_impl, c, rhs_out);
}

int trapbec_step_rt(trapbec_ctx* c, int nsteps, double* t_inout) {
  if (!c || nsteps < 0) return TRAPBEC_ERR_ARG;
  int rc = finish_steps(c);
  if (rc) return rc;
  if ((rc = apply_staged(c))) return rc;
  if (t_inout) c->t = *t_inout;
  rc = DISPATCH(c, do_step_rt, c, nsteps);
  if (t_inout) *t_inout = c->t;
  return rc;
}

int trapbec_step_rt_async(trapbec_ctx* c, int nsteps, double* t_inout) {
  if (!c || nsteps < 0) return TRAPBEC_ERR_ARG;
  int rc = apply_staged(c);
  if (rc) return rc;
  if (t_inout) c->t = *t_inout;
  c->step_async = true;
  rc = DISPATCH(c, do_step_rt, c, nsteps);
  c->step_async = false;
  if (t_inout) *t_inout = c->t;
  return rc;
}

int trapbec_set_psi_async(trapbec_ctx* c, const void* psi, int layout) {
  if (!c || !psi) return TRAPBEC_ERR_ARG;
  if (layout != TRAPBEC_LAYOUT_INTERIOR) {
    set_error("trapbec_set_psi_async takes the interior layout");
    return TRAPBEC_ERR_ARG;
  }
  int rc = ensure_async(c, true, false);
  if (rc) return rc;
  if (c->stage_free_rec) CK(cudaStreamWaitEvent(c->cs_in, c->ev_stage_free, 0));
  CK(cudaMemcpyAsync(c->stage, psi, c->n * c->esz, cudaMemcpyHostToDevice, c->cs_in));
  CK(cudaEventRecord(c->ev_staged, c->cs_in));
  c->staged_pending = true;
  return TRAPBEC_OK;
}

int trapbec_get_psi_async(trapbec_ctx* c, void* psi, int layout) {
  if (!c || !psi) return TRAPBEC_ERR_ARG;
  if (layout != TRAPBEC_LAYOUT_INTERIOR) {
    set_error("trapbec_get_psi_async takes the interior layout");
    return TRAPBEC_ERR_ARG;
  }
  int rc = ensure_async(c, false, true);
  if (rc) return rc;
  if ((rc = DISPATCH(c, apply_pending_scale, c))) return rc;
  if (c->snap_drained_rec) CK(cudaStreamWaitEvent(c->st, c->ev_snap_drained, 0));
  if ((rc = copy_state(c, c->snap, c->psi[c->cur]))) return rc;
  CK(cudaEventRecord(c->ev_snap_ready, c->st));
  CK(cudaStreamWaitEvent(c->cs_out, c->ev_snap_ready, 0));
  CK(cudaMemcpyAsync(psi, c->snap, c->n * c->esz, cudaMemcpyDeviceToHost, c->cs_out));
  CK(cudaEventRecord(c->ev_snap_drained, c->cs_out));
  c->snap_drained_rec = true;
  c->out_pending = true;
  return TRAPBEC_OK;
}

int trapbec_wait_psi(trapbec_ctx* c) {
  if (!c) return TRAPBEC_ERR_ARG;
  if (c->out_pending) {
    CK(cudaEventSynchronize(c->ev_snap_drained));
    c->out_pending = false;
  }
  return TRAPBEC_OK;
}

int trapbec_synchronize(trapbec_ctx* c) {
  if (!c) return TRAPBEC_ERR_ARG;
  int rc = finish_steps(c);
  if (c->cs_in) CK(cudaStreamSynchronize(c->cs_in));
  if (c->cs_out) CK(cudaStreamSynchronize(c->cs_out));
  CK(cudaStreamSynchronize(c->st));
  c->out_pending = false;
  return rc;
}

int trapbec_step_imag(trapbec_ctx* c, int nsteps, int variant, double tol, int* steps_done, double* stat_out) {
  if (!c || nsteps < 0) return TRAPBEC_ERR_ARG;
  int sd = 0;
  double st = 0;
  int rc = finish_steps(c);
  if (rc) return rc;
  if ((rc = apply_staged(c))) return rc;
  if (variant == TRAPBEC_IMAG_REF_EULER) rc = DISPATCH(c, do_imag_euler, c, nsteps, &sd, &st);
  else if (variant == TRAPBEC_IMAG_RK3_RENORM) rc = DISPATCH(c, do_imag_rk3, c, nsteps, tol, &sd, &st);
  else { set_error("bad imaginary-time variant"); return TRAPBEC_ERR_ARG; }
  if (steps_done) *steps_done = sd;
  if (stat_out) *stat_out = st;
  return rc;
}

int trapbec_set_imag_stop(trapbec_ctx* c, int mode, double energy_scale) {
  if (!c) return TRAPBEC_ERR_ARG;
  if (mode == TRAPBEC_STOP_REL) {
    c->imag_stop = mode;
    c->imag_escale = 0.0;
    return TRAPBEC_OK;
  }
  if ((mode != TRAPBEC_STOP_ABS && mode != TRAPBEC_STOP_ABS_PER_NORM) || !(energy_scale > 0.0) ||
      !std::isfinite(energy_scale)) {
    set_error("trapbec_set_imag_stop: mode must be TRAPBEC_STOP_REL, or TRAPBEC_STOP_ABS(_PER_NORM) with a finite "
              "energy_scale > 0");
    return TRAPBEC_ERR_ARG;
  }
  c->imag_stop = mode;
  c->imag_escale = energy_scale;
  return TRAPBEC_OK;
}

}  // extern "C"
namespace {
template <typename T> int diag_impl(trapbec_ctx* c, trapbec_diag_out* o) {
  int rc = apply_pending_scale<T>(c);
  if (rc) return rc;
  if ((rc = run_diag<T>(c))) return rc;
  fill_diag<T>(c, c->host_red, o);
  return TRAPBEC_OK;
}
}  // namespace
extern "C" {

int trapbec_diag(trapbec_ctx* c, trapbec_diag_out* out) {
  if (!c || !out) return TRAPBEC_ERR_ARG;
  int rc = finish_steps(c);
  if (rc) return rc;
  return DISPATCH(c, diag_impl, c, out);
}

int trapbec_diag_async(trapbec_ctx* c) {
  if (!c) return TRAPBEC_ERR_ARG;
  return DISPATCH(c, diag_async_impl, c);
}

int trapbec_diag_wait(trapbec_ctx* c, trapbec_diag_out* out) {
  if (!c || !out) return TRAPBEC_ERR_ARG;
  if (!c->diag_pending) {
    set_error("trapbec_diag_wait: no trapbec_diag_async is pending");
    return TRAPBEC_ERR_STATE;
  }
  c->diag_pending = false;
  CK(cudaEventSynchronize(c->ev_diag));
  if (c->adiag->err != 0) {   // the flag stays set on the device: the next waiting call reports it too
    set_error("device-side wait timed out in the tiled stage kernel (code " + std::to_string(c->adiag->err) +
              ") before the diagnostics");
    return TRAPBEC_ERR_TIMEOUT;
  }
  if (c->prec == TRAPBEC_FP64) fill_diag<double>(c, c->adiag->red, out);
  else fill_diag<float>(c, c->adiag->red, out);
  return TRAPBEC_OK;
}

}  // extern "C"
namespace {
template <typename T> int field_diag_impl(trapbec_ctx* c, void* out, int which) {
  int rc = apply_pending_scale<T>(c);
  if (rc) return rc;
  const trapbec_params& p = c->p;
  DiagFieldArgs<T> a;
  a.psi = (const c_t<T>*)c->psi[c->cur];
  a.nx = p.nx; a.ny = p.ny; a.nz = p.nz;
  a.nmx = p.nx / (p.nprocx > 0 ? p.nprocx : 1);
  a.nmy = p.ny / (p.nprocy > 0 ? p.nprocy : 1);
  a.bc = p.boundaries;
  a.bcz = (p.periodicz || p.boundaries == TRAPBEC_BC_PERIODIC) ? TRAPBEC_BC_PERIODIC : p.boundaries;
  a.hx = (T)p.lx / (T)p.nx; a.hy = (T)p.ly / (T)p.ny; a.hz = (T)p.lz / (T)p.nz;   // initial.f90:26
  void* buf = nullptr;
  CK(cudaMalloc(&buf, 3 * c->n * sizeof(T)));
  a.out = (T*)buf;
  if (which == 0) velocity_kernel<T><<<simple_grid(c), SIMPLE_THREADS, 0, c->st>>>(a);
  else qpressure_kernel<T><<<simple_grid(c), SIMPLE_THREADS, 0, c->st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, buf, 3 * c->n * sizeof(T), cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  cudaFree(buf);
  c->launches++;
  if (e != cudaSuccess) { set_error(std::string("diagnostic field: ") + cudaGetErrorString(e)); return TRAPBEC_ERR_CUDA; }
  return TRAPBEC_OK;
}
}  // namespace
extern "C" {

int trapbec_set_wait_limit(trapbec_ctx* c, uint32_t limit, int inject) {
  if (!c) return TRAPBEC_ERR_ARG;
  c->wait_us = limit ? limit : 2000000u;
  c->inject_wait = inject ? 1 : 0;
  return TRAPBEC_OK;
}

int trapbec_force_vortex(trapbec_ctx* c, double x0, double y0, double dir) {
  if (!c) return TRAPBEC_ERR_ARG;
  if (dir != 1.0 && dir != -1.0) { set_error("force_vortex: dir must be +1 or -1"); return TRAPBEC_ERR_ARG; }
  c->force_args[0] = x0; c->force_args[1] = y0; c->force_args[2] = dir;
  return trapbec_init_state(c, "force_vortex", nullptr);
}

int trapbec_force_random_points(trapbec_ctx* c, uint64_t seed, uint64_t draw, double drawn[3]) {
  if (!c) return TRAPBEC_ERR_ARG;
  // runif draws of force.f90:20-28 in the context precision, from a
  // counter-based stream: draw d of seed s is reproducible on its own
  tbh::Rng rng{tbh::Rng::mix(seed ^ tbh::Rng::mix(draw + 0x632be59bd9b4e019ULL))};
  const bool f64 = c->p.precision == TRAPBEC_FP64;
  auto runif = [&](double lo, double hi) {
    if (f64) return lo + rng.next() * (hi - lo);
    const float u = (float)rng.next();
    return (double)((float)lo + u * ((float)hi - (float)lo));
  };
  const double lx = f64 ? c->p.lx : (double)(float)c->p.lx, ly = f64 ? c->p.ly : (double)(float)c->p.ly;
  const double x0 = runif(-lx / 4.0, lx / 4.0);
  const double y0 = runif(-ly / 4.0, ly / 4.0);
  const double dir = runif(0.0, 1.0) < 0.5 ? -1.0 : 1.0;
  if (drawn) { drawn[0] = x0; drawn[1] = y0; drawn[2] = dir; }
  return trapbec_force_vortex(c, x0, y0, dir);
}

int trapbec_get_velocity(trapbec_ctx* c, void* vel_out) {
  if (!c || !vel_out) return TRAPBEC_ERR_ARG;
  return DISPATCH(c, field_diag_impl, c, vel_out, 0);
}

int trapbec_get_qpressure(trapbec_ctx* c, void* qp_out) {
  if (!c || !qp_out) return TRAPBEC_ERR_ARG;
  return DISPATCH(c, field_diag_impl, c, qp_out, 1);
}

int trapbec_set_scalar(trapbec_ctx* c, int which, double v) {
  if (!c) return TRAPBEC_ERR_ARG;
  switch (which) {
    case TRAPBEC_SCALAR_OMEGA_Z: c->omega = v; c->p.omega_z = v; break;
    case TRAPBEC_SCALAR_DT_RE: c->dt_re = v; break;
    case TRAPBEC_SCALAR_DT_IM: c->dt_im = v; break;
    case TRAPBEC_SCALAR_GAMMA: c->gamma = v; break;
    case TRAPBEC_SCALAR_T: c->t = v; break;
    case TRAPBEC_SCALAR_ADVECTIVE_VX: c->vx = v; c->p.advective_vx = v; break;
    case TRAPBEC_SCALAR_NORM_TARGET: c->norm_target = v; c->norm_user = v > 0.0; break;
    default: set_error("unknown scalar"); return TRAPBEC_ERR_ARG;
  }
  return TRAPBEC_OK;
}

int trapbec_get_scalar(trapbec_ctx* c, int which, double* v) {
  if (!c || !v) return TRAPBEC_ERR_ARG;
  switch (which) {
    case TRAPBEC_SCALAR_OMEGA_Z: *v = c->omega; break;
    case TRAPBEC_SCALAR_DT_RE: *v = c->dt_re; break;
    case TRAPBEC_SCALAR_DT_IM: *v = c->dt_im; break;
    case TRAPBEC_SCALAR_GAMMA: *v = c->gamma; break;
    case TRAPBEC_SCALAR_T: *v = c->t; break;
    case TRAPBEC_SCALAR_ADVECTIVE_VX: *v = c->vx; break;
    case TRAPBEC_SCALAR_NORM_TARGET: *v = c->norm_target; break;
    default: set_error("unknown scalar"); return TRAPBEC_ERR_ARG;
  }
  return TRAPBEC_OK;
}

int trapbec_set_kernel(trapbec_ctx* c, int kind, int tile_z, int tile_y) {
  if (!c || kind < 0 || kind > 2) return TRAPBEC_ERR_ARG;
  if (kind == 1) {
    c->kernel_kind = 1;
    return TRAPBEC_OK;
  }
  int shape = 0;   // the context changes only once the request is valid
  const int ns = c->prec == TRAPBEC_FP64 ? tiled_nshapes<double>() : tiled_nshapes<float>();
  if (tile_z < 0) {  // select a built shape by index: tile_z = -(index + 1)
    shape = -tile_z - 1;
    if (shape >= ns) { set_error("no tiled kernel shape with this index"); return TRAPBEC_ERR_UNSUPPORTED; }
  } else if (tile_z || tile_y) {
    shape = -1;
    for (int i = 0; i < ns && shape < 0; ++i) {
      Shape sh = c->prec == TRAPBEC_FP64 ? tiled_shape<double>(i) : tiled_shape<float>(i);
      if (sh.tz == tile_z && sh.ty == tile_y) shape = i;
    }
    if (shape < 0) {
      set_error("no tiled kernel is built for this tile shape");
      return TRAPBEC_ERR_UNSUPPORTED;
    }
  }
  // an explicit shape serves every launch; the default picks the first shape
  // that plans for the general launches and the real-time shape for the rest
  const bool expl = tile_z || tile_y;
  const int shape_rt = expl ? shape : -1;
  if (!expl) shape = -1;
  c->tile_z = tile_z;
  c->tile_y = tile_y;
  if (c->prec == TRAPBEC_FP64) make_plans<double>(c, shape, shape_rt);
  else make_plans<float>(c, shape, shape_rt);
  if (kind == 2 && !c->plan_valid) {
    set_error("tiled kernel not available for this grid / tile shape");
    return TRAPBEC_ERR_UNSUPPORTED;
  }
  c->kernel_kind = kind;
  return TRAPBEC_OK;
}

int trapbec_set_chunk(trapbec_ctx* c, int chunk) {
  if (!c || chunk == INT_MIN) return TRAPBEC_ERR_ARG;
  c->chunk_user = chunk;
  if (c->plan_valid) { c->plan.chunk = auto_chunk(c); c->plan.chunk_s1 = 0; }
  if (c->plan_rt_valid) { c->plan_rt.chunk = auto_chunk(c); c->plan_rt.chunk_s1 = 0; }
  return TRAPBEC_OK;
}

int trapbec_get_tile_shape(trapbec_ctx* c, int real_time, int* tile_z, int* tile_y) {
  if (!c || !tile_z || !tile_y) return TRAPBEC_ERR_ARG;
  const bool valid = c->kernel_kind != 1 && (real_time ? c->plan_rt_valid : c->plan_valid);
  const TiledPlan& pl = real_time ? c->plan_rt : c->plan;
  *tile_z = valid ? pl.tz : 0;
  *tile_y = valid ? pl.ty : 0;
  return TRAPBEC_OK;
}

int trapbec_set_stage_form(trapbec_ctx* c, int form) {
  if (!c || (form != TRAPBEC_RK3_THREE_STAGE && form != TRAPBEC_RK3_DEFERRED && form != TRAPBEC_RK3_COMPENSATED &&
             form != TRAPBEC_RK3_PSI_DIFF))
    return TRAPBEC_ERR_ARG;
  if (form == TRAPBEC_RK3_COMPENSATED) {
    if (c->prec != TRAPBEC_FP32) {
      set_error("the compensated form is for FP32 contexts (an FP64 state keeps its increments)");
      return TRAPBEC_ERR_UNSUPPORTED;
    }
    if (!c->lo) {
      CK(cudaMalloc(&c->lo, c->n * c->esz));
      c->lo_valid = false;
    }
  }
  if (form != c->stage_form) psi_changed(c);
  c->stage_form = form;
  if (form == TRAPBEC_RK3_DEFERRED && c->prec == TRAPBEC_FP32 && !c->p.two_dim && !c->w2) {
    // the second w buffer, then plans that know it
    CK(cudaMalloc(&c->w2, c->n * c->esz));
    CK(cudaMemsetAsync(c->w2, 0, c->n * c->esz, c->st));
    CK(cudaStreamSynchronize(c->st));
    make_plans<float>(c, c->shape, c->shape_rt);
  }
  return TRAPBEC_OK;
}

int trapbec_get_stage_form(trapbec_ctx* c, int* form) {
  if (!c || !form) return TRAPBEC_ERR_ARG;
  StageArgs<float> a;
  std::memset(&a, 0, sizeof(a));
  bool plain = true;
  if (c->prec == TRAPBEC_FP32) {
    a = base_args<float>(c, c->t);
    plain = tiled_plain(a);
  }
  if (c->stage_form == TRAPBEC_RK3_COMPENSATED) {
    *form = TRAPBEC_RK3_COMPENSATED;   // or the step reports TRAPBEC_ERR_UNSUPPORTED
    return TRAPBEC_OK;
  }
  if (c->prec == TRAPBEC_FP64) {
    StageArgs<double> a64 = base_args<double>(c, c->t);
    plain = tiled_plain(a64);
  }
  const bool tiled_rt = c->kernel_kind != 1 && c->plan_rt_valid && plain;
  if (c->stage_form == TRAPBEC_RK3_PSI_DIFF && tiled_rt && c->plan_rt.pdiff_ok) {
    *form = TRAPBEC_RK3_PSI_DIFF;
    return TRAPBEC_OK;
  }
  *form = (c->stage_form == TRAPBEC_RK3_DEFERRED && c->prec == TRAPBEC_FP32 && tiled_rt && c->plan_rt.defer_ok)
              ? TRAPBEC_RK3_DEFERRED
              : TRAPBEC_RK3_THREE_STAGE;
  return TRAPBEC_OK;
}

}  // extern "C"
namespace {
struct TuneKey {
  trapbec_params p;
  bool operator==(const TuneKey& o) const { return std::memcmp(&p, &o.p, sizeof(p)) == 0; }
};
struct TuneVal { int shape, chunk, chunk_s1; double ms; };
std::vector<std::pair<TuneKey, TuneVal>> g_tune_cache;
std::mutex g_tune_mu;

template <typename T> int autotune_impl(trapbec_ctx* c, int steps, TuneVal* best) {
  TuneKey key;
  std::memset(&key.p, 0, sizeof(key.p));
  key.p.nx = c->p.nx; key.p.ny = c->p.ny; key.p.nz = c->p.nz;
  key.p.precision = c->p.precision; key.p.boundaries = c->p.boundaries; key.p.periodicz = c->p.periodicz;
  key.p.potential = c->p.potential;
  key.p.reserved[0] = c->stage_form;   // each form is timed on its own (the compensated one on other shapes)
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (auto& kv : g_tune_cache)
      if (kv.first == key) { *best = kv.second; return TRAPBEC_OK; }
  }
  // save the state (both buffers: psi and w) and the time
  void* save = nullptr;
  CK(cudaMalloc(&save, c->n * c->esz));
  CK(cudaMemcpyAsync(save, c->psi[c->cur], c->n * c->esz, cudaMemcpyDeviceToDevice, c->st));
  const double t_save = c->t;
  const int cur_save = c->cur;
  TuneVal bv{-1, 0, 0, 1e300};
  const int ns = tiled_nshapes<T>();
  int rc = TRAPBEC_OK;
  for (int sh = 0; sh < ns && rc == TRAPBEC_OK; ++sh) {
    TiledPlan plan;
    if (plan_tiled<T>(c->p, c->psi, c->w, c->w2, c->nsm, sh, c->d_err, &plan) != 0) continue;
    if (c->stage_form == TRAPBEC_RK3_COMPENSATED && !plan.comp_ok) continue;
    if (c->stage_form == TRAPBEC_RK3_PSI_DIFF && !plan.pdiff_ok) continue;
    // contiguous unit ranges per CTA (chunk > 0) and the strided order (chunk < 0)
    std::vector<int> chunks = {16, 32, 64, c->p.nx, -64, -128, -256};
    for (int L : chunks) {
      if (L > c->p.nx || -L > c->p.nx) continue;
      plan.chunk = L;
      c->plan_rt = plan;
      c->plan_rt_valid = true;
      c->kernel_kind = 2;
      if ((rc = do_step_rt<T>(c, 1))) break;     // warm-up
      if ((rc = do_step_rt<T>(c, steps))) break;
      double ms = c->last_ms / steps;
      if (ms < bv.ms) bv = TuneVal{sh, L, 0, ms};
      CK(cudaMemcpyAsync(c->psi[cur_save], save, c->n * c->esz, cudaMemcpyDeviceToDevice, c->st));
      c->cur = cur_save;
      c->t = t_save;
    }
  }
  // On the best shape, the stage-1 kinds in the contiguous tile-major order
  // and the other stages in the strided one: the stage-1 kinds are not bound
  // by HBM and pay for the strided order's extra segment starts more than
  // they gain from its L2 reuse.
  if (rc == TRAPBEC_OK && bv.shape >= 0) {
    TiledPlan plan;
    if (plan_tiled<T>(c->p, c->psi, c->w, c->w2, c->nsm, bv.shape, c->d_err, &plan) == 0) {
      for (int L : {-64, -128, -256}) {
        if (-L > c->p.nx) continue;
        plan.chunk = L;
        plan.chunk_s1 = c->p.nx;
        c->plan_rt = plan;
        c->plan_rt_valid = true;
        c->kernel_kind = 2;
        if ((rc = do_step_rt<T>(c, 1)) || (rc = do_step_rt<T>(c, steps))) break;
        const double ms = c->last_ms / steps;
        if (ms < bv.ms) bv = TuneVal{bv.shape, L, c->p.nx, ms};
        CK(cudaMemcpyAsync(c->psi[cur_save], save, c->n * c->esz, cudaMemcpyDeviceToDevice, c->st));
        c->cur = cur_save;
        c->t = t_save;
      }
    }
  }
  CK(cudaMemcpyAsync(c->psi[cur_save], save, c->n * c->esz, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  cudaFree(save);
  c->cur = cur_save;
  c->t = t_save;
  c->kernel_kind = 0;
  psi_changed(c);
  if (rc) return rc;
  if (bv.shape < 0) { set_error("no tiled kernel shape fits this grid"); return TRAPBEC_ERR_UNSUPPORTED; }
  if (plan_tiled<T>(c->p, c->psi, c->w, c->w2, c->nsm, bv.shape, c->d_err, &c->plan_rt) != 0) return TRAPBEC_ERR_CUDA;
  c->plan_rt.chunk = bv.chunk;
  c->plan_rt.chunk_s1 = bv.chunk_s1;
  c->plan_rt_valid = true;
  c->shape_rt = bv.shape;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache.push_back({key, bv});
  }
  *best = bv;
  return TRAPBEC_OK;
}
}  // namespace
extern "C" {

int trapbec_autotune(trapbec_ctx* c, int steps, int* tile_z, int* tile_y, int* chunk, double* ms_per_step) {
  if (!c || steps < 1) return TRAPBEC_ERR_ARG;
  TuneVal bv;
  int rc = finish_steps(c);
  if (rc) return rc;
  rc = DISPATCH(c, autotune_impl, c, steps, &bv);
  if (rc) return rc;
  if (!c->plan_rt_valid || c->plan_rt.shape != bv.shape) {   // a cached choice
    int r2 = c->prec == TRAPBEC_FP64 ? plan_tiled<double>(c->p, c->psi, c->w, c->w2, c->nsm, bv.shape, c->d_err, &c->plan_rt)
                                     : plan_tiled<float>(c->p, c->psi, c->w, c->w2, c->nsm, bv.shape, c->d_err, &c->plan_rt);
    if (r2) return TRAPBEC_ERR_CUDA;
    c->plan_rt_valid = true;
    c->shape_rt = bv.shape;
  }
  c->plan_rt.chunk = bv.chunk;
  c->plan_rt.chunk_s1 = bv.chunk_s1;
  Shape sh = c->prec == TRAPBEC_FP64 ? tiled_shape<double>(bv.shape) : tiled_shape<float>(bv.shape);
  if (tile_z) *tile_z = sh.tz;
  if (tile_y) *tile_y = sh.ty;
  if (chunk) *chunk = bv.chunk;
  if (ms_per_step) *ms_per_step = bv.ms;
  return TRAPBEC_OK;
}

int trapbec_launch_count(trapbec_ctx* c, int64_t* count) {
  if (!c || !count) return TRAPBEC_ERR_ARG;
  *count = c->launches;
  return TRAPBEC_OK;
}

int trapbec_last_kernel_ms(trapbec_ctx* c, double* ms) {
  if (!c || !ms) return TRAPBEC_ERR_ARG;
  int rc = finish_steps(c);
  if (rc) return rc;
  *ms = c->last_ms;
  return TRAPBEC_OK;
}

// ------------------------------------------------------------------ I/O ---
int trapbec_write_var(trapbec_ctx* c, const char* datadir, int itime, int shots, double t, int imaginary) {
  if (!c || !datadir || shots <= 0) return TRAPBEC_ERR_ARG;
  std::vector<char> buf(c->n * c->esz);
  int rc = trapbec_get_psi(c, buf.data(), TRAPBEC_LAYOUT_INTERIOR);
  if (rc) return rc;
  return trapbec_write_var_host(&c->p, datadir, itime, shots, t, imaginary, buf.data());
}

int trapbec_write_field(trapbec_ctx* c, const char* datadir, int itime, int shots, int which) {
  if (!c || !datadir || shots <= 0 || (which != TRAPBEC_FIELD_VELOCITY && which != TRAPBEC_FIELD_QPRESSURE))
    return TRAPBEC_ERR_ARG;
  const size_t rsz = c->p.precision == TRAPBEC_FP64 ? 8 : 4;
  std::vector<char> buf(3 * c->n * rsz);
  int rc = which == TRAPBEC_FIELD_VELOCITY ? trapbec_get_velocity(c, buf.data()) : trapbec_get_qpressure(c, buf.data());
  if (rc) return rc;
  // output.f90:81,87 name the files with an i2.2 edit descriptor, which
  // prints "**" once itime/shots passes 99
  const int q = itime / shots;
  char num[8];
  if (q >= 0 && q <= 99) std::snprintf(num, sizeof(num), "%02d", q);
  else std::snprintf(num, sizeof(num), "**");
  const std::string name = std::string(datadir) + "/proc000/" +
                           (which == TRAPBEC_FIELD_VELOCITY ? "vel" : "qpress") + num + ".dat";
  return tbh::write_field_file(name, buf.data(), buf.size());
}

int trapbec_write_restart(trapbec_ctx* c, const char* datadir, int itime, double t) {
  if (!c || !datadir) return TRAPBEC_ERR_ARG;
  std::vector<char> buf(c->n * c->esz);
  int rc = trapbec_get_psi(c, buf.data(), TRAPBEC_LAYOUT_INTERIOR);
  if (rc) return rc;
  return trapbec_write_restart_host(&c->p, datadir, itime, t, buf.data());
}

int trapbec_host_alloc(size_t bytes, void** out) {
  if (!out || bytes == 0) return TRAPBEC_ERR_ARG;
  *out = nullptr;
  const cudaError_t e = cudaMallocHost(out, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    set_error(std::string("trapbec_host_alloc: ") + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TRAPBEC_ERR_NOMEM : TRAPBEC_ERR_CUDA;
  }
  return TRAPBEC_OK;
}

void trapbec_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int trapbec_read_restart(trapbec_ctx* c, const char* datadir, int* nstart, double* t) {
  if (!c || !datadir || !nstart || !t) return TRAPBEC_ERR_ARG;
  int rc0 = finish_steps(c);
  if (rc0) return rc0;
  c->staged_pending = false;   // the restart state replaces a queued one
  // The reference reader looks in proc%02d (initial.f90:44,800) while the
  // writer uses proc%03d (output.f90:103); accept both, proc000 first.
  std::vector<char> buf(c->n * c->esz);
  std::string d(datadir);
  int rc = tbh::read_restart_file(d + "/proc000/var.dat", &c->p, nstart, t, buf.data(), buf.size());
  if (rc) rc = tbh::read_restart_file(d + "/proc00/var.dat", &c->p, nstart, t, buf.data(), buf.size());
  if (rc) return rc;
  c->t = *t;
  return trapbec_set_psi(c, buf.data(), TRAPBEC_LAYOUT_INTERIOR);
}

}  // extern "C"
