// batch.cu -- many independent imaginary-time ground-state solves in one
// persistent launch per RK3 stage.
//
// Each instance is its own grid (size, box, harmonic trap, rotation, step):
// psi[2], w, coordinate and potential tables, and a TMA descriptor set.  A
// descriptor table (InstDesc) holds, per instance and per step parity, the
// arguments of the three stages.  One launch of the tiled stage kernel in
// BATCH mode walks the concatenated (tile, x-plane) units of all active
// instances, split evenly over a persistent grid; a segment picks up its
// instance's arguments and tensor maps from the table.  The fused reductions
// (energy of the incoming state in stage 1, norm of the new state in stage 3)
// land in per-(CTA, segment) slots tagged with the instance; one block per
// instance then combines its slots in a fixed order and updates that
// instance's control block (renormalisation factor, energy, |dE|/|E|,
// convergence), exactly as the single-grid loop does.  A converged instance's
// segments become no-ops.  The K-step loop (3 stage launches and 2 finalisers
// per step) is captured once in a CUDA graph and replayed;
// between replays the host drops converged instances from the work list, so
// the load stays balanced over the remaining ones.  The tile shape is picked
// by timing every built shape on the actual batch (autotuner).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../include/trapbec.h"
#include "host_coords.h"
#include "host_util.h"
#include "imag_ctrl.cuh"
#include "kernels_init.cuh"
#include "tiled_impl.cuh"

using namespace tb;
using tbh::set_error;

#define BCK(call)                                                                           \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                        \
      return e_ == cudaErrorMemoryAllocation ? TRAPBEC_ERR_NOMEM : TRAPBEC_ERR_CUDA;        \
    }                                                                                       \
  } while (0)

namespace {

constexpr int BATCH_SMAX = 8;        // partial slots per CTA (segments per CTA per launch)
constexpr int BATCH_NSHAPES_F32 = 2; // (64,8) and (128,8) tiles
constexpr int BATCH_NSHAPES_F64 = 1; // (32,8)

struct BInst {
  trapbec_params p;
  size_t n = 0;
  void* psi[2] = {nullptr, nullptr};
  void* w = nullptr;
  void *xx = nullptr, *yy = nullptr, *zz = nullptr, *px = nullptr, *py = nullptr, *pz = nullptr;
  int cur = 0;         // buffer holding the state
  int steps = 0;       // steps taken in the current solve
  int prev_step = 0;   // ctrl.step seen at the last check
  double dV = 0.0;
  long long units = 0; // work units of this instance for the current shape
  int ntz = 0, nty = 0;
  double escale = 0.0; // energy scale of the absolute stop tests
};

}  // namespace

struct trapbec_batch {
  int prec = TRAPBEC_FP32;
  int stop_mode = TRAPBEC_STOP_REL;   // trapbec_imag_stop of later solves
  int ninst = 0;
  int nsm = 0;
  size_t esz = 8, rsz = 4;
  cudaStream_t st = nullptr;
  std::vector<BInst> in;
  void* d_desc = nullptr;       // InstDesc<T>[ninst]
  std::vector<unsigned char> h_desc;
  size_t desc_size = 0;
  ImagCtrl* d_ctrl = nullptr;
  ImagCtrl* h_ctrl = nullptr;   // pinned
  long long* d_ustart = nullptr;
  long long* h_ustart = nullptr;
  int* d_act = nullptr;
  int* h_act = nullptr;
  double* d_part = nullptr;
  int* d_tag = nullptr;
  int* d_err = nullptr;
  int* h_err = nullptr;
  int max_grid = 0;
  int shape = -1;               // chosen batch shape
  int grid = 0;                 // persistent grid of that shape
  cudaGraphExec_t gexec = nullptr;
  int graph_k = 0, graph_shape = -1;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double solve_ms = 0.0;
  int64_t launches = 0;
};

namespace {

template <typename T> struct BShape;
// FP32 shapes of the batch
template <int I> struct BShapeF32;
template <> struct BShapeF32<0> { static constexpr int TZ = 64, TY = 8, R = 2; };
template <> struct BShapeF32<1> { static constexpr int TZ = 128, TY = 8, R = 2; };
struct BShapeF64 { static constexpr int TZ = 32, TY = 8, R = 2; };

// The batch runs the imaginary-time variant of the stage kernel: every
// instance has a harmonic or no potential, a rotating or no frame and the
// fixed reductions of the imaginary-time loop (fill_desc).
template <typename T, int TZ, int TY, int R> struct BK {
  using G = TileGeom<T, TZ, TY, R, 8, 0>;
  static int prepare(int nsm, int* grid) {
    auto k1 = stage_tiled_kernel<T, TZ, TY, R, 8, 0, ST_S1, VAR_IMAG, true>;
    auto k2 = stage_tiled_kernel<T, TZ, TY, R, 8, 0, ST_S2, VAR_IMAG, true>;
    auto k3 = stage_tiled_kernel<T, TZ, TY, R, 8, 0, ST_S3, VAR_IMAG, true>;
    if (cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, KindGeom<T, G, ST_S1>::SMEM) != cudaSuccess)
      return 1;
    for (auto k : {k2, k3})
      if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM) != cudaSuccess) return 1;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k2, G::NT, G::SMEM) != cudaSuccess || nb < 1) return 1;
    *grid = nb * nsm;
    return 0;
  }
  static void launch(int kind, const BatchArgs& ba, int grid, cudaStream_t st) {
    TiledArgs<T> dummy;
    std::memset(&dummy, 0, sizeof(dummy));
    CUtensorMap dm;
    std::memset(&dm, 0, sizeof(dm));
    if (kind == ST_S1) stage_tiled_kernel<T, TZ, TY, R, 8, 0, ST_S1, VAR_IMAG, true><<<grid, G::NT, KindGeom<T, G, ST_S1>::SMEM, st>>>(dm, dm, dummy, ba);
    else if (kind == ST_S2) stage_tiled_kernel<T, TZ, TY, R, 8, 0, ST_S2, VAR_IMAG, true><<<grid, G::NT, KindGeom<T, G, ST_S2>::SMEM, st>>>(dm, dm, dummy, ba);
    else stage_tiled_kernel<T, TZ, TY, R, 8, 0, ST_S3, VAR_IMAG, true><<<grid, G::NT, KindGeom<T, G, ST_S3>::SMEM, st>>>(dm, dm, dummy, ba);
  }
  static int encode(const trapbec_params& p, void* const psi[2], void* w, CUtensorMap* tm, CUtensorMap* tmw) {
    return encode_maps<T, TZ, TY, R, 8, 0>(p, psi, w, tm, tmw);
  }
};

template <typename T> int shape_tz(int s) {
  if (sizeof(T) == 8) return BShapeF64::TZ;
  return s == 0 ? BShapeF32<0>::TZ : BShapeF32<1>::TZ;
}
template <typename T> int shape_ty(int s) {
  if (sizeof(T) == 8) return BShapeF64::TY;
  return s == 0 ? BShapeF32<0>::TY : BShapeF32<1>::TY;
}

template <typename T> int shape_prepare(int s, int nsm, int* grid) {
  if (sizeof(T) == 8) return BK<double, BShapeF64::TZ, BShapeF64::TY, BShapeF64::R>::prepare(nsm, grid);
  if (s == 0) return BK<float, BShapeF32<0>::TZ, BShapeF32<0>::TY, BShapeF32<0>::R>::prepare(nsm, grid);
  return BK<float, BShapeF32<1>::TZ, BShapeF32<1>::TY, BShapeF32<1>::R>::prepare(nsm, grid);
}
template <typename T> void shape_launch(int s, int kind, const BatchArgs& ba, int grid, cudaStream_t st) {
  if (sizeof(T) == 8) BK<double, BShapeF64::TZ, BShapeF64::TY, BShapeF64::R>::launch(kind, ba, grid, st);
  else if (s == 0) BK<float, BShapeF32<0>::TZ, BShapeF32<0>::TY, BShapeF32<0>::R>::launch(kind, ba, grid, st);
  else BK<float, BShapeF32<1>::TZ, BShapeF32<1>::TY, BShapeF32<1>::R>::launch(kind, ba, grid, st);
}
template <typename T> int shape_encode(int s, const trapbec_params& p, void* const psi[2], void* w, CUtensorMap* tm,
                                       CUtensorMap* tmw) {
  if (sizeof(T) == 8) return BK<double, BShapeF64::TZ, BShapeF64::TY, BShapeF64::R>::encode(p, psi, w, tm, tmw);
  if (s == 0) return BK<float, BShapeF32<0>::TZ, BShapeF32<0>::TY, BShapeF32<0>::R>::encode(p, psi, w, tm, tmw);
  return BK<float, BShapeF32<1>::TZ, BShapeF32<1>::TY, BShapeF32<1>::R>::encode(p, psi, w, tm, tmw);
}

// Per-instance finalisers: block i combines the partial slots tagged i in slot
// order (fixed partition per thread, fixed tree) and updates ctrl[i].
__device__ void gather_instance(const double* __restrict__ part, const int* __restrict__ tag, int nslots, int inst,
                                double* out /* shared NRED */) {
  FinAcc a;
  a.init();
  for (int b = threadIdx.x; b < nslots; b += FIN_THREADS) {
    if (tag[b] != inst) continue;
    double v[NRED];
#pragma unroll
    for (int q = 0; q < NRED; ++q) v[q] = part[(size_t)b * NRED + q];
    a.add(v);
  }
  fin_tree(a, out);
}

// FP32 batches: the stage kernel stores each slot's sums as float-float
// pairs (block_reduce_sums with FFOUT), so the finaliser combines them in FP32
// arithmetic (one fixed pairwise tree, as fin_tree) and only its nine results
// and the control update are FP64: GB300 issues FP64 at about one lane
// operation per SM clock, which made the FP64 finaliser a large share of a
// small batch's step.
__device__ void gather_instance_ff(const double* __restrict__ part, const int* __restrict__ tag, int nslots, int inst,
                                   double* out /* shared NRED */) {
  __shared__ FF shf[6][FIN_THREADS];
  __shared__ float shm[3][FIN_THREADS];
  FF acc[6];
#pragma unroll
  for (int q = 0; q < 6; ++q) acc[q].hi = acc[q].lo = 0.f;
  float mx = 0.f, mn = 3.0e38f, nf = 0.f;
  const float2* pf = reinterpret_cast<const float2*>(part);
  auto take = [&](int b) {
    const float2* v = pf + (size_t)b * NRED;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const float2 x = v[q];
      FF y;
      y.hi = x.x;
      y.lo = x.y;
      acc[q] = ff_add(acc[q], y);
    }
    mx = fmaxf(mx, v[6].x);
    mn = fminf(mn, v[7].x);
    nf = fmaxf(nf, v[8].x);
  };
  // the tags of a thread's first GATHER_UNROLL slots are loaded together
  // (one memory latency instead of one per slot), then the matching slots
  // are combined in slot order; slots beyond that (large grids) follow
  constexpr int GATHER_UNROLL = 8;
  int tg[GATHER_UNROLL];
#pragma unroll
  for (int i = 0; i < GATHER_UNROLL; ++i) {
    const int b = threadIdx.x + i * FIN_THREADS;
    tg[i] = b < nslots ? tag[b] : -1;
  }
#pragma unroll
  for (int i = 0; i < GATHER_UNROLL; ++i)
    if (tg[i] == inst) take(threadIdx.x + i * FIN_THREADS);
  for (int b = threadIdx.x + GATHER_UNROLL * FIN_THREADS; b < nslots; b += FIN_THREADS)
    if (tag[b] == inst) take(b);
  const int t = threadIdx.x;
#pragma unroll
  for (int q = 0; q < 6; ++q) shf[q][t] = acc[q];
  shm[0][t] = mx;
  shm[1][t] = mn;
  shm[2][t] = nf;
  __syncthreads();
  for (int s = FIN_THREADS / 2; s >= 32; s >>= 1) {
    if (t < s) {
#pragma unroll
      for (int q = 0; q < 6; ++q) shf[q][t] = ff_add(shf[q][t], shf[q][t + s]);
      shm[0][t] = fmaxf(shm[0][t], shm[0][t + s]);
      shm[1][t] = fminf(shm[1][t], shm[1][t + s]);
      shm[2][t] = fmaxf(shm[2][t], shm[2][t + s]);
    }
    __syncthreads();
  }
  if (t < 32) {
    FF x[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) x[q] = shf[q][t];
    float a = shm[0][t], b = shm[1][t], c = shm[2][t];
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        FF y;
        y.hi = __shfl_down_sync(0xffffffffu, x[q].hi, s);
        y.lo = __shfl_down_sync(0xffffffffu, x[q].lo, s);
        x[q] = ff_add(x[q], y);
      }
      a = fmaxf(a, __shfl_down_sync(0xffffffffu, a, s));
      b = fminf(b, __shfl_down_sync(0xffffffffu, b, s));
      c = fmaxf(c, __shfl_down_sync(0xffffffffu, c, s));
    }
    if (t == 0) {
#pragma unroll
      for (int q = 0; q < 6; ++q) out[q] = (double)x[q].hi + (double)x[q].lo;
      out[6] = a;
      out[7] = b;
      out[8] = c;
    }
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(FIN_THREADS) batch_fin_energy_kernel(const double* __restrict__ part,
                                                                       const int* __restrict__ tag, int nslots,
                                                                       const int* __restrict__ act, int nact,
                                                                       ImagCtrl* ctrl) {
  if ((int)blockIdx.x >= nact) return;
  const int inst = act[blockIdx.x];
  ImagCtrl* c = ctrl + inst;
  if (c->converged || c->nonfinite) return;
  __shared__ double r[NRED];
  if constexpr (sizeof(T) == 4) gather_instance_ff(part, tag, nslots, inst, r);
  else gather_instance(part, tag, nslots, inst, r);
  if (threadIdx.x == 0) imag_energy_update(r, c);
}

template <typename T>
__global__ void __launch_bounds__(FIN_THREADS) batch_fin_norm_kernel(const double* __restrict__ part,
                                                                     const int* __restrict__ tag, int nslots,
                                                                     const int* __restrict__ act, int nact,
                                                                     ImagCtrl* ctrl) {
  if ((int)blockIdx.x >= nact) return;
  const int inst = act[blockIdx.x];
  ImagCtrl* c = ctrl + inst;
  if (c->converged || c->nonfinite) return;
  __shared__ double r[NRED];
  if constexpr (sizeof(T) == 4) gather_instance_ff(part, tag, nslots, inst, r);
  else gather_instance(part, tag, nslots, inst, r);
  if (threadIdx.x == 0) imag_norm_update(r, c);
}

// Fill the descriptor of instance i for shape s: tensor maps and, for both
// step parities, the three stage argument sets.
template <typename T> int fill_desc(trapbec_batch* b, int i, int s) {
  BInst& I = b->in[i];
  InstDesc<T>* d = reinterpret_cast<InstDesc<T>*>(b->h_desc.data()) + i;
  std::memset(d, 0, sizeof(*d));
  if (shape_encode<T>(s, I.p, I.psi, I.w, d->tm, &d->tmw)) {
    set_error("batch: TMA descriptor encoding failed");
    return TRAPBEC_ERR_CUDA;
  }
  d->buf0 = I.psi[0];
  const trapbec_params& p = I.p;
  const int TZ = shape_tz<T>(s), TY = shape_ty<T>(s);
  I.ntz = (p.nz + TZ - 1) / TZ;
  I.nty = (p.ny + TY - 1) / TY;
  I.units = (long long)I.ntz * I.nty * p.nx;
  const T hx = (T)p.lx / (T)p.nx, hy = (T)p.ly / (T)p.ny, hz = (T)p.lz / (T)p.nz;
  const T eps = std::numeric_limits<T>::epsilon();
  for (int par = 0; par < 2; ++par) {
    for (int st = 0; st < 3; ++st) {
      TiledArgs<T>& ta = d->ta[par][st];
      StageArgs<T>& a = ta.s;
      // at parity par the step starts from buffer cur ^ par; stages alternate buffers
      const int in0 = I.cur ^ par;
      const int in = (st == 1) ? (in0 ^ 1) : in0;
      a.psi_in = (const c_t<T>*)I.psi[in];
      a.psi_out = (c_t<T>*)I.psi[in ^ 1];
      a.w = (c_t<T>*)I.w;
      a.xx = (const T*)I.xx; a.yy = (const T*)I.yy; a.zz = (const T*)I.zz;
      a.px = (const T*)I.px; a.py = (const T*)I.py; a.pz = (const T*)I.pz;
      a.trap = nullptr;
      a.red = nullptr;
      a.nx = p.nx; a.ny = p.ny; a.nz = p.nz;
      a.bc = p.boundaries;
      a.zper = 0;
      a.two_dim = 0;
      a.pot_mode = p.potential == TRAPBEC_POT_HARMONIC ? POT_HARM : POT_NONE;
      a.frame_mode = std::fabs((T)p.omega_z) > eps ? FRAME_ROT : FRAME_NONE;
      a.omega = (T)p.omega_z;
      a.reduce = st == 0 ? 2 : (st == 2 ? 1 : 0);
      a.ix2 = (T)1 / ((T)180 * (hx * hx));
      a.iy2 = (T)1 / ((T)180 * (hy * hy));
      a.iz2 = (T)1 / ((T)180 * (hz * hz));
      a.ix1 = (T)1 / ((T)60 * hx);
      a.iy1 = (T)1 / ((T)60 * hy);
      a.c_re = (T)0.5 * (T)p.dt_re;   // d psi / d tau = rhs / 2
      a.c_im = 0;
      a.A = st == 0 ? (T)0 : (st == 1 ? (T)(-2.) / (T)3. : (T)(-1));
      a.B = st == 0 ? (T)1 / (T)3 : (st == 1 ? (T)1 : (T)0.5);
      a.scale = 1;
      a.ctrl = b->d_ctrl + i;
      a.use_ctrl_scale = st == 0 ? 1 : 0;
      ta.ntz = I.ntz;
      ta.nty = I.nty;
      ta.units = I.units;
      ta.err = b->d_err;
      ta.bcz = TRAPBEC_BC_ZERO;
      ta.fix_y = 0;
      ta.fix_z = 0;
      ta.chunk = p.nx;
      ta.wait_us = WAIT_US_DEFAULT;
      ta.inject_wait = 0;
      fill_coeffs<T>(ta);
    }
  }
  return TRAPBEC_OK;
}

template <typename T> int create_impl(trapbec_batch* b) {
  for (int i = 0; i < b->ninst; ++i) {
    BInst& I = b->in[i];
    const trapbec_params& p = I.p;
    I.n = (size_t)p.nx * p.ny * p.nz;
    BCK(cudaMalloc(&I.psi[0], I.n * b->esz));
    BCK(cudaMalloc(&I.psi[1], I.n * b->esz));
    BCK(cudaMalloc(&I.w, I.n * b->esz));
    BCK(cudaMemsetAsync(I.psi[0], 0, I.n * b->esz, b->st));
    BCK(cudaMemsetAsync(I.psi[1], 0, I.n * b->esz, b->st));
    std::vector<T> xx, yy, zz, px, py, pz;
    tbh::make_coords<T>(p, xx, yy, zz);
    tbh::make_harm_tables<T>(p, xx, yy, zz, px, py, pz);
    void** bufs[6] = {&I.xx, &I.yy, &I.zz, &I.px, &I.py, &I.pz};
    const std::vector<T>* src[6] = {&xx, &yy, &zz, &px, &py, &pz};
    for (int k = 0; k < 6; ++k) {
      BCK(cudaMalloc(bufs[k], sizeof(T) * src[k]->size()));
      BCK(cudaMemcpy(*bufs[k], src[k]->data(), sizeof(T) * src[k]->size(), cudaMemcpyHostToDevice));
    }
    const double hx = (double)((T)p.lx / (T)p.nx), hy = (double)((T)p.ly / (T)p.ny), hz = (double)((T)p.lz / (T)p.nz);
    I.dV = hx * hy * hz;
  }
  b->desc_size = sizeof(InstDesc<T>);
  b->h_desc.assign(b->desc_size * b->ninst, 0);
  BCK(cudaMalloc(&b->d_desc, b->desc_size * b->ninst));
  BCK(cudaMalloc(&b->d_ctrl, sizeof(ImagCtrl) * b->ninst));
  BCK(cudaMallocHost(&b->h_ctrl, sizeof(ImagCtrl) * b->ninst));
  std::memset(b->h_ctrl, 0, sizeof(ImagCtrl) * b->ninst);
  BCK(cudaMalloc(&b->d_ustart, sizeof(long long) * (b->ninst + 1)));
  BCK(cudaMallocHost(&b->h_ustart, sizeof(long long) * (b->ninst + 1)));
  BCK(cudaMalloc(&b->d_act, sizeof(int) * b->ninst));
  BCK(cudaMallocHost(&b->h_act, sizeof(int) * b->ninst));
  BCK(cudaMalloc(&b->d_err, sizeof(int)));
  BCK(cudaMallocHost(&b->h_err, sizeof(int)));
  BCK(cudaMemset(b->d_err, 0, sizeof(int)));
  // the largest persistent grid over the shapes sizes the partial slots
  const int ns = sizeof(T) == 8 ? BATCH_NSHAPES_F64 : BATCH_NSHAPES_F32;
  b->max_grid = 0;
  for (int s = 0; s < ns; ++s) {
    int g = 0;
    if (shape_prepare<T>(s, b->nsm, &g)) { set_error("batch: kernel set-up failed"); return TRAPBEC_ERR_CUDA; }
    b->max_grid = std::max(b->max_grid, g);
  }
  const size_t nslots = (size_t)b->max_grid * BATCH_SMAX;
  BCK(cudaMalloc(&b->d_part, sizeof(double) * NRED * nslots));
  BCK(cudaMalloc(&b->d_tag, sizeof(int) * nslots));
  BCK(cudaMemset(b->d_tag, 0xff, sizeof(int) * nslots));
  BCK(cudaStreamSynchronize(b->st));
  return TRAPBEC_OK;
}

// One replay's worth of steps.  nact instances are active; the kernels read
// the work list from the device tables, the instance count is a launch
// argument, so the graph is rebuilt when it changes.
template <typename T> int enqueue_steps(trapbec_batch* b, int s, int k, int nact) {
  const int nslots = b->grid * BATCH_SMAX;
  BatchArgs ba;
  ba.desc = b->d_desc;
  ba.ustart = b->d_ustart;
  ba.act = b->d_act;
  ba.nact = nact;
  ba.part = b->d_part;
  ba.part_tag = b->d_tag;
  ba.smax = BATCH_SMAX;
  for (int t = 0; t < k; ++t) {
    ba.par = t & 1;
    shape_launch<T>(s, ST_S1, ba, b->grid, b->st);
    batch_fin_energy_kernel<T><<<nact, FIN_THREADS, 0, b->st>>>(b->d_part, b->d_tag, nslots, b->d_act, nact, b->d_ctrl);
    shape_launch<T>(s, ST_S2, ba, b->grid, b->st);
    shape_launch<T>(s, ST_S3, ba, b->grid, b->st);
    batch_fin_norm_kernel<T><<<nact, FIN_THREADS, 0, b->st>>>(b->d_part, b->d_tag, nslots, b->d_act, nact, b->d_ctrl);
    b->launches += 5;
  }
  BCK(cudaGetLastError());
  return TRAPBEC_OK;
}

template <typename T> int upload_work(trapbec_batch* b, int s, const std::vector<int>& act) {
  // descriptors first: they set each instance's unit count for shape s
  for (int i = 0; i < b->ninst; ++i)
    if (int rc = fill_desc<T>(b, i, s)) return rc;
  long long u = 0;
  for (size_t k = 0; k < act.size(); ++k) {
    b->h_act[k] = act[k];
    b->h_ustart[k] = u;
    u += b->in[act[k]].units;
  }
  b->h_ustart[act.size()] = u;
  BCK(cudaMemcpyAsync(b->d_desc, b->h_desc.data(), b->h_desc.size(), cudaMemcpyHostToDevice, b->st));
  BCK(cudaMemcpyAsync(b->d_act, b->h_act, sizeof(int) * act.size(), cudaMemcpyHostToDevice, b->st));
  BCK(cudaMemcpyAsync(b->d_ustart, b->h_ustart, sizeof(long long) * (act.size() + 1), cudaMemcpyHostToDevice, b->st));
  // Clear the slot tags for this work list.  Every S1 and S3 launch over one
  // work list writes the same slots (one per CTA and grid it touches, tagged
  // with that grid, whether or not the grid has converged), so within a graph
  // replay no slot carries a stale tag and the steps need no clearing.
  BCK(cudaMemsetAsync(b->d_tag, 0xff, sizeof(int) * (size_t)b->max_grid * BATCH_SMAX, b->st));
  return TRAPBEC_OK;
}

int check_err(trapbec_batch* b) {
  BCK(cudaMemcpyAsync(b->h_err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->st));
  BCK(cudaStreamSynchronize(b->st));
  if (*b->h_err) {
    const int code = *b->h_err;
    *b->h_err = 0;
    cudaMemset(b->d_err, 0, sizeof(int));
    set_error("batch: device error code " + std::to_string(code) +
              (code == TERR_TOO_MANY_SEGMENTS ? " (too many segments per CTA)" : " (bounded wait timed out)"));
    return TRAPBEC_ERR_TIMEOUT;
  }
  return TRAPBEC_OK;
}

void reset_ctrl(trapbec_batch* b, int i, double tol) {
  ImagCtrl& c = b->h_ctrl[i];
  std::memset(&c, 0, sizeof(c));
  c.scale = 1.0;
  c.n0 = -1.0;   // set from the initial state by the first energy finaliser
  c.tol = tol;
  c.dV = b->in[i].dV;
  c.escale = b->in[i].escale;
  c.stop_mode = b->stop_mode;
  c.rel = INFINITY;
}

// Time 2 steps of each shape on the batch and keep the fastest; the states
// are restored afterwards.
template <typename T> int autotune(trapbec_batch* b, double tol) {
  const int ns = sizeof(T) == 8 ? BATCH_NSHAPES_F64 : BATCH_NSHAPES_F32;
  if (ns == 1) {
    b->shape = 0;
    return shape_prepare<T>(0, b->nsm, &b->grid) ? TRAPBEC_ERR_CUDA : TRAPBEC_OK;
  }
  std::vector<void*> save(b->ninst, nullptr);
  for (int i = 0; i < b->ninst; ++i) {
    BCK(cudaMalloc(&save[i], b->in[i].n * b->esz));
    BCK(cudaMemcpyAsync(save[i], b->in[i].psi[b->in[i].cur], b->in[i].n * b->esz, cudaMemcpyDeviceToDevice, b->st));
  }
  std::vector<int> act(b->ninst);
  for (int i = 0; i < b->ninst; ++i) act[i] = i;
  double best = 1e300;
  int rc = TRAPBEC_OK;
  for (int s = 0; s < ns && rc == TRAPBEC_OK; ++s) {
    int g = 0;
    if (shape_prepare<T>(s, b->nsm, &g)) continue;
    b->grid = g;
    for (int i = 0; i < b->ninst; ++i) reset_ctrl(b, i, 0.0);
    if ((rc = upload_work<T>(b, s, act))) break;
    if (cudaMemcpyAsync(b->d_ctrl, b->h_ctrl, sizeof(ImagCtrl) * b->ninst, cudaMemcpyHostToDevice, b->st)) {
      rc = TRAPBEC_ERR_CUDA;
      break;
    }
    if ((rc = enqueue_steps<T>(b, s, 2, b->ninst))) break;   // warm-up
    cudaEventRecord(b->e0, b->st);
    if ((rc = enqueue_steps<T>(b, s, 2, b->ninst))) break;
    cudaEventRecord(b->e1, b->st);
    cudaEventSynchronize(b->e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, b->e0, b->e1);
    if (ms < best) { best = ms; b->shape = s; }
    for (int i = 0; i < b->ninst; ++i)
      if (cudaMemcpyAsync(b->in[i].psi[b->in[i].cur], save[i], b->in[i].n * b->esz, cudaMemcpyDeviceToDevice, b->st))
        rc = TRAPBEC_ERR_CUDA;
  }
  cudaStreamSynchronize(b->st);
  for (void* p : save) cudaFree(p);
  if (rc) return rc;
  if ((rc = check_err(b))) return rc;
  if (b->shape < 0) { set_error("batch: no tile shape fits these grids"); return TRAPBEC_ERR_UNSUPPORTED; }
  shape_prepare<T>(b->shape, b->nsm, &b->grid);
  return TRAPBEC_OK;
}

template <typename T> int solve_impl(trapbec_batch* b, int max_steps, double tol, int check_every, int* steps_out,
                                     double* e_out, double* mu_out) {
  if (b->shape < 0) {
    if (int rc = autotune<T>(b, tol)) return rc;
  }
  const int s = b->shape;
  const int k = std::max(2, check_every);
  for (int i = 0; i < b->ninst; ++i) {
    reset_ctrl(b, i, tol);
    b->in[i].steps = 0;
    b->in[i].prev_step = 0;
  }
  BCK(cudaMemcpyAsync(b->d_ctrl, b->h_ctrl, sizeof(ImagCtrl) * b->ninst, cudaMemcpyHostToDevice, b->st));
  cudaGraphExec_t gexec = nullptr;
  int graph_nact = -1, graph_k = -1;
  BCK(cudaEventRecord(b->e0, b->st));
  int rc = TRAPBEC_OK;
  while (true) {
    std::vector<int> act;
    for (int i = 0; i < b->ninst; ++i) {
      const ImagCtrl& c = b->h_ctrl[i];
      if (!c.converged && !c.nonfinite && b->in[i].steps < max_steps) act.push_back(i);
    }
    if (act.empty()) break;
    // the active instances have made the same number of steps in this call; a
    // replay never takes them past max_steps
    int left = max_steps;
    for (int i : act) left = std::min(left, max_steps - b->in[i].steps);
    const int kk = std::min(k, std::max(1, left));
    if ((rc = upload_work<T>(b, s, act))) break;
    if ((int)act.size() != graph_nact || kk != graph_k) {   // capture the kk-step loop for this work-list size
      if (gexec) cudaGraphExecDestroy(gexec);
      gexec = nullptr;
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { rc = TRAPBEC_ERR_CUDA; break; }
      int erc = enqueue_steps<T>(b, s, kk, (int)act.size());
      cudaError_t ce = cudaStreamEndCapture(b->st, &g);
      if (erc || ce != cudaSuccess) { set_error("batch: graph capture failed"); rc = TRAPBEC_ERR_CUDA; break; }
      ce = cudaGraphInstantiate(&gexec, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) { set_error("batch: graph instantiation failed"); rc = TRAPBEC_ERR_CUDA; break; }
      graph_nact = (int)act.size();
      graph_k = kk;
      b->launches -= 5LL * kk;  // counted below per replay
    }
    if (cudaGraphLaunch(gexec, b->st) != cudaSuccess) { set_error("batch: graph launch failed"); rc = TRAPBEC_ERR_CUDA; break; }
    b->launches += 5LL * kk;
    if (cudaMemcpyAsync(b->h_ctrl, b->d_ctrl, sizeof(ImagCtrl) * b->ninst, cudaMemcpyDeviceToHost, b->st) ||
        cudaStreamSynchronize(b->st)) {
      set_error("batch: control read-back failed");
      rc = TRAPBEC_ERR_CUDA;
      break;
    }
    if ((rc = check_err(b))) break;
    for (int i : act) {
      BInst& I = b->in[i];
      const int delta = b->h_ctrl[i].step - I.prev_step;
      I.prev_step = b->h_ctrl[i].step;
      I.steps += delta;
      I.cur ^= (delta & 1);
    }
  }
  if (gexec) cudaGraphExecDestroy(gexec);
  BCK(cudaEventRecord(b->e1, b->st));
  BCK(cudaEventSynchronize(b->e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, b->e0, b->e1);
  b->solve_ms = ms;
  if (rc) return rc;
  // apply the pending renormalisation of every instance
  for (int i = 0; i < b->ninst; ++i) {
    BInst& I = b->in[i];
    const double sc = b->h_ctrl[i].scale;
    if (sc != 1.0) {
      scale_kernel<T><<<std::max(1, b->nsm * 4), 256, 0, b->st>>>((c_t<T>*)I.psi[I.cur], I.n, (T)sc);
      b->launches++;
      b->h_ctrl[i].scale = 1.0;
    }
    if (steps_out) steps_out[i] = I.steps;
    if (e_out) e_out[i] = b->h_ctrl[i].energy;
    if (mu_out) mu_out[i] = b->h_ctrl[i].mu;
  }
  BCK(cudaMemcpyAsync(b->d_ctrl, b->h_ctrl, sizeof(ImagCtrl) * b->ninst, cudaMemcpyHostToDevice, b->st));
  BCK(cudaStreamSynchronize(b->st));
  for (int i = 0; i < b->ninst; ++i)
    if (b->h_ctrl[i].nonfinite) {
      set_error("batch: non-finite energy or norm in instance " + std::to_string(i));
      return TRAPBEC_ERR_NONFINITE;
    }
  return TRAPBEC_OK;
}

template <typename T> int init_state_batch(trapbec_batch* b, int i, const char* name, const trapbec_init_args* ia) {
  BInst& I = b->in[i];
  const trapbec_params& p = I.p;
  std::string nm(name);
  InitArgsDev<T> a;
  std::memset(&a, 0, sizeof(a));
  a.psi = (c_t<T>*)I.psi[I.cur];
  a.xx = (const T*)I.xx; a.yy = (const T*)I.yy; a.zz = (const T*)I.zz;
  a.nx = p.nx; a.ny = p.ny; a.nz = p.nz;
  a.Lx = (T)p.lx; a.Ly = (T)p.ly; a.Lz = (T)p.lz;
  a.harm_wx = (T)p.harm_wx; a.harm_wy = (T)p.harm_wy; a.harm_wz = (T)p.harm_wz;
  if (nm == "thomas_fermi") {
    a.kind = IK_TF;
  } else if (nm == "tf_vortex_line" || nm == "tf_vortex_ring" || nm == "tf_noise") {
    if (!ia) { set_error("batch init_state: workload states need trapbec_init_args"); return TRAPBEC_ERR_ARG; }
    a.kind = nm == "tf_vortex_line" ? IK_TF_LINE : (nm == "tf_vortex_ring" ? IK_TF_RING : IK_TF_NOISE);
    a.d[0] = ia->amp; a.d[1] = ia->r_tf2[0]; a.d[2] = ia->r_tf2[1]; a.d[3] = ia->r_tf2[2];
    a.d[4] = ia->ring_radius; a.d[5] = ia->core2; a.d[6] = ia->noise_amp;
    a.seed = ia->seed;
  } else {
    set_error("batch init_state: supported states are thomas_fermi, tf_noise, tf_vortex_line, tf_vortex_ring");
    return TRAPBEC_ERR_ARG;
  }
  init_state_kernel<T><<<std::max(1, b->nsm * 4), 256, 0, b->st>>>(a);
  b->launches++;
  BCK(cudaGetLastError());
  BCK(cudaStreamSynchronize(b->st));
  return TRAPBEC_OK;
}

void free_batch(trapbec_batch* b) {
  if (!b) return;
  if (b->st) cudaStreamSynchronize(b->st);
  for (BInst& I : b->in) {
    void* bufs[] = {I.psi[0], I.psi[1], I.w, I.xx, I.yy, I.zz, I.px, I.py, I.pz};
    for (void* p : bufs) if (p) cudaFree(p);
  }
  void* dev[] = {b->d_desc, b->d_ctrl, b->d_ustart, b->d_act, b->d_part, b->d_tag, b->d_err};
  for (void* p : dev) if (p) cudaFree(p);
  void* host[] = {b->h_ctrl, b->h_ustart, b->h_act, b->h_err};
  for (void* p : host) if (p) cudaFreeHost(p);
  if (b->e0) cudaEventDestroy(b->e0);
  if (b->e1) cudaEventDestroy(b->e1);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

}  // namespace

extern "C" {

int trapbec_batch_create(int ninst, const trapbec_params* params, trapbec_batch** out) {
  if (!out) return TRAPBEC_ERR_ARG;
  *out = nullptr;
  if (ninst <= 0 || !params) { set_error("batch: need at least one instance"); return TRAPBEC_ERR_ARG; }
  const int prec = params[0].precision;
  for (int i = 0; i < ninst; ++i) {
    const trapbec_params& p = params[i];
    if (p.precision != prec) { set_error("batch: all instances must share one precision"); return TRAPBEC_ERR_ARG; }
    if (p.two_dim || p.nx < 8 || p.ny < 8 || p.nz < 8 || (prec == TRAPBEC_FP32 && (p.nz % 2))) {
      set_error("batch: grids must be 3D, at least 8 cells per axis, nz even in FP32");
      return TRAPBEC_ERR_ARG;
    }
    if (p.boundaries != TRAPBEC_BC_ZERO || p.periodicz) {
      set_error("batch: instances use 'zero' boundaries (trapped condensates)");
      return TRAPBEC_ERR_UNSUPPORTED;
    }
    if (p.potential != TRAPBEC_POT_HARMONIC && p.potential != TRAPBEC_POT_ZERO) {
      set_error("batch: instances use the 'harmonic' or 'zero' potential");
      return TRAPBEC_ERR_UNSUPPORTED;
    }
    if (p.lbeam || p.advective_vx != 0.0 || p.nprocx > 1 || p.nprocy > 1) {
      set_error("batch: no laser, moving frame or process-grid coordinates in batched solves");
      return TRAPBEC_ERR_UNSUPPORTED;
    }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { set_error("no CUDA device"); return TRAPBEC_ERR_NODEVICE; }
  trapbec_batch* b = new trapbec_batch;
  b->prec = prec;
  b->ninst = ninst;
  b->rsz = prec == TRAPBEC_FP64 ? 8 : 4;
  b->esz = 2 * b->rsz;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev);
  b->in.resize(ninst);
  for (int i = 0; i < ninst; ++i) b->in[i].p = params[i];
  if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess) {
    free_batch(b);
    set_error("batch: stream creation failed");
    return TRAPBEC_ERR_CUDA;
  }
  cudaEventCreate(&b->e0);
  cudaEventCreate(&b->e1);
  int rc = prec == TRAPBEC_FP64 ? create_impl<double>(b) : create_impl<float>(b);
  if (rc) { free_batch(b); return rc; }
  *out = b;
  return TRAPBEC_OK;
}

void trapbec_batch_destroy(trapbec_batch* b) { free_batch(b); }

int trapbec_batch_set_psi(trapbec_batch* b, int inst, const void* psi) {
  if (!b || !psi || inst < 0 || inst >= b->ninst) return TRAPBEC_ERR_ARG;
  BInst& I = b->in[inst];
  BCK(cudaMemcpyAsync(I.psi[I.cur], psi, I.n * b->esz, cudaMemcpyHostToDevice, b->st));
  BCK(cudaStreamSynchronize(b->st));
  return TRAPBEC_OK;
}

int trapbec_batch_get_psi(trapbec_batch* b, int inst, void* psi) {
  if (!b || !psi || inst < 0 || inst >= b->ninst) return TRAPBEC_ERR_ARG;
  BInst& I = b->in[inst];
  BCK(cudaMemcpyAsync(psi, I.psi[I.cur], I.n * b->esz, cudaMemcpyDeviceToHost, b->st));
  BCK(cudaStreamSynchronize(b->st));
  return TRAPBEC_OK;
}

int trapbec_batch_init_state(trapbec_batch* b, int inst, const char* init_cond, const trapbec_init_args* args) {
  if (!b || !init_cond || inst < 0 || inst >= b->ninst) return TRAPBEC_ERR_ARG;
  return b->prec == TRAPBEC_FP64 ? init_state_batch<double>(b, inst, init_cond, args)
                                 : init_state_batch<float>(b, inst, init_cond, args);
}

int trapbec_batch_set_imag_stop(trapbec_batch* b, int mode, const double* energy_scale) {
  if (!b) return TRAPBEC_ERR_ARG;
  if (mode == TRAPBEC_STOP_REL) {
    for (auto& I : b->in) I.escale = 0.0;
    b->stop_mode = mode;
    return TRAPBEC_OK;
  }
  if (mode != TRAPBEC_STOP_ABS && mode != TRAPBEC_STOP_ABS_PER_NORM) {
    set_error("trapbec_batch_set_imag_stop: mode must be TRAPBEC_STOP_REL, TRAPBEC_STOP_ABS or TRAPBEC_STOP_ABS_PER_NORM");
    return TRAPBEC_ERR_ARG;
  }
  for (int i = 0; i < b->ninst; ++i) {
    const double e = energy_scale ? energy_scale[i] : 1.0;
    if (!(e > 0.0) || !std::isfinite(e)) {
      set_error("trapbec_batch_set_imag_stop: energy_scale[" + std::to_string(i) + "] must be finite and > 0");
      return TRAPBEC_ERR_ARG;
    }
  }
  for (int i = 0; i < b->ninst; ++i) b->in[i].escale = energy_scale ? energy_scale[i] : 1.0;
  b->stop_mode = mode;
  return TRAPBEC_OK;
}

int trapbec_batch_solve_imag(trapbec_batch* b, int max_steps, double tol, int check_every, int* steps_out,
                             double* energy_out, double* mu_out) {
  if (!b || max_steps < 0) return TRAPBEC_ERR_ARG;
  return b->prec == TRAPBEC_FP64 ? solve_impl<double>(b, max_steps, tol, check_every, steps_out, energy_out, mu_out)
                                 : solve_impl<float>(b, max_steps, tol, check_every, steps_out, energy_out, mu_out);
}

int trapbec_batch_stats(trapbec_batch* b, double* solve_ms, int* tile_z, int* tile_y, int64_t* launches) {
  if (!b) return TRAPBEC_ERR_ARG;
  if (solve_ms) *solve_ms = b->solve_ms;
  if (tile_z) *tile_z = b->shape < 0 ? 0 : (b->prec == TRAPBEC_FP64 ? shape_tz<double>(b->shape) : shape_tz<float>(b->shape));
  if (tile_y) *tile_y = b->shape < 0 ? 0 : (b->prec == TRAPBEC_FP64 ? shape_ty<double>(b->shape) : shape_ty<float>(b->shape));
  if (launches) *launches = b->launches;
  return TRAPBEC_OK;
}

int trapbec_batch_status(trapbec_batch* b, int inst, double* o) {
  if (!b || !o || inst < 0 || inst >= b->ninst) return TRAPBEC_ERR_ARG;
  BCK(cudaMemcpyAsync(b->h_ctrl, b->d_ctrl, sizeof(ImagCtrl) * b->ninst, cudaMemcpyDeviceToHost, b->st));
  BCK(cudaStreamSynchronize(b->st));
  const ImagCtrl& c = b->h_ctrl[inst];
  o[0] = c.scale; o[1] = c.e_prev; o[2] = c.rel; o[3] = c.energy; o[4] = c.mu;
  o[5] = c.norm; o[6] = c.n0; o[7] = c.step; o[8] = c.converged; o[9] = c.nonfinite;
  return TRAPBEC_OK;
}

}  // extern "C"
