// tiled_f64_s1.cu -- tiled stage kernel, double, TZ=64 TY=8 R=2, 8 ring slots.
#include "tiled_impl.cuh"

namespace tb {
int plan_f64_s1(const trapbec_params& p, void* const psi[2], void* w, void* w2, int nsm, int* err, TiledPlan* plan) {
  return plan_shape<double, 64, 8, 2, 8, 0>(p, psi, w, w2, nsm, err, plan);
}
int launch_f64_s1(const TiledPlan& plan, int kind, const StageArgs<double>& a, cudaStream_t st, int red_cap, int* nblk) {
  return launch_shape<double, 64, 8, 2, 8, 0>(plan, kind, a, st, red_cap, nblk);
}
}  // namespace tb
