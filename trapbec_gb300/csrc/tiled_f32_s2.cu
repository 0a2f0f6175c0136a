// tiled_f32_s2.cu -- tiled stage kernel, float, TZ=64 TY=16 R=2, 8 ring slots.
#include "tiled_impl.cuh"

namespace tb {
int plan_f32_s2(const trapbec_params& p, void* const psi[2], void* w, void* w2, int nsm, int* err, TiledPlan* plan) {
  return plan_shape<float, 64, 16, 2, 8, 0>(p, psi, w, w2, nsm, err, plan);
}
int launch_f32_s2(const TiledPlan& plan, int kind, const StageArgs<float>& a, cudaStream_t st, int red_cap, int* nblk) {
  return launch_shape<float, 64, 16, 2, 8, 0>(plan, kind, a, st, red_cap, nblk);
}
}  // namespace tb
