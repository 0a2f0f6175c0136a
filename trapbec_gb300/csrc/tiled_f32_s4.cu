// tiled_f32_s4.cu -- tiled stage kernel, float, TZ=64 TY=32 R=4, 6 ring slots (default real-time shape).
#include "tiled_impl.cuh"

namespace tb {
int plan_f32_s4(const trapbec_params& p, void* const psi[2], void* w, void* w2, int nsm, int* err, TiledPlan* plan) {
  return plan_shape<float, 64, 32, 4, 6, 0>(p, psi, w, w2, nsm, err, plan);
}
int launch_f32_s4(const TiledPlan& plan, int kind, const StageArgs<float>& a, cudaStream_t st, int red_cap, int* nblk) {
  return launch_shape<float, 64, 32, 4, 6, 0>(plan, kind, a, st, red_cap, nblk);
}
}  // namespace tb
