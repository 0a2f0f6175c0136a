// tiled_dispatch.cu -- shape dispatch of the tiled stage kernel.  Each shape
// is compiled in its own translation unit (tiled_<prec>_s<i>.cu).
#include "tiled_api.h"

namespace tb {

int plan_f32_s0(const trapbec_params&, void* const[2], void*, void*, int, int*, TiledPlan*);
int plan_f32_s1(const trapbec_params&, void* const[2], void*, void*, int, int*, TiledPlan*);
int plan_f32_s2(const trapbec_params&, void* const[2], void*, void*, int, int*, TiledPlan*);
int plan_f32_s3(const trapbec_params&, void* const[2], void*, void*, int, int*, TiledPlan*);
int plan_f32_s4(const trapbec_params&, void* const[2], void*, void*, int, int*, TiledPlan*);
int plan_f64_s0(const trapbec_params&, void* const[2], void*, void*, int, int*, TiledPlan*);
int plan_f64_s1(const trapbec_params&, void* const[2], void*, void*, int, int*, TiledPlan*);
int launch_f32_s0(const TiledPlan&, int, const StageArgs<float>&, cudaStream_t, int, int*);
int launch_f32_s1(const TiledPlan&, int, const StageArgs<float>&, cudaStream_t, int, int*);
int launch_f32_s2(const TiledPlan&, int, const StageArgs<float>&, cudaStream_t, int, int*);
int launch_f32_s3(const TiledPlan&, int, const StageArgs<float>&, cudaStream_t, int, int*);
int launch_f32_s4(const TiledPlan&, int, const StageArgs<float>&, cudaStream_t, int, int*);
int launch_f64_s0(const TiledPlan&, int, const StageArgs<double>&, cudaStream_t, int, int*);
int launch_f64_s1(const TiledPlan&, int, const StageArgs<double>&, cudaStream_t, int, int*);

template <>
int plan_tiled<float>(const trapbec_params& p, void* const psi[2], void* w, void* w2, int nsm, int shape, int* err,
                      TiledPlan* plan) {
  int rc;
  switch (shape) {
    case 0: rc = plan_f32_s0(p, psi, w, w2, nsm, err, plan); break;
    case 1: rc = plan_f32_s1(p, psi, w, w2, nsm, err, plan); break;
    case 2: rc = plan_f32_s2(p, psi, w, w2, nsm, err, plan); break;
    case 3: rc = plan_f32_s3(p, psi, w, w2, nsm, err, plan); break;
    case 4: rc = plan_f32_s4(p, psi, w, w2, nsm, err, plan); break;
    default: return 9;
  }
  if (rc == 0) plan->shape = shape;
  return rc;
}

template <>
int launch_tiled<float>(const TiledPlan& plan, int kind, const StageArgs<float>& a, cudaStream_t st, int red_cap,
                        int* nblk) {
  switch (plan.shape) {
    case 0: return launch_f32_s0(plan, kind, a, st, red_cap, nblk);
    case 1: return launch_f32_s1(plan, kind, a, st, red_cap, nblk);
    case 2: return launch_f32_s2(plan, kind, a, st, red_cap, nblk);
    case 3: return launch_f32_s3(plan, kind, a, st, red_cap, nblk);
    case 4: return launch_f32_s4(plan, kind, a, st, red_cap, nblk);
  }
  return 9;
}

template <>
int plan_tiled<double>(const trapbec_params& p, void* const psi[2], void* w, void* w2, int nsm, int shape, int* err,
                       TiledPlan* plan) {
  int rc;
  switch (shape) {
    case 0: rc = plan_f64_s0(p, psi, w, w2, nsm, err, plan); break;
    case 1: rc = plan_f64_s1(p, psi, w, w2, nsm, err, plan); break;
    default: return 9;
  }
  if (rc == 0) plan->shape = shape;
  return rc;
}

template <>
int launch_tiled<double>(const TiledPlan& plan, int kind, const StageArgs<double>& a, cudaStream_t st, int red_cap,
                         int* nblk) {
  switch (plan.shape) {
    case 0: return launch_f64_s0(plan, kind, a, st, red_cap, nblk);
    case 1: return launch_f64_s1(plan, kind, a, st, red_cap, nblk);
  }
  return 9;
}

}  // namespace tb
