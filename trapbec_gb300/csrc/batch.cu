// batch.cu -- batched imaginary-time ground states (placeholder until the
// persistent multi-instance kernel lands).
#include "../../include/trapbec.h"
#include "host_util.h"

extern "C" {
int trapbec_batch_create(int, const trapbec_params*, trapbec_batch** out) {
  if (out) *out = nullptr;
  tbh::set_error("batched solver not built yet");
  return TRAPBEC_ERR_UNSUPPORTED;
}
void trapbec_batch_destroy(trapbec_batch*) {}
int trapbec_batch_set_psi(trapbec_batch*, int, const void*) { return TRAPBEC_ERR_UNSUPPORTED; }
int trapbec_batch_get_psi(trapbec_batch*, int, void*) { return TRAPBEC_ERR_UNSUPPORTED; }
int trapbec_batch_solve_imag(trapbec_batch*, int, double, int, int*, double*, double*) {
  return TRAPBEC_ERR_UNSUPPORTED;
}
}
