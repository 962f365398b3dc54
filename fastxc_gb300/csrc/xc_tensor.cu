// BF16 hi/lo split tensor-core contraction S(f) = Y(f)^H Y(f) (placeholder
// until the tcgen05 kernel lands: reports FXC_ERR_UNSUPPORTED).
#include "xc.cuh"

namespace fxc {

struct XcTensorPlan {
  int unused;
};

int xc_tensor_plan_init(fxc_ctx*, fxc_pairplan* plan) {
  plan->tensor = nullptr;
  return FXC_OK;
}

void xc_tensor_plan_free(fxc_pairplan* plan) {
  delete plan->tensor;
  plan->tensor = nullptr;
}

int xc_stack_tensor_launch(fxc_ctx*, const fxc_pairplan*, const float2*, int64_t, int, int,
                           int64_t, const uint8_t*, float, float2*, int64_t) {
  set_error("tensor-core contraction not built yet");
  return FXC_ERR_UNSUPPORTED;
}

}  // namespace fxc
