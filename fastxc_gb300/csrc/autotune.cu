// Autotuner of the xc stack: picks the tile shape / method for a shape by
// timing the candidates on a sample of frequency bins of the real input.
//
// Candidates: the plain FP32 kernel (16 x 16 channel tiles, 64 bins per CTA,
// register-tiled complex MACs) and the tcgen05 BF16 hi/lo contraction
// (128 x N channel tiles per bin, including its pack pass). Each candidate
// runs twice on the first `sample` bins (the second run is timed with CUDA
// events on the context's stream); the per-bin cost does not depend on the
// bin, so the faster sample is the faster full run. Decisions are cached
// per (device, channels, windows, pairs, pair-tile count) for the process.
#include <map>
#include <mutex>
#include <tuple>

#include "context.cuh"
#include "xc.cuh"

namespace fxc {
namespace {

struct TuneKey {
  int dev, nchan;
  int64_t nwin, npairs, ntiles;
  bool operator<(const TuneKey& o) const {
    return std::tie(dev, nchan, nwin, npairs, ntiles) < std::tie(o.dev, o.nchan, o.nwin, o.npairs, o.ntiles);
  }
};

struct TuneResult {
  int method;
  float ms_plain, ms_tensor;
};

std::mutex g_mu;
std::map<TuneKey, TuneResult> g_cache;

}  // namespace
}  // namespace fxc

using namespace fxc;

extern "C" {

int fxc_xc_autotune(fxc_ctx* ctx, const fxc_pairplan* plan, const float* d_spec, int64_t nwin, int32_t nchan,
                    int32_t nspec, int64_t spec_pitch, int32_t* method, float* ms_plain, float* ms_tensor) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(plan && d_spec && method, "null argument");
  FXC_CHECK_ARG(nwin > 0 && nchan > 0 && nspec > 0 && spec_pitch >= nspec, "invalid shape");
  const TuneKey key{ctx->device, nchan, nwin, plan->npairs, plan->ntiles};
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      *method = it->second.method;
      if (ms_plain) *ms_plain = it->second.ms_plain;
      if (ms_tensor) *ms_tensor = it->second.ms_tensor;
      return FXC_OK;
    }
  }
  if (plan->npairs == 0) {
    *method = FXC_XC_PLAIN;
    return FXC_OK;
  }
  const int sample = std::min<int>(nspec, 512);
  const int64_t pitch = xc_stack_pitch(sample);
  FXC_TRY(ctx->scratch.reserve((size_t)plan->npairs * pitch * sizeof(float2)));
  float2* stack = reinterpret_cast<float2*>(ctx->scratch.ptr);
  const float2* spec = reinterpret_cast<const float2*>(d_spec);
  cudaEvent_t e0, e1;
  FXC_CUDA_TRY(cudaEventCreate(&e0));
  FXC_CUDA_TRY(cudaEventCreate(&e1));
  float ms[2] = {-1.f, -1.f};
  const int cand[2] = {FXC_XC_PLAIN, FXC_XC_TENSOR};
  int rc = FXC_OK;
  for (int c = 0; c < 2 && rc == FXC_OK; ++c) {
    for (int rep = 0; rep < 2 && rc == FXC_OK; ++rep) {
      if (rep == 1) cudaEventRecord(e0, ctx->stream);
      rc = xc_stack_launch(ctx, plan, spec, nwin, nchan, sample, spec_pitch, nullptr, 1.0f, stack, pitch, cand[c]);
      if (rep == 1) cudaEventRecord(e1, ctx->stream);
    }
    if (rc == FXC_OK && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms[c], e0, e1);
    if (rc != FXC_OK && cand[c] == FXC_XC_TENSOR) {
      // the tensor path is optional (e.g. a plan without tensor tiles): fall
      // back to timing the plain kernel alone
      ms[c] = -1.f;
      rc = FXC_OK;
      clear_error();
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  FXC_TRY(rc);
  FXC_TRY(ctx_check_device_error(ctx));
  TuneResult r;
  r.ms_plain = ms[0];
  r.ms_tensor = ms[1];
  r.method = (ms[1] >= 0.f && ms[1] < ms[0]) ? FXC_XC_TENSOR : FXC_XC_PLAIN;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache[key] = r;
  }
  *method = r.method;
  if (ms_plain) *ms_plain = r.ms_plain;
  if (ms_tensor) *ms_tensor = r.ms_tensor;
  return FXC_OK;
}

}  // extern "C"
