// Memory planners: how much work one library call may take under a device
// memory budget.
//
// The reference sizes its batches from a memory model of its own buffers:
// xc pair blocks under 0.90 x free VRAM and 0.80 x MemAvailable
// (native/xc/memory/memory.cu:112-399), sac2spec frame batches under
// 0.70 x free VRAM (native/sac2spec/device_memory_estimate.cu:7-37), and the
// TF-PWS frequency chunk K by binary search under -M with the model
// 12GN + 32N + 4G + K(8GN + 16N + 8) plus the cuFFT workspace
// (native/tfpws/include/tfpws_schedule.hpp:70-80,149-217).
//
// This library's buffers differ, so its planners use its own model, kept
// next to the code that reserves the memory: every planner below is a
// byte count of exactly the buffers the matching call reserves (context
// scratch, plus the caller's inputs and outputs where the executables place
// them), and a binary search for the largest unit count (pairs, traces)
// whose bytes fit. In particular TF-PWS needs no frequency chunk: the
// reference materialises (G+1) x K x N voice spectra per chunk, while this
// library forms each (pair, frequency) block's voices in shared memory, so
// its footprint does not depend on K and the planner sizes the pair batch
// instead.
#include <algorithm>

#include "context.cuh"
#include "xc.cuh"

namespace fxc {
int64_t xc_packed_chunks(int32_t nchan, int64_t nwin, int32_t nspec);
}

using namespace fxc;

namespace {

constexpr int64_t al256(int64_t x) { return (x + 255) & ~int64_t(255); }
constexpr int64_t kXcChunkWindows = 64;  // fxc_xc_run_host's window chunk
constexpr int64_t kXcRing = 3;           // and its ring of chunk buffers
constexpr int64_t kPlanBytesPerPair = 64;  // pair tiles, maps and tensor tiles (bound)

// Device bytes of one fxc_xc_run_host call over `npairs` pairs: the chunk
// ring, the mask, the NCF staging, the stacked spectra, and on the tensor
// path the packed operands of one chunk and the bin-major rows (counted at
// their whole-bin size, the larger of the two contraction layouts).
int64_t xc_host_bytes(int64_t npairs, int64_t nwin, int32_t nchan, int64_t spec_pitch, int32_t nspec,
                      int32_t cc_size, bool tensor, bool mask) {
  const int64_t chunk = 8 * (int64_t)nchan * spec_pitch * kXcChunkWindows;
  int64_t b = al256(chunk) * kXcRing;
  if (mask) b += al256(nwin * (int64_t)nchan);
  b += al256(4 * npairs * (int64_t)cc_size);
  b += 8 * xc_stack_pitch(nspec) * npairs;
  if (tensor) {
    b += 16 * xc_packed_chunks(nchan, std::min<int64_t>(nwin, kXcChunkWindows), nspec);
    b += 8 * ((npairs + 3) / 4 * 4) * (int64_t)nspec;
  }
  return b + kPlanBytesPerPair * npairs;
}

// Device bytes of one stacking batch of the ncf_pws / ncf_tfpws executables:
// their buffers (traces, groups, weights, linear stacks, output) and the
// library's scratch for the batch (PWS: the analytic-signal sums per pair;
// TF-PWS: the analytic spectra of every group and linear stack, the output
// spectra and the Gaussian window table).
int64_t stack_batch_bytes(int mode, int64_t ntraces, int64_t npairs, int64_t ngroups, int64_t max_groups,
                          int32_t n) {
  const int64_t tr = 4 * ntraces * n;
  const int64_t pairs = 4 * npairs * n;
  int64_t b = al256(tr) + al256(tr) + al256(4 * ntraces) + al256(pairs) + al256(pairs);
  b += al256(16 * npairs) + 256;  // group offsets / counts staging
  if (mode == 0) {
    // PWS partial sums: pairs x group chunks x n complex; fxc_pws_run takes
    // ceil(8 waves x 6 CTAs x SMs / pairs) chunks of at least two groups of
    // the pair with the most groups (bound: 160 SMs)
    const int64_t want = std::max<int64_t>(1, (8 * 6 * 160 + npairs - 1) / std::max<int64_t>(npairs, 1));
    const int64_t chunks = std::max<int64_t>(1, std::min<int64_t>(want, (max_groups + 1) / 2));
    b += 8 * (int64_t)n * npairs * chunks;
  } else {
    const int64_t nfreq = n / 2 + 1;
    b += al256(8 * npairs) + al256(4 * npairs) + al256(8 * ngroups * n) + al256(8 * npairs * n) +
         al256(8 * npairs * n) + al256(4 * nfreq * n);
  }
  return b;
}

}  // namespace

extern "C" int fxc_plan_xc_pairs(int64_t npairs, int64_t nwin, int32_t nchan, int64_t spec_pitch,
                                 const fxc_xc_shape* shape, int method, int has_mask, int64_t budget_bytes,
                                 int64_t* pairs_per_call, int64_t* bytes_per_call) {
  clear_error();
  FXC_CHECK_ARG(shape && pairs_per_call, "null shape or output");
  FXC_CHECK_ARG(npairs >= 0 && nwin >= 0 && nchan > 0 && spec_pitch >= shape->nspec && budget_bytes > 0,
                "invalid sizes");
  const bool tensor = method == FXC_XC_TENSOR;
  auto bytes = [&](int64_t p) {
    return xc_host_bytes(p, nwin, nchan, spec_pitch, shape->nspec, shape->cc_size, tensor, has_mask != 0);
  };
  if (npairs == 0) {
    *pairs_per_call = 0;
    if (bytes_per_call) *bytes_per_call = 0;
    return FXC_OK;
  }
  if (bytes(1) > budget_bytes) {
    set_error("one pair of %d channels x %lld windows x nspec %d needs %lld device bytes, above the budget of %lld",
              nchan, (long long)nwin, shape->nspec, (long long)bytes(1), (long long)budget_bytes);
    return FXC_ERR_NOMEM;
  }
  int64_t lo = 1, hi = npairs;  // bytes(lo) fits; find the largest fitting count
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo + 1) / 2;
    if (bytes(mid) <= budget_bytes)
      lo = mid;
    else
      hi = mid - 1;
  }
  *pairs_per_call = lo;
  if (bytes_per_call) *bytes_per_call = bytes(lo);
  return FXC_OK;
}

extern "C" int fxc_plan_stack_traces(int mode, int32_t nsamples, int32_t traces_per_pair, int32_t substack,
                                     int64_t budget_bytes, int64_t* max_traces, int64_t* bytes_per_batch) {
  clear_error();
  FXC_CHECK_ARG(max_traces != nullptr, "null output");
  FXC_CHECK_ARG((mode == 0 || mode == 1) && nsamples > 0 && traces_per_pair > 0 && budget_bytes > 0,
                "invalid arguments");
  const int64_t b = substack >= 2 ? substack : 1;
  auto bytes = [&](int64_t npairs) {
    const int64_t per_pair = (traces_per_pair + b - 1) / b;
    return stack_batch_bytes(mode, npairs * traces_per_pair, npairs, npairs * per_pair, per_pair, nsamples);
  };
  if (bytes(1) > budget_bytes) {
    set_error("one pair of %d traces x %d samples needs %lld device bytes, above the budget of %lld",
              traces_per_pair, nsamples, (long long)bytes(1), (long long)budget_bytes);
    return FXC_ERR_NOMEM;
  }
  int64_t lo = 1, hi = 1;
  while (bytes(hi * 2) <= budget_bytes && hi < (int64_t(1) << 40) / traces_per_pair) hi *= 2;
  hi *= 2;
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo + 1) / 2;
    if (bytes(mid) <= budget_bytes)
      lo = mid;
    else
      hi = mid - 1;
  }
  *max_traces = lo * traces_per_pair;
  if (bytes_per_batch) *bytes_per_batch = bytes(lo);
  return FXC_OK;
}

extern "C" int fxc_stack_batch_bytes(int mode, int64_t ntraces, int32_t npairs, int64_t ngroups,
                                     int64_t max_groups_per_pair, int32_t nsamples, int64_t* bytes) {
  clear_error();
  FXC_CHECK_ARG(bytes != nullptr && (mode == 0 || mode == 1) && ntraces >= 0 && npairs >= 0 && ngroups >= 0 &&
                    max_groups_per_pair >= 0 && nsamples > 0,
                "invalid arguments");
  *bytes = stack_batch_bytes(mode, ntraces, npairs, ngroups, max_groups_per_pair, nsamples);
  return FXC_OK;
}

extern "C" int fxc_xc_host_bytes(int64_t npairs, int64_t nwin, int32_t nchan, int64_t spec_pitch,
                                 const fxc_xc_shape* shape, int method, int has_mask, int64_t* bytes) {
  clear_error();
  FXC_CHECK_ARG(shape && bytes, "null shape or output");
  FXC_CHECK_ARG(npairs >= 0 && nwin >= 0 && nchan > 0 && spec_pitch >= shape->nspec, "invalid sizes");
  *bytes = xc_host_bytes(npairs, nwin, nchan, spec_pitch, shape->nspec, shape->cc_size, method == FXC_XC_TENSOR,
                         has_mask != 0);
  return FXC_OK;
}
