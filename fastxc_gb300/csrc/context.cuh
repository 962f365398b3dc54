// Context object behind the opaque fxc_ctx handle.
#pragma once

#include <string>
#include <vector>

#include "fxc_common.cuh"

namespace fxc {

// A device buffer grown on demand and reused across calls on one context.
struct Scratch {
  void* ptr = nullptr;
  size_t bytes = 0;
  int reserve(size_t need);
  void release();
};

void count_launch(int n = 1);
int ctx_enter(fxc_ctx* ctx);
int ctx_check_device_error(fxc_ctx* ctx);

}  // namespace fxc

namespace fxc {
struct KernelTimeRec {
  std::string name;
  cudaEvent_t start, stop;
};
}  // namespace fxc

struct fxc_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 148;
  fxc::Scratch scratch;   // per-pair stacked spectra between stack and finalize
  fxc::Scratch scratch2;  // host-call staging (device copies of host inputs)
  fxc::Scratch scratch3;  // packed bf16 hi/lo operands of the tensor-core path
  fxc::Scratch scratch4;  // sac2spec intermediate rows (time rows, weights, spectra)
  fxc::Scratch scratch5;  // bin-major stack rows of the whole-bin tensor-core contraction
  int* d_err = nullptr;   // device error word: set by kernels whose bounded waits time out
  cudaStream_t copy_stream = nullptr;  // host<->device copies of the host-buffer entry points
  bool ktime_on = false;               // fxc_ctx_kernel_timing
  std::vector<fxc::KernelTimeRec> ktimes;
  // phases of the last fxc_xc_run_host while kernel timing is on (ms):
  // total, copy-stream busy, last H2D copy end, compute busy, tail after the
  // last H2D copy, finalize + D2H; -1 when not measured
  double host_phase_ms[6] = {-1, -1, -1, -1, -1, -1};
};

namespace fxc {
// Brackets one launch with events on the context stream while kernel timing
// is enabled (a no-op otherwise): construct before the launch, stop() after.
struct KernelTimer {
  fxc_ctx* ctx;
  const char* name;
  cudaEvent_t start = nullptr;
  KernelTimer(fxc_ctx* c, const char* n) : ctx(c), name(n) {
    if (ctx->ktime_on && cudaEventCreate(&start) == cudaSuccess) {
      if (cudaEventRecord(start, ctx->stream) != cudaSuccess) {
        cudaEventDestroy(start);
        start = nullptr;
      }
    } else {
      start = nullptr;
    }
  }
  void stop() {
    if (!start) return;
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) == cudaSuccess && cudaEventRecord(e, ctx->stream) == cudaSuccess) {
      ctx->ktimes.push_back(KernelTimeRec{name, start, e});
    } else {
      if (e) cudaEventDestroy(e);
      cudaEventDestroy(start);
    }
    start = nullptr;
  }
  ~KernelTimer() {
    if (start) cudaEventDestroy(start);
  }
};
}  // namespace fxc
