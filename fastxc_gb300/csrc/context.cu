// Library runtime: error reporting, contexts, scratch memory, launch counting.
#include <mutex>
#include <string>
#include <vector>

#include "context.cuh"

namespace fxc {

static thread_local std::string g_last_error;
static thread_local int64_t g_launches = 0;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

void count_launch(int n) { g_launches += n; }

int num_sms() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (cached[dev] == 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      v = 148;
    cached[dev] = v;
  }
  return cached[dev];
}

int Scratch::reserve(size_t need) {
  if (need <= bytes) return FXC_OK;
  if (ptr) {
    cudaError_t e = cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    if (e != cudaSuccess) {
      set_error("cudaFree(scratch) failed: %s", cudaGetErrorString(e));
      return FXC_ERR_CUDA;
    }
  }
  size_t rounded = (need + (1u << 20) - 1) & ~size_t((1u << 20) - 1);
  cudaError_t e = cudaMalloc(&ptr, rounded);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    ptr = nullptr;
    set_error("cudaMalloc(%zu bytes of scratch) failed: %s", rounded, cudaGetErrorString(e));
    return FXC_ERR_NOMEM;
  }
  bytes = rounded;
  return FXC_OK;
}

void Scratch::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

int ctx_enter(fxc_ctx* ctx) {
  FXC_CHECK_ARG(ctx != nullptr, "null context");
  FXC_CUDA_TRY(cudaSetDevice(ctx->device));
  return FXC_OK;
}

// Reads (and clears) the device error word after the stream is idle.
int ctx_check_device_error(fxc_ctx* ctx) {
  int h = 0;
  FXC_CUDA_TRY(cudaMemcpy(&h, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (h != 0) {
    FXC_CUDA_TRY(cudaMemset(ctx->d_err, 0, sizeof(int)));
    set_error("a kernel's bounded wait timed out (device error word %d); results of that launch are invalid", h);
    return FXC_ERR_TIMEOUT;
  }
  return FXC_OK;
}

}  // namespace fxc

using namespace fxc;

extern "C" {

const char* fxc_last_error(void) { return g_last_error.c_str(); }

int fxc_version(void) { return 100; }

int64_t fxc_launch_count(void) { return g_launches; }

void fxc_launch_count_reset(void) { g_launches = 0; }

int fxc_ctx_create(int device, void* stream, fxc_ctx** out) {
  clear_error();
  FXC_CHECK_ARG(out != nullptr, "out is null");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    (void)cudaGetLastError();
    set_error("no CUDA device available (%s)", cudaGetErrorString(e));
    return FXC_ERR_NODEVICE;
  }
  FXC_CHECK_ARG(device >= 0 && device < count, "device %d out of range [0,%d)", device, count);
  FXC_CUDA_TRY(cudaSetDevice(device));
  cudaDeviceProp prop;
  FXC_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10) {
    set_error("device %d is sm_%d%d; this library is built for sm_103a only", device, prop.major,
              prop.minor);
    return FXC_ERR_UNSUPPORTED;
  }
  fxc_ctx* c = new (std::nothrow) fxc_ctx();
  if (!c) {
    set_error("host allocation of context failed");
    return FXC_ERR_NOMEM;
  }
  c->device = device;
  c->stream = (cudaStream_t)stream;
  c->num_sms = prop.multiProcessorCount;
  cudaError_t e1 = cudaMalloc(&c->d_err, 256);
  cudaError_t e2 = e1 == cudaSuccess ? cudaMemset(c->d_err, 0, 256) : e1;
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    (void)cudaGetLastError();
    if (c->d_err) cudaFree(c->d_err);
    delete c;
    set_error("allocation of the context error word failed: %s", cudaGetErrorString(e2));
    return FXC_ERR_NOMEM;
  }
  *out = c;
  return FXC_OK;
}

static void ktime_drop(fxc_ctx* ctx) {
  for (auto& r : ctx->ktimes) {
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.stop);
  }
  ctx->ktimes.clear();
}

int fxc_ctx_kernel_timing(fxc_ctx* ctx, int enable) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  if (!enable) {
    cudaStreamSynchronize(ctx->stream);
    ktime_drop(ctx);
  }
  ctx->ktime_on = enable != 0;
  return FXC_OK;
}

int fxc_ctx_kernel_time(fxc_ctx* ctx, const char* kernel, double* total_ms, int64_t* launches) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(kernel && total_ms && launches, "null argument");
  FXC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  double sum = 0.0;
  int64_t n = 0;
  std::vector<KernelTimeRec> keep;
  for (auto& r : ctx->ktimes) {
    if (r.name == kernel) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, r.start, r.stop) == cudaSuccess) {
        sum += ms;
        ++n;
      }
      cudaEventDestroy(r.start);
      cudaEventDestroy(r.stop);
    } else {
      keep.push_back(r);
    }
  }
  ctx->ktimes.swap(keep);
  *total_ms = sum;
  *launches = n;
  return FXC_OK;
}

int fxc_ctx_destroy(fxc_ctx* ctx) {
  if (!ctx) return FXC_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ktime_drop(ctx);
  ctx->scratch.release();
  ctx->scratch2.release();
  ctx->scratch3.release();
  ctx->scratch4.release();
  ctx->scratch5.release();
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  delete ctx;
  return FXC_OK;
}

int fxc_ctx_set_stream(fxc_ctx* ctx, void* stream) {
  FXC_CHECK_ARG(ctx != nullptr, "null context");
  ctx->stream = (cudaStream_t)stream;
  return FXC_OK;
}

int fxc_ctx_synchronize(fxc_ctx* ctx) {
  FXC_TRY(ctx_enter(ctx));
  FXC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ctx_check_device_error(ctx);
}

// ---- CUDA-graph capture of a launch sequence --------------------------------

struct fxc_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int device = 0;
};

int fxc_graph_begin(fxc_ctx* ctx) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(ctx->stream != nullptr, "graph capture needs a context on a non-default stream");
  FXC_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  return FXC_OK;
}

int fxc_graph_end(fxc_ctx* ctx, fxc_graph** out) {
  clear_error();
  FXC_CHECK_ARG(out != nullptr, "null output");
  *out = nullptr;
  FXC_TRY(ctx_enter(ctx));
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (e != cudaSuccess || g == nullptr) {
    (void)cudaGetLastError();
    if (g) cudaGraphDestroy(g);
    set_error("graph capture failed (a captured call synchronised or allocated?): %s", cudaGetErrorString(e));
    return FXC_ERR_CUDA;
  }
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    cudaGraphDestroy(g);
    set_error("graph instantiation failed: %s", cudaGetErrorString(e));
    return FXC_ERR_CUDA;
  }
  fxc_graph* r = new fxc_graph();
  r->graph = g;
  r->exec = x;
  r->device = ctx->device;
  *out = r;
  return FXC_OK;
}

int fxc_graph_launch(fxc_ctx* ctx, const fxc_graph* g) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(g != nullptr && g->exec != nullptr, "null graph");
  FXC_CHECK_ARG(g->device == ctx->device, "graph captured on device %d, context on %d", g->device, ctx->device);
  FXC_CUDA_TRY(cudaGraphLaunch(g->exec, ctx->stream));
  return FXC_OK;
}

int fxc_graph_destroy(fxc_graph* g) {
  if (!g) return FXC_OK;
  cudaSetDevice(g->device);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return FXC_OK;
}

int fxc_device_alloc(fxc_ctx* ctx, size_t bytes, void** out) {
  clear_error();
  FXC_CHECK_ARG(out != nullptr, "out is null");
  *out = nullptr;
  FXC_TRY(ctx_enter(ctx));
  if (bytes == 0) return FXC_OK;
  cudaError_t e = cudaMalloc(out, bytes);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    *out = nullptr;
    set_error("device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    return FXC_ERR_NOMEM;
  }
  return FXC_OK;
}

int fxc_device_free(fxc_ctx* ctx, void* ptr) {
  clear_error();
  if (!ptr) return FXC_OK;
  FXC_TRY(ctx_enter(ctx));
  FXC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  FXC_CUDA_TRY(cudaFree(ptr));
  return FXC_OK;
}

int fxc_host_alloc(size_t bytes, void** out) {
  clear_error();
  FXC_CHECK_ARG(out != nullptr, "out is null");
  *out = nullptr;
  if (bytes == 0) return FXC_OK;
  cudaError_t e = cudaMallocHost(out, bytes);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    *out = nullptr;
    set_error("page-locked host allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    return FXC_ERR_NOMEM;
  }
  return FXC_OK;
}

int fxc_host_free(void* ptr) {
  clear_error();
  if (!ptr) return FXC_OK;
  FXC_CUDA_TRY(cudaFreeHost(ptr));
  return FXC_OK;
}

int fxc_memcpy(fxc_ctx* ctx, void* dst, const void* src, size_t bytes, int kind) {
  clear_error();
  FXC_TRY(ctx_enter(ctx));
  FXC_CHECK_ARG(kind >= FXC_COPY_H2D && kind <= FXC_COPY_D2D, "invalid copy kind %d", kind);
  if (bytes == 0) return FXC_OK;
  FXC_CHECK_ARG(dst && src, "null pointer");
  const cudaMemcpyKind k = kind == FXC_COPY_H2D   ? cudaMemcpyHostToDevice
                           : kind == FXC_COPY_D2H ? cudaMemcpyDeviceToHost
                                                  : cudaMemcpyDeviceToDevice;
  FXC_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, k, ctx->stream));
  return FXC_OK;
}

}  // extern "C"
