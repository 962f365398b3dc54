// Host side of the FFT library: factorisation into Stockham stages and the
// per-device cache of twiddle tables.
#include <cmath>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "fft.cuh"

namespace fxc {

static const int kOddRadices[] = {3, 5, 7, 11, 13, 17, 19, 23, 29, 31};

static bool factorize(int n, std::vector<int>* out) {
  out->clear();
  if (n < 1) return false;
  int m = n;
  // powers of two: as many radix-8 stages as possible, then one 4 or 2
  int twos = 0;
  while (m % 2 == 0) {
    m /= 2;
    ++twos;
  }
  while (twos >= 3) {
    out->push_back(8);
    twos -= 3;
  }
  if (twos == 2) out->push_back(4);
  if (twos == 1) out->push_back(2);
  for (int r : kOddRadices) {
    while (m % r == 0) {
      out->push_back(r);
      m /= r;
    }
  }
  if (m != 1) return false;
  if ((int)out->size() > kFftMaxStages) return false;
  return true;
}

bool fft_length_supported(int n) {
  std::vector<int> f;
  return factorize(n, &f);
}

int fft_make_plan(int n, const float2* tw, int tw_stride, FftPlan* out) {
  std::vector<int> f;
  if (!factorize(n, &f)) {
    set_error("FFT length %d has a prime factor above 31 (not supported by the in-CTA FFT)", n);
    return FXC_ERR_UNSUPPORTED;
  }
  FftPlan p{};
  p.n = n;
  p.nstages = (int)f.size();
  for (int i = 0; i < p.nstages; ++i) p.radix[i] = f[i];
  p.tw = tw;
  p.tw_stride = tw_stride;
  p.perm = nullptr;
  FXC_TRY(fft_perm_table(p, &p.perm));
  *out = p;
  return FXC_OK;
}

int fft_make_plan_with(int n, const float2* tw, int tw_stride, const int* perm, FftPlan* out) {
  std::vector<int> f;
  if (!factorize(n, &f)) {
    set_error("FFT length %d has a prime factor above 31 (not supported by the in-CTA FFT)", n);
    return FXC_ERR_UNSUPPORTED;
  }
  FftPlan p{};
  p.n = n;
  p.nstages = (int)f.size();
  for (int i = 0; i < p.nstages; ++i) p.radix[i] = f[i];
  p.tw = tw;
  p.tw_stride = tw_stride;
  p.perm = perm;
  *out = p;
  return FXC_OK;
}

void fft_twiddle_values(int len, float2* out) {
  const double two_pi = 6.283185307179586476925286766559;
  for (int k = 0; k < len; ++k) {
    double a = two_pi * (double)k / (double)len;
    out[k] = make_float2((float)std::cos(a), (float)(-std::sin(a)));
  }
}

void fft_perm_values(const FftPlan& p, int* out) {
  for (int k = 0; k < p.n; ++k) out[k] = fft_digit_pos(p, k);
}

int fft_perm_table(const FftPlan& p, const int** out) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, int*> cache;
  int dev = 0;
  FXC_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_pair(dev, p.n);
  auto it = cache.find(key);
  if (it != cache.end()) {
    *out = it->second;
    return FXC_OK;
  }
  std::vector<int> h((size_t)p.n);
  for (int k = 0; k < p.n; ++k) h[k] = fft_digit_pos(p, k);
  int* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(int) * (size_t)p.n);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error("cudaMalloc of FFT permutation (n %d) failed: %s", p.n, cudaGetErrorString(e));
    return FXC_ERR_NOMEM;
  }
  e = cudaMemcpy(d, h.data(), sizeof(int) * (size_t)p.n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    set_error("upload of FFT permutation failed: %s", cudaGetErrorString(e));
    return FXC_ERR_CUDA;
  }
  cache[key] = d;
  *out = d;
  return FXC_OK;
}

int fft_twiddles(int len, const float2** out) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, float2*> cache;
  int dev = 0;
  FXC_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_pair(dev, len);
  auto it = cache.find(key);
  if (it != cache.end()) {
    *out = it->second;
    return FXC_OK;
  }
  std::vector<float2> h((size_t)len);
  // exp(-2 pi i k / len) evaluated in double from the reduced angle, so that
  // the table is symmetric and correctly rounded.
  const double two_pi = 6.283185307179586476925286766559;
  for (int k = 0; k < len; ++k) {
    double a = two_pi * (double)k / (double)len;
    h[k] = make_float2((float)std::cos(a), (float)(-std::sin(a)));
  }
  float2* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(float2) * (size_t)len);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error("cudaMalloc of twiddle table (len %d) failed: %s", len, cudaGetErrorString(e));
    return FXC_ERR_NOMEM;
  }
  e = cudaMemcpy(d, h.data(), sizeof(float2) * (size_t)len, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    set_error("upload of twiddle table failed: %s", cudaGetErrorString(e));
    return FXC_ERR_CUDA;
  }
  cache[key] = d;
  *out = d;
  return FXC_OK;
}

}  // namespace fxc
