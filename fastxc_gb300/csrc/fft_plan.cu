// Host side of the FFT library: factorisation into Stockham stages and the
// per-device cache of twiddle tables.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <map>
#include <tuple>
#include <mutex>
#include <utility>
#include <vector>

#include "fft.cuh"
#include "fft_any.cuh"

namespace fxc {

static const int kOddRadices[] = {3, 5, 7, 11, 13, 17, 19, 23, 29, 31};

// Largest composite radix for lengths above kFftSmallNmax, whose kernels run
// one 1024-thread CTA per SM (64 registers a thread): the register-resident
// butterflies of radix 12, 14, 15 and 21 spill there, so those lengths take
// one more pass over shared memory instead.
#ifndef FXC_FFT_LARGE_MAX_COMPOSITE
#define FXC_FFT_LARGE_MAX_COMPOSITE 21
#endif
constexpr int kSmallMaxComposite = 21;
constexpr int kFftSmallNmaxPlan = 4096;  // kFftSmallNmax of fft_launch.cuh

static int max_composite_for(int n) {
  return n > kFftSmallNmaxPlan ? FXC_FFT_LARGE_MAX_COMPOSITE : kSmallMaxComposite;
}

// Stages of an n-point transform: radix-8 stages for the powers of two, the
// leftover 2 or 4 folded with an odd prime into a composite radix (14, 10,
// 6 or 12), 3s folded with 5s (15), with 7s (21) or with each other (9),
// then the remaining primes; composites above max_composite_for(n) are not
// formed. Fewer stages mean fewer passes over shared memory and fewer
// barriers, as long as every radix fits one thread's registers.
// max_composite < 0: the default for the length (max_composite_for); 0: no
// composite radices; otherwise the largest composite formed.
static bool factorize(int n, std::vector<int>* out, int max_composite = -1) {
  out->clear();
  if (n < 1) return false;
  int m = n;
  int twos = 0;
  while (m % 2 == 0) {
    m /= 2;
    ++twos;
  }
  std::map<int, int> odd;  // prime -> multiplicity
  for (int r : kOddRadices) {
    while (m % r == 0) {
      ++odd[r];
      m /= r;
    }
  }
  if (m != 1) return false;
  auto take = [&](int r) {
    auto it = odd.find(r);
    if (it == odd.end() || it->second == 0) return false;
    --it->second;
    return true;
  };
  const int cmax = max_composite < 0 ? max_composite_for(n) : max_composite;
  for (; twos >= 3; twos -= 3) out->push_back(8);
  if (twos == 1) {
    if (cmax >= 14 && take(7)) out->push_back(14);
    else if (cmax >= 10 && take(5)) out->push_back(10);
    else if (cmax >= 6 && take(3)) out->push_back(6);
    else out->push_back(2);
  } else if (twos == 2) {
    if (cmax >= 12 && take(3)) out->push_back(12);
    else out->push_back(4);
  }
  while (cmax >= 15 && odd[3] >= 1 && odd[5] >= 1) {
    --odd[3];
    --odd[5];
    out->push_back(15);
  }
  while (cmax >= 21 && odd[3] >= 1 && odd[7] >= 1) {
    --odd[3];
    --odd[7];
    out->push_back(21);
  }
  while (cmax >= 9 && odd[3] >= 2) {
    odd[3] -= 2;
    out->push_back(9);
  }
  for (int r : kOddRadices)
    for (int k = 0; k < odd[r]; ++k) out->push_back(r);
  if ((int)out->size() > kFftMaxStages) return false;
  return true;
}

// Sub-transform lengths L_s = n / (radix[0] ... radix[s]) and their
// multiply-high magic numbers.
static void fill_lmag(FftPlan* p) {
  int L = p->n;
  for (int s = 0; s < kFftMaxStages; ++s) {
    if (s < p->nstages) {
      L /= p->radix[s];
      p->lmag[s] = fft_lmag(L);
    } else {
      p->lmag[s] = 0;
    }
  }
}

bool fft_length_supported(int n) {
  std::vector<int> f;
  return factorize(n, &f);
}

int fft_make_plan(int n, const float2* tw, int tw_stride, FftPlan* out, bool composites) {
  return fft_make_plan_limited(n, tw, tw_stride, out, composites ? -1 : 0);
}

int fft_make_plan_limited(int n, const float2* tw, int tw_stride, FftPlan* out, int max_composite) {
  std::vector<int> f;
  if (!factorize(n, &f, max_composite)) {
    set_error("FFT length %d has a prime factor above 31 (not supported by the in-CTA FFT)", n);
    return FXC_ERR_UNSUPPORTED;
  }
  FftPlan p{};
  p.n = n;
  p.nstages = (int)f.size();
  for (int i = 0; i < p.nstages; ++i) p.radix[i] = f[i];
  fill_lmag(&p);
  p.tw = tw;
  p.tw_stride = tw_stride;
  p.perm = nullptr;
  FXC_TRY(fft_perm_table(p, &p.perm));
  *out = p;
  return FXC_OK;
}

int fft_make_plan_ascending(int n, const float2* tw, int tw_stride, FftPlan* out) {
  std::vector<int> f;
  if (!factorize(n, &f)) {
    set_error("FFT length %d has a prime factor above 31 (not supported by the in-CTA FFT)", n);
    return FXC_ERR_UNSUPPORTED;
  }
  std::sort(f.begin(), f.end());
  FftPlan p{};
  p.n = n;
  p.nstages = (int)f.size();
  for (int i = 0; i < p.nstages; ++i) p.radix[i] = f[i];
  fill_lmag(&p);
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
  fill_lmag(&p);
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
  // one table per device, length and radix sequence (composite radices make
  // different digit orders for the same length)
  static std::map<std::tuple<int, int, std::vector<int>>, int*> cache;
  int dev = 0;
  FXC_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_tuple(dev, p.n, std::vector<int>(p.radix, p.radix + p.nstages));
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

int fft_iperm_table(const FftPlan& p, const int** out) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, std::vector<int>>, int*> cache;
  int dev = 0;
  FXC_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_tuple(dev, p.n, std::vector<int>(p.radix, p.radix + p.nstages));
  auto it = cache.find(key);
  if (it != cache.end()) {
    *out = it->second;
    return FXC_OK;
  }
  std::vector<int> h((size_t)p.n);
  for (int k = 0; k < p.n; ++k) h[(size_t)fft_digit_pos(p, k)] = k;
  int* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(int) * (size_t)p.n);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error("cudaMalloc of FFT inverse permutation (n %d) failed: %s", p.n, cudaGetErrorString(e));
    return FXC_ERR_NOMEM;
  }
  e = cudaMemcpy(d, h.data(), sizeof(int) * (size_t)p.n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    set_error("upload of FFT inverse permutation failed: %s", cudaGetErrorString(e));
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

// ---------------------------------------------------------------------------
// Bluestein tables
// ---------------------------------------------------------------------------

// Forward DFT (exp(-)) of a 2-3-5-7-smooth length in double precision:
// recursive decimation in time by the smallest prime factor.
static void host_fft(std::vector<std::complex<double>>& a) {
  const size_t n = a.size();
  if (n <= 1) return;
  size_t r = 2;
  while (n % r) ++r;
  const size_t l = n / r;
  std::vector<std::vector<std::complex<double>>> sub(r, std::vector<std::complex<double>>(l));
  for (size_t j = 0; j < l; ++j)
    for (size_t q = 0; q < r; ++q) sub[q][j] = a[j * r + q];
  for (size_t q = 0; q < r; ++q) host_fft(sub[q]);
  const double two_pi = 6.283185307179586476925286766559;
  for (size_t k = 0; k < n; ++k) {
    std::complex<double> acc = 0.0;
    for (size_t q = 0; q < r; ++q) {
      const double ang = -two_pi * (double)((q * k) % n) / (double)n;
      acc += sub[q][k % l] * std::complex<double>(std::cos(ang), std::sin(ang));
    }
    a[k] = acc;
  }
}

static bool smooth2357(int m) {
  for (int r : {2, 3, 5, 7})
    while (m % r == 0) m /= r;
  return m == 1;
}

static int upload(const void* h, size_t bytes, void** d) {
  cudaError_t e = cudaMalloc(d, bytes);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error("cudaMalloc of %zu bytes for FFT tables failed: %s", bytes, cudaGetErrorString(e));
    return FXC_ERR_NOMEM;
  }
  e = cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(*d);
    set_error("upload of FFT tables failed: %s", cudaGetErrorString(e));
    return FXC_ERR_CUDA;
  }
  return FXC_OK;
}

int any_plan(int n, int direct_max, int bluestein_max, AnyPlan* out) {
  FXC_CHECK_ARG(n >= 1, "transform length %d", n);
  AnyPlan a{};
  a.n = n;
  if (n <= direct_max && fft_length_supported(n)) {
    const float2* tw = nullptr;
    FXC_TRY(fft_twiddles(n, &tw));
    FXC_TRY(fft_make_plan(n, tw, 1, &a.p, false));
    FXC_TRY(fft_iperm_table(a.p, &a.iperm));
    *out = a;
    return FXC_OK;
  }
  int m = 2 * n - 1;
  while (!smooth2357(m)) ++m;
  if (m > bluestein_max) {
    set_error("transform length %d needs a Bluestein length %d above the in-CTA limit %d", n, m,
              bluestein_max);
    return FXC_ERR_UNSUPPORTED;
  }
  const float2* tw = nullptr;
  FXC_TRY(fft_twiddles(m, &tw));
  FXC_TRY(fft_make_plan(m, tw, 1, &a.p, false));
  static std::mutex mu;
  static std::map<std::pair<int, int>, std::pair<float2*, float2*>> cache;
  int dev = 0;
  FXC_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_pair(dev, n);
  auto it = cache.find(key);
  if (it == cache.end()) {
    // w_k = exp(-i pi k^2 / n) with k^2 reduced mod 2n; kernel b_j = conj(w_j)
    // for |j| < n placed circularly in length m; khat = DFT_m(b) / m stored at
    // the DIF position of each frequency.
    const double pi = 3.14159265358979323846264338327950288;
    std::vector<std::complex<double>> w((size_t)n), b((size_t)m, 0.0);
    for (int k = 0; k < n; ++k) {
      const uint64_t q = ((uint64_t)k * (uint64_t)k) % (2ull * (uint64_t)n);
      const double ang = pi * (double)q / (double)n;
      w[k] = std::complex<double>(std::cos(ang), -std::sin(ang));
    }
    b[0] = std::conj(w[0]);
    for (int j = 1; j < n; ++j) b[j] = b[(size_t)m - j] = std::conj(w[j]);
    host_fft(b);
    std::vector<float2> hw((size_t)n), hk((size_t)m);
    for (int k = 0; k < n; ++k) hw[k] = make_float2((float)w[k].real(), (float)w[k].imag());
    for (int k = 0; k < m; ++k) {
      const std::complex<double> v = b[k] / (double)m;
      hk[fft_digit_pos(a.p, k)] = make_float2((float)v.real(), (float)v.imag());
    }
    void *dw = nullptr, *dk = nullptr;
    FXC_TRY(upload(hw.data(), sizeof(float2) * hw.size(), &dw));
    const int rc = upload(hk.data(), sizeof(float2) * hk.size(), &dk);
    if (rc != FXC_OK) {
      cudaFree(dw);
      return rc;
    }
    it = cache.emplace(key, std::make_pair((float2*)dw, (float2*)dk)).first;
  }
  a.chirp = it->second.first;
  a.khat = it->second.second;
  *out = a;
  return FXC_OK;
}

}  // namespace fxc
