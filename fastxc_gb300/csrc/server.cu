// Correlation serving engine: a request loop over resident station spectra.
//
// No counterpart in the reference (its stages are batch executables). A job
// asks for the linear-stack NCFs of every cross-station component pair of a
// station subarray over a day range, optionally with a phase-weighted stack
// over the days. The engine
//   * keeps station-day spectra ([nstep windows][3 components][nspec]
//     complex, the stepack payload of one station-day) resident in an HBM
//     arena with LRU eviction of entries no running job uses; entries come
//     from fxc_server_put_spectra or, in synthetic mode, from a seeded
//     generator kernel (a cache fill);
//   * admits queued jobs first-fit by free working memory (a second HBM
//     arena) and free slots -- a job that waited longer than
//     max_wait_s blocks later ones from passing it;
//   * runs every admitted job on its own slot (host thread + CUDA stream +
//     library context), so jobs that arrive while others run overlap on the
//     device: continuous batching at job granularity;
//   * per job: gathers the subarray's spectra chunk by chunk into a
//     [windows][channels][nspec] block, stacks all pairs with the tensor-core
//     or plain kernel (accumulating over chunks), finalizes the NCFs and, for
//     PWS jobs, stacks the per-day NCFs with fxc_pws_run; results are copied
//     to host memory and the device memory is returned at once.
// Every result depends only on the job and its spectra (all kernels are
// deterministic), so a job's NCFs are the same alone and in any mix.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "context.cuh"
#include "xc.cuh"

namespace fxc {

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over one device arena (offsets, 256-byte aligned).
class Arena {
 public:
  int init(size_t bytes) {
    bytes_ = bytes & ~size_t(255);
    cudaError_t e = cudaMalloc(&base_, bytes_);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      base_ = nullptr;
      set_error("server arena of %zu bytes: %s", bytes_, cudaGetErrorString(e));
      return FXC_ERR_NOMEM;
    }
    free_.clear();
    free_[0] = bytes_;
    used_ = 0;
    return FXC_OK;
  }
  void release() {
    if (base_) cudaFree(base_);
    base_ = nullptr;
  }
  // nullptr when no free block is large enough
  char* alloc(size_t n) {
    n = (n + 255) & ~size_t(255);
    if (n == 0) n = 256;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < n) continue;
      const size_t off = it->first, len = it->second;
      free_.erase(it);
      if (len > n) free_[off + n] = len - n;
      used_ += n;
      sizes_[off] = n;
      return base_ + off;
    }
    return nullptr;
  }
  void free(char* p) {
    if (!p) return;
    const size_t off = (size_t)(p - base_);
    auto s = sizes_.find(off);
    if (s == sizes_.end()) return;
    size_t n = s->second;
    sizes_.erase(s);
    used_ -= n;
    size_t start = off;
    auto next = free_.lower_bound(off);
    if (next != free_.end() && next->first == off + n) {
      n += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        start = prev->first;
        n += prev->second;
        free_.erase(prev);
      }
    }
    free_[start] = n;
  }
  size_t bytes() const { return bytes_; }
  size_t used() const { return used_; }

 private:
  char* base_ = nullptr;
  size_t bytes_ = 0, used_ = 0;
  std::map<size_t, size_t> free_;   // offset -> length
  std::map<size_t, size_t> sizes_;  // allocated offset -> length
};

// Seeded synthetic station-day spectra: per (window, bin) a common complex
// source term with a station-dependent delay plus station noise; values are
// a pure function of (seed, station, day, delta code, window, component, bin).
__device__ __forceinline__ uint32_t mix32(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return (uint32_t)x;
}
__device__ __forceinline__ float unit(uint64_t key) {
  return (float)(mix32(key) >> 8) * (1.0f / 8388608.0f) - 1.0f;  // [-1, 1)
}

__global__ void k_synth_spectra(float2* __restrict__ out, int nstep, int nspec, uint64_t seed,
                                int station, int day, int dcode) {
  const int64_t total = (int64_t)nstep * 3 * nspec;
  const float tau = 0.01f * (float)(station % 997);  // delay in units of 1/nspec cycles
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int f = (int)(i % nspec);
    const int64_t wc = i / nspec;
    const int c = (int)(wc % 3);
    const int w = (int)(wc / 3);
    const uint64_t kc = (((seed * 1000003ull + (uint64_t)day) * 131ull + (uint64_t)dcode) * 100003ull +
                         (uint64_t)w) * 65537ull + (uint64_t)f;
    const float sr = unit(kc * 2 + 1), si = unit(kc * 2 + 2);
    float sn, cs;
    sincospif(2.0f * tau * (float)f / (float)nspec, &sn, &cs);
    const uint64_t kn = ((kc * 1009ull + (uint64_t)station) * 7ull + (uint64_t)c) * 2ull;
    out[i] = make_float2(0.8f * (sr * cs - si * sn) + unit(kn + 11), 0.8f * (sr * sn + si * cs) + unit(kn + 12));
  }
}

// chunk[w][c][f] = entry[ent(w / nstep, c / 3)][w % nstep][c % 3][f]
// chunk[w][c][0, fw) = entry[w / nstep][c / 3][w % nstep][c % 3][f0, f0 + fw)
__global__ void k_gather_spectra(const float2* const* __restrict__ entries, int nsta, int ndays,
                                 int nstep, int nspec, int f0, int fw, float2* __restrict__ chunk) {
  const int nchan = 3 * nsta;
  const int64_t rows = (int64_t)ndays * nstep * nchan;
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const int c = (int)(r % nchan);
    const int64_t w = r / nchan;
    const int d = (int)(w / nstep), ws = (int)(w % nstep);
    const float2* src = entries[(int64_t)d * nsta + c / 3] + ((int64_t)ws * 3 + c % 3) * nspec + f0;
    float2* dst = chunk + r * fw;
    for (int f = threadIdx.x; f < fw; f += blockDim.x) dst[f] = __ldg(src + f);
  }
}

struct Entry {
  char* ptr = nullptr;
  size_t bytes = 0;
  int refs = 0;
  uint64_t tick = 0;
  cudaEvent_t ready = nullptr;  // recorded after the fill
  cudaEvent_t last = nullptr;   // recorded after the last use
};

// Working-memory layout of a job (byte offsets into its work block). Linear
// jobs: K days pinned per pass group, bins gathered fchunk at a time, the
// stack accumulated over the day groups. PWS jobs: one day at a time (all
// bins), streaming phasor / linear sums over the days.
struct Layout {
  int K = 1;
  int64_t blk = 0;  // pairs held at once (all of the job's)
  size_t chunk = 0, packed = 0, stack = 0, ncf = 0, ptrs = 0, traces = 0, lin = 0, out = 0;
  size_t total = 0;
};

struct Job {
  int64_t id = 0;
  fxc_job desc{};
  std::vector<int32_t> stations;
  // geometry
  int nspec = 0, nstep = 0, cc_size = 0, kdays = 1, fchunk = 0;
  fxc_xc_shape shape{};
  int64_t npairs = 0;
  size_t work_bytes = 0;
  size_t entry_bytes = 0;
  Layout layout;
  // state
  int status = 0;  // 0 queued, 1 running, 2 done, < 0 error code
  std::string error;
  double t_submit = 0, t_start = 0, t_end = 0;
  std::vector<float> ncf, pws;
};

struct EntryKey {
  int station, day, dcode;
  bool operator<(const EntryKey& o) const {
    if (station != o.station) return station < o.station;
    if (day != o.day) return day < o.day;
    return dcode < o.dcode;
  }
};
EntryKey key_of(int station, int day, int dcode) { return EntryKey{station, day, dcode}; }

}  // namespace

}  // namespace fxc

using namespace fxc;

struct fxc_server {
  fxc_server_config cfg{};
  Arena cache, work;
  std::mutex mu;  // cache, work arena, queue, jobs
  std::condition_variable cv;
  std::map<EntryKey, Entry> entries;
  uint64_t tick = 0;
  std::deque<Job*> queue;
  std::map<int64_t, Job*> jobs;
  int64_t next_id = 1;
  int free_slots = 0;
  int waiters = 0;
  bool stop = false;
  std::vector<std::thread> threads;
  std::vector<fxc_ctx*> ctxs;
  std::vector<cudaStream_t> streams;
  std::atomic<int64_t> done_jobs{0}, pair_windows{0};
  // geometry cache per delta code
  std::map<int, std::pair<int, int>> geom;  // dcode -> (nspec, nstep)
};

namespace fxc {
namespace {

int dcode_of(float delta) { return (int)llround((double)delta * 1e6); }

// nspec / nstep of one station-day's spectra at this delta: the sac2spec
// planning for a day-long record, the configured window and shift, and the
// largest lag the engine serves (lag_max_s).
int geometry(fxc_server* s, float delta, int* nspec, int* nstep) {
  const int dc = dcode_of(delta);
  auto it = s->geom.find(dc);
  if (it == s->geom.end()) {
    const double b[5] = {1, 0, 0, 0, 0}, a[5] = {1, 0, 0, 0, 0};
    const float lo = 0.1f, hi = 1.0f;
    fxc_s2s_plan p;
    FXC_TRY(fxc_s2s_plan_init(86400.0f, s->cfg.win_len, s->cfg.win_len, s->cfg.lag_max, delta, b, a, &lo, &hi, 1,
                              0, 0, 0, &p));
    it = s->geom.emplace(dc, std::make_pair((int)p.nspec, (int)p.nstep)).first;
  }
  *nspec = it->second.first;
  *nstep = it->second.second;
  return FXC_OK;
}

// Pins (and fills if absent) every entry of one chunk; makes `stream` wait
// for their fills. Called with s->mu held. Returns FXC_ERR_NOMEM when the
// cache cannot make room now (the caller retries later).
int pin_entries(fxc_server* s, const Job* j, int day0, int ndays, cudaStream_t stream,
                std::vector<const float2*>* ptrs, std::vector<EntryKey>* keys) {
  const int dc = dcode_of(j->desc.delta);
  ptrs->clear();
  keys->clear();
  for (int d = 0; d < ndays; ++d) {
    for (int st : j->stations) {
      const EntryKey k = key_of(st, day0 + d, dc);
      auto it = s->entries.find(k);
      if (it == s->entries.end()) {
        if (!s->cfg.synthetic) {
          set_error("spectra of station %d day %d delta %g are not resident", st, day0 + d, j->desc.delta);
          for (const EntryKey& kk : *keys) --s->entries[kk].refs;
          return FXC_ERR_INVALID;
        }
        char* p = s->cache.alloc(j->entry_bytes);
        while (!p) {
          // evict the least recently used entry that no job holds and whose
          // last use has completed
          EntryKey victim{0, 0, 0};
          uint64_t best = UINT64_MAX;
          bool found = false;
          for (auto& kv : s->entries) {
            Entry& e = kv.second;
            if (e.refs > 0 || e.tick >= best) continue;
            if (e.last && cudaEventQuery(e.last) != cudaSuccess) continue;
            if (e.ready && cudaEventQuery(e.ready) != cudaSuccess) continue;
            best = e.tick;
            victim = kv.first;
            found = true;
          }
          if (!found) {
            for (const EntryKey& kk : *keys) --s->entries[kk].refs;
            set_error("spectra cache full (%zu bytes in use)", s->cache.used());
            return FXC_ERR_NOMEM;
          }
          Entry& e = s->entries[victim];
          s->cache.free(e.ptr);
          if (e.ready) cudaEventDestroy(e.ready);
          if (e.last) cudaEventDestroy(e.last);
          s->entries.erase(victim);
          p = s->cache.alloc(j->entry_bytes);
        }
        Entry e;
        e.ptr = p;
        e.bytes = j->entry_bytes;
        cudaEventCreateWithFlags(&e.ready, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&e.last, cudaEventDisableTiming);
        k_synth_spectra<<<1024, 256, 0, stream>>>(reinterpret_cast<float2*>(p), j->nstep, j->nspec, s->cfg.seed,
                                                   st, day0 + d, dc);
        count_launch();
        cudaEventRecord(e.ready, stream);
        it = s->entries.emplace(k, e).first;
      } else if (it->second.ready) {
        cudaStreamWaitEvent(stream, it->second.ready, 0);
      }
      Entry& e = it->second;
      ++e.refs;
      e.tick = ++s->tick;
      ptrs->push_back(reinterpret_cast<const float2*>(e.ptr));
      keys->push_back(k);
    }
  }
  return FXC_OK;
}

void unpin_entries(fxc_server* s, const std::vector<EntryKey>& keys, cudaStream_t stream) {
  for (const EntryKey& k : keys) {
    auto it = s->entries.find(k);
    if (it == s->entries.end()) continue;
    --it->second.refs;
    if (it->second.last) cudaEventRecord(it->second.last, stream);
  }
}

#define JOB_TRY(expr)             \
  do {                            \
    const int _rc = (expr);       \
    if (_rc != FXC_OK) return _rc; \
  } while (0)

size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

Layout job_layout(const Job* j) {
  Layout L;
  const int nsta = (int)j->stations.size(), nchan = 3 * nsta;
  const bool pws = j->desc.pws != 0;
  const size_t cc = (size_t)j->cc_size, pitch = (size_t)xc_stack_pitch(j->nspec);
  L.K = pws ? 1 : j->kdays;
  L.blk = j->npairs;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += al256(bytes);
    return o;
  };
  const int fw = pws ? j->nspec : j->fchunk;  // bins gathered per pass
  L.chunk = take((size_t)L.K * j->nstep * nchan * fw * 8);
  L.packed = take(j->desc.method != FXC_XC_PLAIN ? (size_t)xc_packed_chunks(nchan, (int64_t)L.K * j->nstep, fw) * 16 : 0);
  L.stack = take((size_t)L.blk * pitch * 8);
  L.ncf = take((size_t)L.blk * cc * 4);
  L.ptrs = take((size_t)L.K * nsta * sizeof(void*));
  if (pws) {
    L.traces = take((size_t)L.blk * cc * 8);  // streaming phasor sums (complex)
    L.lin = take((size_t)L.blk * cc * 4);
    L.out = take((size_t)L.blk * cc * 4);
  }
  L.total = off;
  return L;
}

// Pins days [day, day + nd) of the job's stations (filled on a miss) and
// uploads their entry pointers to d_ptrs.
int pin_days(fxc_server* s, Job* j, int day, int nd, cudaStream_t st, const float2** d_ptrs,
             std::vector<EntryKey>* keys) {
  std::vector<const float2*> ptrs;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    int rc;
    // the cache may be full of entries other running jobs hold: wait for them
    while ((rc = pin_entries(s, j, day, nd, st, &ptrs, keys)) == FXC_ERR_NOMEM && !s->stop)
      s->cv.wait_for(lk, std::chrono::milliseconds(2));
    JOB_TRY(rc);
  }
  FXC_CUDA_TRY(cudaMemcpyAsync(d_ptrs, ptrs.data(), ptrs.size() * sizeof(void*), cudaMemcpyHostToDevice, st));
  // the host pointer table must outlive the upload
  FXC_CUDA_TRY(cudaStreamSynchronize(st));
  return FXC_OK;
}

int gather_bins(Job* j, int nd, int f0, int fw, cudaStream_t st, const float2** d_ptrs, float2* chunk) {
  const int nsta = (int)j->stations.size();
  const int64_t rows = (int64_t)nd * j->nstep * 3 * nsta;
  k_gather_spectra<<<(unsigned)std::min<int64_t>(rows, 152 * 64), 256, 0, st>>>(d_ptrs, nsta, nd, j->nstep, j->nspec,
                                                                               f0, fw, chunk);
  count_launch();
  FXC_LAUNCH_CHECK();
  return FXC_OK;
}

void unpin_days(fxc_server* s, const std::vector<EntryKey>& keys, cudaStream_t st) {
  std::lock_guard<std::mutex> lk(s->mu);
  unpin_entries(s, keys, st);
}

struct PlanGuard {
  fxc_pairplan* p = nullptr;
  ~PlanGuard() { fxc_pairplan_destroy(p); }
};

int run_job(fxc_server* s, int slot, Job* j, char* work) {
  fxc_ctx* ctx = s->ctxs[slot];
  cudaStream_t st = s->streams[slot];
  const int nsta = (int)j->stations.size();
  const int nchan = 3 * nsta;
  const int D = j->desc.ndays;
  const int nspec = j->nspec, nstep = j->nstep;
  const int64_t pitch = xc_stack_pitch(nspec);
  int method = j->desc.method;  // < 0: autotuned on the first gathered block
  const Layout& L = j->layout;
  float2* chunk = reinterpret_cast<float2*>(work + L.chunk);
  uint4* packed = reinterpret_cast<uint4*>(work + L.packed);
  float2* stack = reinterpret_cast<float2*>(work + L.stack);
  float* ncf = reinterpret_cast<float*>(work + L.ncf);
  const float2** d_ptrs = reinterpret_cast<const float2**>(work + L.ptrs);
  // pair list: station pairs a < b in job order, components i, j
  std::vector<int32_t> src, rec;
  src.reserve((size_t)j->npairs);
  rec.reserve((size_t)j->npairs);
  for (int a = 0; a < nsta; ++a)
    for (int b = a + 1; b < nsta; ++b)
      for (int ci = 0; ci < 3; ++ci)
        for (int cj = 0; cj < 3; ++cj) {
          src.push_back(3 * a + ci);
          rec.push_back(3 * b + cj);
        }
  const size_t cc = (size_t)j->cc_size;
  if (s->cfg.keep_results) {
    j->ncf.resize((size_t)j->npairs * cc);
    if (j->desc.pws) j->pws.resize((size_t)j->npairs * cc);
  }
  PlanGuard pg;
  JOB_TRY(fxc_pairplan_create(ctx, src.data(), rec.data(), j->npairs, nchan, &pg.p));
  // one stacking pass: bins [f0, f0 + fw) of the nd pinned days into
  // stack[:, f0 : f0 + fw) (added to it when accumulate)
  auto pass = [&](int nd, int f0, int fw, float scale, int accumulate) -> int {
    const int64_t nwin = (int64_t)nd * nstep;
    int rc = gather_bins(j, nd, f0, fw, st, d_ptrs, chunk);
    if (rc == FXC_OK && method < 0) {
      int32_t m = FXC_XC_PLAIN;
      rc = fxc_xc_autotune(ctx, pg.p, reinterpret_cast<const float*>(chunk), nwin, nchan, fw, fw, &m, nullptr, nullptr);
      method = m;
    }
    if (rc != FXC_OK) return rc;
    if (method == FXC_XC_TENSOR) {
      rc = xc_pack_launch(ctx, chunk, nwin, nchan, fw, fw, nullptr, packed);
      if (rc == FXC_OK) rc = xc_gemm_launch(ctx, pg.p, packed, nwin, fw, scale, stack + f0, pitch, accumulate);
      return rc;
    }
    return xc_stack_launch(ctx, pg.p, chunk, nwin, nchan, fw, fw, nullptr, scale, stack + f0, pitch, FXC_XC_PLAIN,
                           accumulate);
  };
  if (!j->desc.pws) {
    const float scale = 1.0f / (float)(D * nstep);
    for (int d0 = 0; d0 < D; d0 += L.K) {
      const int nd = std::min(L.K, D - d0);
      std::vector<EntryKey> keys;
      JOB_TRY(pin_days(s, j, j->desc.day0 + d0, nd, st, d_ptrs, &keys));
      int rc = FXC_OK;
      // all windows of the pinned days per pass, bins in passes of fchunk
      for (int f0 = 0; f0 < nspec && rc == FXC_OK; f0 += j->fchunk)
        rc = pass(nd, f0, std::min(j->fchunk, nspec - f0), scale, d0 > 0);
      unpin_days(s, keys, st);
      JOB_TRY(rc);
    }
    JOB_TRY(xc_finalize_launch(ctx, stack, j->npairs, pitch, &j->shape, ncf));
    if (s->cfg.keep_results)
      FXC_CUDA_TRY(cudaMemcpyAsync(j->ncf.data(), ncf, (size_t)j->npairs * cc * 4, cudaMemcpyDeviceToHost, st));
  } else {
    // PWS over the days, streamed: per day the NCF of every pair, its unit
    // analytic phasor and the NCF itself are added (weight 1/D) to running
    // sums; PWS = linear x |phasor sum|^power at the end
    float* acc = reinterpret_cast<float*>(work + L.traces);
    float* lin = reinterpret_cast<float*>(work + L.lin);
    float* out = reinterpret_cast<float*>(work + L.out);
    FXC_CUDA_TRY(cudaMemsetAsync(acc, 0, (size_t)j->npairs * cc * 8, st));
    FXC_CUDA_TRY(cudaMemsetAsync(lin, 0, (size_t)j->npairs * cc * 4, st));
    for (int d = 0; d < D; ++d) {
      std::vector<EntryKey> keys;
      JOB_TRY(pin_days(s, j, j->desc.day0 + d, 1, st, d_ptrs, &keys));
      const int rc = pass(1, 0, nspec, 1.0f / (float)nstep, 0);
      unpin_days(s, keys, st);
      JOB_TRY(rc);
      JOB_TRY(xc_finalize_launch(ctx, stack, j->npairs, pitch, &j->shape, ncf));
      JOB_TRY(fxc_pws_stream_add(ctx, ncf, (int64_t)cc, (int32_t)j->npairs, j->cc_size, 1.0f / (float)D, acc, lin));
    }
    JOB_TRY(fxc_pws_stream_finish(ctx, acc, lin, (int32_t)j->npairs, j->cc_size, j->desc.pws_power, out));
    if (s->cfg.keep_results) {
      FXC_CUDA_TRY(cudaMemcpyAsync(j->ncf.data(), lin, (size_t)j->npairs * cc * 4, cudaMemcpyDeviceToHost, st));
      FXC_CUDA_TRY(cudaMemcpyAsync(j->pws.data(), out, (size_t)j->npairs * cc * 4, cudaMemcpyDeviceToHost, st));
    }
  }
  FXC_CUDA_TRY(cudaStreamSynchronize(st));
  return ctx_check_device_error(ctx);
}

void slot_main(fxc_server* s, int slot) {
  cudaSetDevice(s->cfg.device);
  for (;;) {
    Job* j = nullptr;
    char* work = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      for (;;) {
        if (s->stop) return;
        // first fit in arrival order; a job that waited past max_wait_s is
        // not overtaken
        const double t = now_s();
        for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
          Job* c = *it;
          char* w = s->work.alloc(c->work_bytes);
          if (w) {
            j = c;
            work = w;
            s->queue.erase(it);
            break;
          }
          if (t - c->t_submit > s->cfg.max_wait_s) break;
        }
        if (j) break;
        s->cv.wait_for(lk, std::chrono::milliseconds(5));
      }
      j->status = 1;
      j->t_start = now_s();
    }
    const int rc = run_job(s, slot, j, work);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->work.free(work);
      j->t_end = now_s();
      if (rc == FXC_OK) {
        j->status = 2;
        s->done_jobs++;
        s->pair_windows += j->npairs * (int64_t)j->desc.ndays * j->nstep;
      } else {
        j->status = rc;
        j->error = fxc_last_error();
      }
    }
    s->cv.notify_all();
  }
}

}  // namespace
}  // namespace fxc

extern "C" {

int fxc_server_create(const fxc_server_config* cfg, fxc_server** out) {
  clear_error();
  FXC_CHECK_ARG(cfg && out, "null argument");
  FXC_CHECK_ARG(cfg->slots >= 1 && cfg->slots <= 64, "slots %d outside [1, 64]", cfg->slots);
  FXC_CHECK_ARG(cfg->cache_gib > 0 && cfg->work_gib > 0, "arena sizes must be positive");
  FXC_CHECK_ARG(cfg->win_len > 0 && cfg->lag_max > 0, "win_len and lag_max must be positive");
  *out = nullptr;
  fxc_server* s = new fxc_server();
  s->cfg = *cfg;
  if (s->cfg.max_wait_s <= 0) s->cfg.max_wait_s = 1e30;
  FXC_CUDA_TRY(cudaSetDevice(cfg->device));
  int rc = s->cache.init((size_t)(cfg->cache_gib * 1073741824.0));
  if (rc == FXC_OK) rc = s->work.init((size_t)(cfg->work_gib * 1073741824.0));
  for (int i = 0; rc == FXC_OK && i < cfg->slots; ++i) {
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      set_error("stream creation failed");
      rc = FXC_ERR_CUDA;
      break;
    }
    s->streams.push_back(st);
    fxc_ctx* c = nullptr;
    rc = fxc_ctx_create(cfg->device, st, &c);
    if (rc == FXC_OK) s->ctxs.push_back(c);
  }
  if (rc != FXC_OK) {
    const std::string msg = fxc_last_error();
    for (fxc_ctx* c : s->ctxs) fxc_ctx_destroy(c);
    for (cudaStream_t st : s->streams) cudaStreamDestroy(st);
    s->cache.release();
    s->work.release();
    delete s;
    set_error("%s", msg.c_str());
    return rc;
  }
  for (int i = 0; i < cfg->slots; ++i) s->threads.emplace_back(slot_main, s, i);
  *out = s;
  return FXC_OK;
}

int fxc_server_put_spectra(fxc_server* s, int32_t station, int32_t day, float delta, const float* h_spec) {
  clear_error();
  FXC_CHECK_ARG(s && h_spec, "null argument");
  int nspec = 0, nstep = 0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    FXC_TRY(geometry(s, delta, &nspec, &nstep));
  }
  const size_t bytes = (size_t)nstep * 3 * nspec * 8;
  std::lock_guard<std::mutex> lk(s->mu);
  const EntryKey k = key_of(station, day, dcode_of(delta));
  auto it = s->entries.find(k);
  FXC_CHECK_ARG(it == s->entries.end() || it->second.refs == 0, "entry in use");
  char* p = it != s->entries.end() ? it->second.ptr : s->cache.alloc(bytes);
  if (!p) {
    set_error("spectra cache full");
    return FXC_ERR_NOMEM;
  }
  FXC_CUDA_TRY(cudaMemcpy(p, h_spec, bytes, cudaMemcpyHostToDevice));
  if (it == s->entries.end()) {
    Entry e;
    e.ptr = p;
    e.bytes = bytes;
    e.tick = ++s->tick;
    cudaEventCreateWithFlags(&e.last, cudaEventDisableTiming);
    s->entries.emplace(k, e);
  }
  return FXC_OK;
}

int fxc_server_geometry(fxc_server* s, float delta, int32_t* nspec, int32_t* nstep) {
  clear_error();
  FXC_CHECK_ARG(s && nspec && nstep, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  int a = 0, b = 0;
  FXC_TRY(geometry(s, delta, &a, &b));
  *nspec = a;
  *nstep = b;
  return FXC_OK;
}

int fxc_server_submit(fxc_server* s, const fxc_job* job, int64_t* id) {
  clear_error();
  FXC_CHECK_ARG(s && job && id && job->stations, "null argument");
  FXC_CHECK_ARG(job->nsta >= 2 && job->ndays >= 1, "a job needs >= 2 stations and >= 1 day");
  FXC_CHECK_ARG(job->method == FXC_XC_PLAIN || job->method == FXC_XC_TENSOR || job->method == -1,
                "unknown method %d", job->method);
  FXC_CHECK_ARG(job->lag > 0 && job->lag <= s->cfg.lag_max, "lag %g outside (0, %g]", job->lag, s->cfg.lag_max);
  Job* j = new Job();
  j->desc = *job;
  j->stations.assign(job->stations, job->stations + job->nsta);
  j->desc.stations = nullptr;
  int rc;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    rc = geometry(s, job->delta, &j->nspec, &j->nstep);
  }
  if (rc == FXC_OK) rc = fxc_xc_shape_init(j->nspec, j->nstep, job->delta, job->lag, &j->shape);
  if (rc != FXC_OK) {
    delete j;
    return rc;
  }
  j->cc_size = j->shape.cc_size;
  j->npairs = 9LL * job->nsta * (job->nsta - 1) / 2;
  j->entry_bytes = (size_t)j->nstep * 3 * j->nspec * 8;
  // days per pass: the pinned station-days of one pass stay within half the
  // spectra arena; bins per pass: the gathered block stays within chunk_gib
  const size_t day_entries = (size_t)job->nsta * j->entry_bytes;
  if (day_entries > s->cache.bytes() / 2) {
    set_error("one day of %d stations needs %zu bytes of spectra, above half the arena (%zu)", job->nsta,
              day_entries, s->cache.bytes());
    delete j;
    return FXC_ERR_NOMEM;
  }
  j->kdays = std::max(1, std::min<int>(job->ndays, (int)(s->cache.bytes() / 2 / day_entries)));
  {
    const double per_bin = (double)j->kdays * j->nstep * 3 * job->nsta * 8 * (job->method != FXC_XC_PLAIN ? 2 : 1);
    int fc = (int)(s->cfg.chunk_gib * 1073741824.0 / per_bin) / 64 * 64;
    j->fchunk = std::max(64, std::min(fc, j->nspec));
  }
  j->layout = job_layout(j);
  j->work_bytes = j->layout.total;
  if (j->work_bytes > s->work.bytes()) {
    set_error("job needs %zu bytes of working memory, the arena holds %zu", j->work_bytes, s->work.bytes());
    delete j;
    return FXC_ERR_NOMEM;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    j->id = s->next_id++;
    j->t_submit = now_s();
    s->jobs[j->id] = j;
    s->queue.push_back(j);
    *id = j->id;
  }
  s->cv.notify_all();
  return FXC_OK;
}

int fxc_server_wait(fxc_server* s, int64_t id, double timeout_s, fxc_job_info* info) {
  clear_error();
  FXC_CHECK_ARG(s && info, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  FXC_CHECK_ARG(it != s->jobs.end(), "unknown job %lld", (long long)id);
  Job* j = it->second;
  ++s->waiters;
  auto done = [&] { return j->status == 2 || j->status < 0 || s->stop; };
  bool ok = true;
  if (timeout_s > 0)
    ok = s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), done);
  else
    s->cv.wait(lk, done);
  --s->waiters;
  s->cv.notify_all();
  if (!ok || (s->stop && j->status != 2 && j->status >= 0)) {
    set_error("job %lld not finished (%s)", (long long)id, s->stop ? "server stopping" : "timeout");
    return FXC_ERR_TIMEOUT;
  }
  info->npairs = j->npairs;
  info->cc_size = j->cc_size;
  info->nspec = j->nspec;
  info->pair_windows = j->npairs * (int64_t)j->desc.ndays * j->nstep;
  info->submit_s = j->t_submit;
  info->start_s = j->t_start;
  info->end_s = j->t_end;
  info->status = j->status == 2 ? FXC_OK : j->status;
  if (j->status < 0) {
    set_error("job %lld failed: %s", (long long)id, j->error.c_str());
    return j->status;
  }
  return FXC_OK;
}

int fxc_server_fetch(fxc_server* s, int64_t id, float* h_ncf, float* h_pws) {
  clear_error();
  FXC_CHECK_ARG(s, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  FXC_CHECK_ARG(it != s->jobs.end(), "unknown job %lld", (long long)id);
  Job* j = it->second;
  FXC_CHECK_ARG(j->status == 2, "job %lld has no result", (long long)id);
  FXC_CHECK_ARG(s->cfg.keep_results, "server created without keep_results");
  if (h_ncf) memcpy(h_ncf, j->ncf.data(), j->ncf.size() * 4);
  if (h_pws) {
    FXC_CHECK_ARG(!j->pws.empty(), "job %lld has no PWS result", (long long)id);
    memcpy(h_pws, j->pws.data(), j->pws.size() * 4);
  }
  return FXC_OK;
}

int fxc_server_release(fxc_server* s, int64_t id) {
  clear_error();
  FXC_CHECK_ARG(s, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  FXC_CHECK_ARG(it != s->jobs.end(), "unknown job %lld", (long long)id);
  FXC_CHECK_ARG(it->second->status == 2 || it->second->status < 0, "job %lld still queued or running",
                (long long)id);
  delete it->second;
  s->jobs.erase(it);
  return FXC_OK;
}

int fxc_server_stats(fxc_server* s, fxc_server_stats_t* out) {
  clear_error();
  FXC_CHECK_ARG(s && out, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  out->jobs_done = s->done_jobs.load();
  out->pair_windows = s->pair_windows.load();
  out->queued = (int64_t)s->queue.size();
  out->cache_entries = (int64_t)s->entries.size();
  out->cache_used_bytes = (int64_t)s->cache.used();
  out->work_used_bytes = (int64_t)s->work.used();
  return FXC_OK;
}

int fxc_server_destroy(fxc_server* s) {
  if (!s) return FXC_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  for (std::thread& t : s->threads) t.join();
  {
    // callers blocked in fxc_server_wait return before the jobs go away
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv.notify_all();
    s->cv.wait(lk, [&] { return s->waiters == 0; });
  }
  for (fxc_ctx* c : s->ctxs) fxc_ctx_destroy(c);
  for (cudaStream_t st : s->streams) cudaStreamDestroy(st);
  for (auto& kv : s->entries) {
    if (kv.second.ready) cudaEventDestroy(kv.second.ready);
    if (kv.second.last) cudaEventDestroy(kv.second.last);
  }
  for (auto& kv : s->jobs) delete kv.second;
  s->cache.release();
  s->work.release();
  delete s;
  return FXC_OK;
}

}  // extern "C"
