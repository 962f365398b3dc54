// Shared driver of the ncf_pws and ncf_tfpws drop-ins: SourcePack groups
// in, one stacked trace per (path_id, component_slot) out, written as
// <prefix>.wNNN.{pack,tsv} shards + a merged sourcepack_index.tsv +
// _SUCCESS, as native/pws/worker/sourcepack_pipeline.cu:334-470 and
// native/tfpws/worker/pipeline.cu:200-330 do.
//
// GB300 flow: groups are dealt round-robin to the -G workers (one per list
// entry, as the reference does); each worker owns a reader thread that reads
// whole batches of groups (equal sample count and delta) into page-locked
// host memory, and a GPU thread that copies a batch once, prestacks it
// (fxc_stack_prestack), stacks every pair of the batch in one launch
// sequence (fxc_pws_run / fxc_tfpws_run), copies the stacks back and
// appends them to the worker's shard. The reader fills batch k+1 while the
// GPU thread works on batch k.
#pragma once

#include <cuda_runtime.h>
#include <getopt.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../csrc/hostio.h"
#include "../csrc/sourcepack_io.h"
#include "fastxc_gb300.h"

namespace stackapp {

using namespace fxcio;

struct Options {
  bool tfpws = false;
  const char* list = nullptr;
  const char* out = nullptr;
  const char* progress = nullptr;
  std::string gpus = "0";
  std::string mem_mib;
  int substack = 1;
  int band_limited = 0;
  double fmin = 0, fmax = 0, taper_hz = -1.0;
};

struct Item {
  SourcePackRecord rec;  // output metadata: the group's first record
  SacHeader hd;          // the first record's header
  unsigned ntrace = 0;
  size_t trace_off = 0;  // first trace of the item inside the batch
};

struct Batch {
  std::vector<Item> items;
  float* h_traces = nullptr;  // page-locked, capacity cap_floats
  size_t cap_floats = 0, ntrace = 0;
  int64_t ngroups = 0;     // substack groups of the batch (device sizing)
  int64_t max_groups = 0;  // and the most of one pair
  unsigned nsamples = 0;
  float delta = 0;
  size_t failed_groups = 0;
  bool last = false;
};

// Hand-off queue between a worker's reader and GPU threads (the batches
// circulate: free -> reader -> full -> GPU thread -> free).
class BatchQueue {
 public:
  void push(Batch* b) {
    std::unique_lock<std::mutex> lk(m_);
    q_.push_back(b);
    cv_.notify_all();
  }
  Batch* pop() {
    std::unique_lock<std::mutex> lk(m_);
    cv_.wait(lk, [&] { return !q_.empty(); });
    Batch* b = q_.front();
    q_.pop_front();
    cv_.notify_all();
    return b;
  }

 private:
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<Batch*> q_;
};

struct Shared {
  Options opt;
  std::string out_dir;
  std::mutex prog_mu;
  Progress prog;
  std::atomic<size_t> completed{0};
  std::atomic<int> failed{0};
};

inline std::vector<std::string> split_commas(const std::string& s) {
  std::vector<std::string> out;
  size_t a = 0;
  for (;;) {
    const size_t p = s.find(',', a);
    out.push_back(s.substr(a, p == std::string::npos ? std::string::npos : p - a));
    if (p == std::string::npos) break;
    a = p + 1;
  }
  return out;
}

// PWS output header (configure_output_header + update_output_stats,
// native/pws/io/sac_output.hpp:21-73).
inline void pws_header(SacHeader* hd, unsigned n, unsigned nseg, unsigned ngroups, size_t gsz,
                       const float* data) {
  hd->i[SI_NPTS] = (int)n;
  hd->i[SI_IFTYPE] = 1;
  hd->i[SI_LEVEN] = 1;
  if (hd->f[SF_DELTA] != -12345.0f) hd->f[SF_E] = hd->f[SF_B] + (float)(n - 1) * hd->f[SF_DELTA];
  hd->f[SF_USER0] = (float)nseg;
  hd->f[SF_USER1] = (float)ngroups;
  hd->f[SF_USER2] = (float)gsz;
  auto setk = [](char* dst, const char* s) {
    memset(dst, ' ', 8);
    memcpy(dst, s, std::min<size_t>(8, strlen(s)));
  };
  setk(hd->kuser[0], "NTRACE");
  setk(hd->kuser[1], "NGROUP");
  setk(hd->kuser[2], "SUBSTK");
  hd->i[SI_NZYEAR] = 2010;
  hd->i[SI_NZJDAY] = 214;
  hd->i[SI_NZHOUR] = hd->i[SI_NZMIN] = hd->i[SI_NZSEC] = hd->i[SI_NZMSEC] = 0;
  if (n == 0) return;
  float mn = data[0], mx = data[0];
  double sum = 0.0;
  for (unsigned i = 0; i < n; ++i) {
    mn = std::min(mn, data[i]);
    mx = std::max(mx, data[i]);
    sum += data[i];
  }
  hd->f[1] = mn;   // depmin
  hd->f[2] = mx;   // depmax
  hd->f[56] = (float)(sum / (double)n);  // depmen
}

// TF-PWS output header (configure_tfpws_output_header,
// native/tfpws/include/tfpws_sac.hpp:9-21).
inline void tfpws_header(SacHeader* hd, unsigned n, unsigned nseg) {
  hd->i[SI_NPTS] = (int)n;
  hd->i[SI_IFTYPE] = 1;
  hd->f[SF_USER0] = (float)nseg;
  hd->i[SI_NZYEAR] = 2010;
  hd->i[SI_NZJDAY] = 214;
  hd->i[SI_NZHOUR] = hd->i[SI_NZMIN] = hd->i[SI_NZMSEC] = 0;
}

class Worker {
 public:
  // budget_bytes: host staging of one batch; device_budget: device bytes one
  // batch may take (fxc_stack_batch_bytes), 0 = no limit
  Worker(Shared* sh, size_t index, int gpu, size_t budget_bytes, int64_t device_budget)
      : sh_(sh), index_(index), gpu_(gpu), budget_(budget_bytes), device_budget_(device_budget) {}

  std::vector<std::vector<SourcePackRecord>> groups;  // dealt round-robin, in order

  void start() {
    alloc_batches();
    reader_ = std::thread([this] { read_loop(); });
    gpu_thread_ = std::thread([this] { gpu_loop(); });
  }
  void join() {
    reader_.join();
    gpu_thread_.join();
    for (Batch* b : all_) {
      fxc_host_free(b->h_traces);
      delete b;
    }
    all_.clear();
  }
  bool ok() const { return ok_; }

 private:
  Shared* sh_;
  size_t index_;
  int gpu_;
  size_t budget_;
  int64_t device_budget_ = 0;
  bool ok_ = true;
  BatchQueue q_;
  std::thread reader_, gpu_thread_;
  PackFileCache cache_;

  static constexpr int kBatches = 3;  // one being read, one queued, one on the GPU
  BatchQueue free_;
  std::vector<Batch*> all_;

  void alloc_batches() {
    for (int i = 0; i < kBatches; ++i) {
      Batch* b = new Batch();
      b->cap_floats = budget_ / sizeof(float);
      if (fxc_host_alloc(b->cap_floats * sizeof(float), (void**)&b->h_traces) != FXC_OK) {
        FXLOG_ERROR("host_staging_alloc_failed", "worker=%zu bytes=%zu error=\"%s\"", index_,
                    b->cap_floats * sizeof(float), fxc_last_error());
        b->h_traces = nullptr;
        b->cap_floats = 0;
      }
      all_.push_back(b);
      free_.push(b);
    }
  }
  static void reset(Batch* b) {
    b->items.clear();
    b->ntrace = 0;
    b->ngroups = 0;
    b->max_groups = 0;
    b->nsamples = 0;
    b->delta = 0;
    b->failed_groups = 0;
    b->last = false;
  }
  Batch* new_batch() {
    Batch* b = free_.pop();
    reset(b);
    return b;
  }

  // Reads one group into the batch; false (and nothing added) on failure.
  bool read_group(const std::vector<SourcePackRecord>& g, Batch* b, unsigned ns) {
    Item it;
    it.rec = g[0];
    if (read_sourcepack_header(&cache_, g[0], &it.hd) != 0) return false;
    it.ntrace = (unsigned)g.size();
    it.trace_off = b->ntrace;
    for (size_t i = 0; i < g.size(); ++i) {
      SacHeader hd;
      if (read_sourcepack_record(&cache_, g[i], &hd, b->h_traces + (b->ntrace + i) * ns, ns) != 0)
        return false;
    }
    b->ntrace += g.size();
    b->items.push_back(it);
    return true;
  }

  void read_loop() {
    Batch* b = new_batch();
    for (size_t k = 0; k < groups.size(); ++k) {
      const std::vector<SourcePackRecord>& g = groups[k];
      SacHeader h0;
      if (!b->h_traces || read_sourcepack_header(&cache_, g[0], &h0) != 0) {
        ++b->failed_groups;
        continue;
      }
      const unsigned ns = sac_data_count(h0);
      const float delta = h0.f[SF_DELTA];
      const size_t need = g.size() * (size_t)ns;
      if (ns == 0 || need > b->cap_floats) {
        FXLOG_ERROR("stack_group_too_large", "path_id=\"%s\" component_slot=%d traces=%zu samples=%u",
                    g[0].path_id.c_str(), g[0].component_slot, g.size(), ns);
        ++b->failed_groups;
        continue;
      }
      const int64_t sub = sh_->opt.substack >= 2 ? sh_->opt.substack : 1;
      const int64_t g_groups = ((int64_t)g.size() + sub - 1) / sub;
      if (device_budget_ > 0) {
        int64_t one = 0;
        fxc_stack_batch_bytes(sh_->opt.tfpws ? 1 : 0, (int64_t)g.size(), 1, g_groups, g_groups, (int32_t)ns, &one);
        if (one > device_budget_) {
          FXLOG_ERROR("stack_group_above_memory_budget", "path_id=\"%s\" component_slot=%d traces=%zu samples=%u "
                      "bytes=%lld budget=%lld", g[0].path_id.c_str(), g[0].component_slot, g.size(), ns,
                      (long long)one, (long long)device_budget_);
          ++b->failed_groups;
          continue;
        }
      }
      auto device_fits = [&]() {
        if (device_budget_ <= 0) return true;
        int64_t bytes = 0;
        fxc_stack_batch_bytes(sh_->opt.tfpws ? 1 : 0, (int64_t)(b->ntrace + g.size()), (int32_t)b->items.size() + 1,
                              b->ngroups + g_groups, std::max(b->max_groups, g_groups), (int32_t)ns, &bytes);
        return bytes <= device_budget_;
      };
      const bool fits = b->items.empty() ||
                        (b->nsamples == ns && b->delta == delta && (b->ntrace * (size_t)ns + need) <= b->cap_floats &&
                         b->items.size() < 8192 && device_fits());
      if (!fits) {
        q_.push(b);
        b = new_batch();
        if (!b->h_traces) {
          ++b->failed_groups;
          continue;
        }
      }
      if (b->items.empty()) {
        b->nsamples = ns;
        b->delta = delta;
      }
      if (!read_group(g, b, ns)) {
        FXLOG_ERROR("stack_group_read_failed", "worker=%zu path_id=\"%s\" component_slot=%d", index_,
                    g[0].path_id.c_str(), g[0].component_slot);
        ++b->failed_groups;
      } else {
        b->ngroups += g_groups;
        b->max_groups = std::max(b->max_groups, g_groups);
      }
    }
    b->last = true;
    q_.push(b);
  }

  void gpu_loop() {
    fxc_ctx* ctx = nullptr;
    StackShardWriter writer;
    const std::string prefix = sh_->opt.tfpws ? "tfpws" : "pws";
    if (writer.open(sh_->out_dir, prefix, index_) != 0) ok_ = false;
    if (ok_ && fxc_ctx_create(gpu_, nullptr, &ctx) != FXC_OK) {
      FXLOG_ERROR("gpu_context_failed", "worker=%zu gpu=%d error=\"%s\"", index_, gpu_, fxc_last_error());
      ok_ = false;
    }
    void* d_buf = nullptr;
    size_t d_cap = 0;
    std::vector<float> h_out;
    for (;;) {
      Batch* b = q_.pop();
      const bool last = b->last;
      sh_->failed += (int)b->failed_groups;
      if (ok_ && !b->items.empty()) {
        if (run_batch(ctx, b, &d_buf, &d_cap, &h_out, &writer) != 0) {
          sh_->failed += (int)b->items.size();
          ok_ = false;
        }
      } else if (!ok_) {
        sh_->failed += (int)b->items.size();
      }
      if (last) break;
      free_.push(b);
    }
    if (ctx) {
      fxc_device_free(ctx, d_buf);
      fxc_ctx_destroy(ctx);
    }
    if (writer.close() != 0) ok_ = false;
  }

  int run_batch(fxc_ctx* ctx, Batch* b, void** d_buf, size_t* d_cap, std::vector<float>* h_out,
                StackShardWriter* writer) {
    const Options& o = sh_->opt;
    const int32_t np = (int32_t)b->items.size();
    const int32_t ns = (int32_t)b->nsamples;
    const size_t tr_bytes = b->ntrace * (size_t)ns * 4;
    const size_t pair_bytes = (size_t)np * ns * 4;
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    // traces | groups (<= traces) | weights (<= traces) | linear | out
    const size_t o_g = al(tr_bytes), o_w = o_g + al(tr_bytes), o_l = o_w + al(b->ntrace * 4);
    const size_t o_o = o_l + al(pair_bytes), total = o_o + al(pair_bytes);
    if (total > *d_cap) {
      fxc_device_free(ctx, *d_buf);
      *d_buf = nullptr;
      *d_cap = 0;
      if (fxc_device_alloc(ctx, total, d_buf) != FXC_OK) {
        FXLOG_ERROR("stack_device_alloc_failed", "bytes=%zu error=\"%s\"", total, fxc_last_error());
        return 1;
      }
      *d_cap = total;
    }
    char* base = (char*)*d_buf;
    float* d_tr = (float*)base;
    float* d_g = (float*)(base + o_g);
    float* d_w = (float*)(base + o_w);
    float* d_l = (float*)(base + o_l);
    float* d_o = (float*)(base + o_o);
    std::vector<int64_t> toff(np), goff(np);
    std::vector<int32_t> tcnt(np), gcnt(np);
    for (int32_t p = 0; p < np; ++p) {
      toff[p] = (int64_t)b->items[p].trace_off;
      tcnt[p] = (int32_t)b->items[p].ntrace;
    }
    int rc = fxc_memcpy(ctx, d_tr, b->h_traces, tr_bytes, FXC_COPY_H2D);
    if (rc == FXC_OK)
      rc = fxc_stack_prestack(ctx, d_tr, toff.data(), tcnt.data(), np, ns, o.substack, o.tfpws ? 1 : 0, d_g,
                              d_w, d_l, goff.data(), gcnt.data());
    if (rc == FXC_OK) {
      if (o.tfpws)
        rc = fxc_tfpws_run(ctx, d_g, d_w, goff.data(), gcnt.data(), np, d_l, ns, b->delta, o.band_limited,
                           (float)o.fmin, (float)o.fmax, (float)o.taper_hz, 1.0f, d_o);
      else
        rc = fxc_pws_run(ctx, d_g, d_w, goff.data(), gcnt.data(), np, d_l, ns, 1.0f, d_o);
    }
    h_out->resize((size_t)np * ns);
    if (rc == FXC_OK) rc = fxc_memcpy(ctx, h_out->data(), d_o, pair_bytes, FXC_COPY_D2H);
    if (rc == FXC_OK) rc = fxc_ctx_synchronize(ctx);
    if (rc != FXC_OK) {
      FXLOG_ERROR("stack_batch_compute_failed", "worker=%zu gpu=%d pairs=%d error=\"%s\"", index_, gpu_, np,
                  fxc_last_error());
      return 1;
    }
    const size_t gsz = o.substack < 2 ? 1 : (size_t)o.substack;
    for (int32_t p = 0; p < np; ++p) {
      Item& it = b->items[p];
      const float* tr = h_out->data() + (size_t)p * ns;
      if (o.tfpws)
        tfpws_header(&it.hd, (unsigned)ns, it.ntrace);
      else
        pws_header(&it.hd, (unsigned)ns, it.ntrace, (unsigned)gcnt[p], gsz, tr);
      if (writer->append(it.rec, it.hd, tr) != 0) {
        ++sh_->failed;
        continue;
      }
      const size_t done = ++sh_->completed;
      std::lock_guard<std::mutex> lk(sh_->prog_mu);
      const std::string detail = "worker=" + std::to_string(index_) + " gpu=" + std::to_string(gpu_) + " " +
                                 it.rec.path_id + ":" + it.rec.src_component + "-" + it.rec.rec_component;
      sh_->prog.update(done, done >= sh_->prog.total ? "DONE" : "RUNNING", detail.c_str());
    }
    return 0;
  }
};

inline int run(const Options& opt) {
  std::vector<std::string> indexes;
  if (read_sourcepack_list(opt.list, &indexes) != 0) return 1;
  const std::vector<std::string> gl = split_commas(opt.gpus);
  std::vector<int> gpus;
  for (const std::string& g : gl) {
    if (g.empty()) {
      FXLOG_ERROR("invalid_gpu_workers", "value=\"%s\"", opt.gpus.c_str());
      return 1;
    }
    gpus.push_back(atoi(g.c_str()));
  }
  std::vector<size_t> mib(gpus.size(), 0);
  if (!opt.mem_mib.empty()) {
    const std::vector<std::string> ml = split_commas(opt.mem_mib);
    if (ml.size() != gpus.size()) {
      FXLOG_ERROR("gpu_memory_list_mismatch", "workers=%zu memory_entries=%zu", gpus.size(), ml.size());
      return 1;
    }
    for (size_t i = 0; i < ml.size(); ++i) mib[i] = (size_t)strtoull(ml[i].c_str(), nullptr, 10);
  }
  Shared sh;
  sh.opt = opt;
  sh.out_dir = absolute_path(opt.out);
  const std::string prefix = opt.tfpws ? "tfpws" : "pws";
  const std::string index_path = join_path(sh.out_dir, "sourcepack_index.tsv");
  const size_t total_groups = count_sourcepack_groups(indexes);
  sh.prog.init(opt.progress, "overall", total_groups, "groups");
  SourcePackGroupReader reader(indexes);
  if (reader.open() != 0) {
    sh.prog.update(0, "FAILED");
    return 1;
  }
  std::vector<Worker*> workers;
  for (size_t i = 0; i < gpus.size(); ++i) {
    // host staging per batch (3 batches circulate per worker): a quarter of
    // the -M cap when given, else 2 GiB. Device bytes per batch
    // (fxc_stack_batch_bytes): the -M cap when given, else 0.9 x the GPU's
    // free memory at start (the reference's resident-chunk budget,
    // native/tfpws/include/tfpws_schedule.hpp:149-217, over this library's
    // buffers).
    const size_t budget = mib[i] ? std::max<size_t>(mib[i] << 20, 64u << 20) / 4 : (size_t)2 << 30;
    int64_t dev_budget = mib[i] ? (int64_t)(mib[i] << 20) : 0;
    if (!dev_budget) {
      size_t free_b = 0, total_b = 0;
      if (cudaSetDevice(gpus[i]) == cudaSuccess && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
        dev_budget = (int64_t)((double)free_b * 0.9);
    }
    workers.push_back(new Worker(&sh, i, gpus[i], budget, dev_budget));
  }
  std::vector<SourcePackRecord> g;
  size_t cursor = 0;
  while (reader.next_group(&g)) workers[cursor++ % workers.size()]->groups.push_back(g);
  FXLOG_INFO("stack_jobs_enqueued", "jobs=%zu workers=%zu", cursor, workers.size());
  for (Worker* w : workers) w->start();
  bool ok = true;
  for (Worker* w : workers) {
    w->join();
    ok = ok && w->ok();
  }
  for (Worker* w : workers) delete w;
  if (!ok || sh.failed.load() != 0) {
    FXLOG_ERROR("stack_pipeline_failed", "failed=%d completed=%zu", sh.failed.load(), sh.completed.load());
    sh.prog.update(sh.completed.load(), "FAILED");
    return 1;
  }
  if (merge_shard_indexes(sh.out_dir, prefix, gpus.size(), index_path) != 0 ||
      write_stack_success(sh.out_dir, prefix, sh.completed.load(), gpus.size(), index_path) != 0) {
    sh.prog.update(sh.completed.load(), "FAILED");
    return 1;
  }
  FXLOG_INFO("stack_pipeline_done", "completed=%zu workers=%zu output_dir=\"%s\"", sh.completed.load(),
             gpus.size(), sh.out_dir.c_str());
  sh.prog.update(total_groups, "DONE");
  return 0;
}

}  // namespace stackapp
