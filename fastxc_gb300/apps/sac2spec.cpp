// sac2spec drop-in: SAC index -> preprocessed, normalised, whitened output
// spectra written as stepack batches.
//
// Command line of the reference (native/sac2spec/arguproc.c:233-469):
//   sac2spec -I <sac_index.tsv> -O <output_root> -L sac_len/win_len/shift_len/xcorr_lag
//            -B <filter.txt> [-C num_ch] [-G gpu list] [-T io threads] [-M MiB list]
//            [-W whiten/phase_only] [-N|--normalize type] [-Q skip,steps,-1] [--debug] [-h]
// Output (native/sac2spec/output_layout.cu, io/stepack_writer.c,
// timestamp_tracker.cu, progress.cu): <root>/stepack/wWWW.bBBBBBB.{stepack,tsv},
// <root>/stepack/<timestamp>/_SUCCESS per finished timestamp,
// <root>/stepack/_SUCCESS, <root>/progress/sac2spec_progress.tsv; exit 0 / 1.
//
// GB300 flow: groups of num_ch rows are cut into batches sized for device
// memory; every -G entry is a worker with a reader thread (SAC files into
// page-locked host memory with -T threads) and a GPU thread (one copy in,
// fxc_s2s_run over all valid windows of every row, one copy out, stepack
// write), so reading batch k+1 overlaps the GPU work on batch k.
#include <dirent.h>
#include <errno.h>
#include <math.h>
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
#include "../csrc/sac2spec_io.h"
#include "fastxc_gb300.h"

using namespace fxcio;

namespace {

struct Args {
  const char* input = nullptr;
  const char* out = nullptr;
  const char* filter = nullptr;
  int num_ch = 3, threads = 1, whiten = 0, phase_only = 0, normalize = 0;
  float sac_len = 0, win_len = 0, shift_len = 0, lag = 0;
  bool have_l = false;
  std::vector<int> gpus{0};
  std::vector<double> mem_mib;
  std::vector<int> skip;
};

void usage() {
  fprintf(stderr,
          "Usage:  sac2spec  -I <input_list> -O <output_root> -L <file/window/shift/ncf_lag> [options]\n"
          "\n"
          "  -I FILE     input SAC index TSV (timestamp nsl_id network station location component sac_path)\n"
          "  -O DIR      output workspace; creates DIR/stepack and DIR/progress\n"
          "  -L A/B/C/D  SAC file length, segment window, segment shift and NCF lag in seconds\n"
          "  -B FILE     Butterworth filter-coefficient file; first band is the broad band\n"
          "  -C INT      channels per NSL/timestamp group (default: 3)\n"
          "  -G LIST     comma-separated GPU ids of the workers, e.g. 0 or 0,0\n"
          "  -T INT      CPU I/O threads across workers (default: 1)\n"
          "  -M LIST     comma-separated MiB caps matching -G; 0 means auto\n"
          "  -W A/B      whitening 0 none, 1 before, 2 after, 3 both / output phase-only 0 or 1\n"
          "  -N INT      time normalisation 0 none, 1 multi-band run-abs, 2 one-bit, 3 run-abs\n"
          "  --normalize INT  alias of -N\n"
          "  -Q LIST     comma-separated window indices to skip, terminated by -1\n"
          "  --debug     accepted for compatibility\n"
          "  -h          show this help and exit\n");
}

[[noreturn]] void fail_usage(const char* msg = nullptr) {
  if (msg) fprintf(stderr, "%s\n", msg);
  usage();
  exit(1);
}

bool parse_int(const char* s, int* out) {
  char* e = nullptr;
  errno = 0;
  const long v = strtol(s, &e, 10);
  if (errno || e == s || *e || v < -2147483647L || v > 2147483647L) return false;
  *out = (int)v;
  return true;
}

bool parse_float(const char* s, float* out) {
  char* e = nullptr;
  errno = 0;
  const float v = strtof(s, &e);
  if (errno || e == s || *e) return false;
  *out = v;
  return true;
}

std::vector<std::string> split(const char* s, char sep) {
  std::vector<std::string> out;
  std::string cur;
  for (const char* p = s; *p; ++p) {
    if (*p == sep) {
      if (!cur.empty()) out.push_back(cur);  // strtok semantics: empty tokens vanish
      cur.clear();
    } else {
      cur.push_back(*p);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

Args parse_args(int argc, char** argv) {
  Args a;
  if (argc < 2) fail_usage();
  for (int i = 1; i < argc; ++i) {
    const char* o = argv[i];
    auto value = [&](const char* name) -> const char* {
      if (i + 1 >= argc) {
        fprintf(stderr, "Error: %s requires a value\n", name);
        fail_usage();
      }
      return argv[++i];
    };
    if (!strcmp(o, "-h") || !strcmp(o, "--help")) {
      usage();
      exit(0);
    }
    if (!strncmp(o, "--", 2)) {
      if (!strcmp(o, "--normalize") || !strcmp(o, "--normalize-type")) {
        a.normalize = atoi(value(o));
      } else if (!strcmp(o, "--debug")) {
      } else {
        fprintf(stderr, "Error: Unknown option %s\n", o);
        fail_usage();
      }
      continue;
    }
    if (o[0] != '-' || o[1] == '\0' || o[2] != '\0') {
      fprintf(stderr, "Error: Invalid option %s\n", o);
      fail_usage();
    }
    char name[3] = {'-', o[1], 0};
    switch (o[1]) {
      case 'I': a.input = value(name); break;
      case 'O': a.out = value(name); break;
      case 'C': a.num_ch = atoi(value(name)); break;
      case 'B': a.filter = value(name); break;
      case 'L': {
        const std::vector<std::string> t = split(value(name), '/');
        if (t.size() != 4 || !parse_float(t[0].c_str(), &a.sac_len) || !parse_float(t[1].c_str(), &a.win_len) ||
            !parse_float(t[2].c_str(), &a.shift_len) || !parse_float(t[3].c_str(), &a.lag)) {
          fprintf(stderr, "Error: -L expects sac_len/win_len/shift_len/xcorr_lag, e.g. 86400/7200/7200/100\n");
          exit(1);
        }
        a.have_l = true;
        break;
      }
      case 'G': {
        a.gpus.clear();
        for (const std::string& t : split(value(name), ',')) {
          int g = -1;
          if (!parse_int(t.c_str(), &g) || g < 0) {
            fprintf(stderr, "Error: Invalid GPU id %s\n", t.c_str());
            exit(1);
          }
          a.gpus.push_back(g);
        }
        if (a.gpus.empty()) {
          fprintf(stderr, "Error: -G requires at least one GPU id\n");
          exit(1);
        }
        break;
      }
      case 'W': {
        const std::vector<std::string> t = split(value(name), '/');
        if (t.size() != 2 || !parse_int(t[0].c_str(), &a.whiten) || !parse_int(t[1].c_str(), &a.phase_only)) {
          fprintf(stderr, "Error: -W expects whiten_type/output_phase_only, e.g. 2/1\n");
          exit(1);
        }
        break;
      }
      case 'N': a.normalize = atoi(value(name)); break;
      case 'Q': {
        a.skip.clear();
        for (const std::string& t : split(value(name), ',')) {
          int v = 0;
          if (!parse_int(t.c_str(), &v)) {
            fprintf(stderr, "Error: Invalid skip step %s\n", t.c_str());
            exit(1);
          }
          if (v == -1) break;
          if (v < 0) {
            fprintf(stderr, "Error: Skip steps must be >= 0, or -1 as terminator\n");
            exit(1);
          }
          a.skip.push_back(v);
        }
        break;
      }
      case 'T': a.threads = atoi(value(name)); break;
      case 'M': {
        a.mem_mib.clear();
        for (const std::string& t : split(value(name), ',')) {
          char* e = nullptr;
          const double v = strtod(t.c_str(), &e);
          if (e == t.c_str() || *e || v < 0.0) {
            fprintf(stderr, "Error: Invalid GPU memory limit %s\n", t.c_str());
            exit(1);
          }
          a.mem_mib.push_back(v);
        }
        if (a.mem_mib.empty()) {
          fprintf(stderr, "Error: -M requires at least one memory limit\n");
          exit(1);
        }
        break;
      }
      default:
        fprintf(stderr, "Error: Unknown option -%c\n", o[1]);
        fail_usage();
    }
  }
  if (!a.input || !a.out || !a.filter || !a.have_l || a.win_len <= 0.0f) {
    if (!a.have_l) fprintf(stderr, "Error: -L sac_len/win_len/shift_len/xcorr_lag is required\n");
    fail_usage();
  }
  if (a.shift_len <= 0.0f) fail_usage("Error: -L shift_len must be > 0");
  if (a.sac_len <= 0.0f) fail_usage("Error: -L sac_len must be > 0");
  if (a.num_ch < 1) fail_usage("Error: -C must be >= 1");
  if (a.threads < 1) fail_usage("Error: -T must be >= 1");
  if (!a.mem_mib.empty() && a.mem_mib.size() != a.gpus.size()) {
    fprintf(stderr, "Error: -M count must match -G count; got %zu memory limits for %zu virtual GPU workers\n",
            a.mem_mib.size(), a.gpus.size());
    exit(1);
  }
  if (a.lag < 0.0f) fail_usage("Error: -L xcorr_lag must be >= 0");
  if (a.whiten < 0 || a.whiten > 3) fail_usage("Error: -W whiten_type must be 0, 1, 2, or 3");
  if (a.phase_only != 0 && a.phase_only != 1) fail_usage("Error: -W output_phase_only must be 0 or 1");
  return a;
}

// Shared run state.
struct Run {
  Args args;
  std::string stepack_root;
  std::vector<SacIndexRow> rows;
  fxc_s2s_plan plan;
  std::vector<float> responses;  // [nfilters][filter_nfft/2+1]
  std::vector<int32_t> steps;    // valid window indices
  float df_out = 0;
  size_t groups = 0, groups_per_batch = 1;
  std::atomic<size_t> next_batch{0};
  std::atomic<int> failed{0};
  S2sProgress progress;
  TimestampTracker tracker;
};

struct Batch {
  size_t start_group = 0, group_count = 0, seq = 0;
  float* h_series = nullptr;  // [rows][npts]
  float* h_out = nullptr;     // [nsteps][rows][nspec] complex
  std::vector<Channel> chans;
  bool ok = true, last = false;
};

class Queue {
 public:
  void push(Batch* b) {
    std::lock_guard<std::mutex> lk(m_);
    q_.push_back(b);
    cv_.notify_all();
  }
  Batch* pop() {
    std::unique_lock<std::mutex> lk(m_);
    cv_.wait(lk, [&] { return !q_.empty(); });
    Batch* b = q_.front();
    q_.pop_front();
    return b;
  }

 private:
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<Batch*> q_;
};

class Worker {
 public:
  Worker(Run* run, int index, int gpu, int io_threads) : r_(run), index_(index), gpu_(gpu), io_(io_threads) {}
  bool ok = true;

  void start() {
    reader_ = std::thread([this] { read_loop(); });
    gthread_ = std::thread([this] { gpu_loop(); });
  }
  void join() {
    reader_.join();
    gthread_.join();
    for (Batch& b : slots_) {
      fxc_host_free(b.h_series);
      fxc_host_free(b.h_out);
    }
  }
  bool alloc(size_t rows_cap) {
    const size_t npts = (size_t)r_->plan.npts;
    const size_t out = r_->steps.size() * rows_cap * (size_t)r_->plan.nspec * 2;
    for (Batch& b : slots_) {
      if (fxc_host_alloc(rows_cap * npts * sizeof(float), (void**)&b.h_series) != FXC_OK ||
          fxc_host_alloc(out * sizeof(float), (void**)&b.h_out) != FXC_OK) {
        FXLOG_ERROR("host_staging_alloc_failed", "worker=%d error=\"%s\"", index_, fxc_last_error());
        return false;
      }
      free_.push(&b);
    }
    return true;
  }

 private:
  Run* r_;
  int index_, gpu_, io_;
  Batch slots_[2];
  Queue free_, full_;
  std::thread reader_, gthread_;
  size_t seq_ = 0;

  bool read_rows(Batch* b) {
    const int nch = r_->args.num_ch;
    const size_t row0 = b->start_group * nch, nrows = b->group_count * nch;
    const int npts = r_->plan.npts;
    b->chans.assign(nrows, Channel());
    std::atomic<size_t> next{0};
    std::atomic<bool> ok{true};
    auto work = [&]() {
      for (size_t i; (i = next++) < nrows && ok;) {
        const SacIndexRow& row = r_->rows[row0 + i];
        SacHeader hd;
        std::vector<float> data;
        if (sac_read(row.sac_path.c_str(), &hd, nullptr, 0) != 0) {
          FXLOG_ERROR("read_sachead_failed", "path=\"%s\"", row.sac_path.c_str());
          ok = false;
          return;
        }
        if (!sac_delta_matches(hd.f[SF_DELTA], r_->plan.delta)) {
          FXLOG_ERROR("sac_delta_mismatch", "path=\"%s\" expected=%.9g observed=%.9g", row.sac_path.c_str(),
                      r_->plan.delta, hd.f[SF_DELTA]);
          ok = false;
          return;
        }
        if (sac_read(row.sac_path.c_str(), &hd, &data, npts) != 0) {
          ok = false;
          return;
        }
        memcpy(b->h_series + i * (size_t)npts, data.data(), sizeof(float) * (size_t)npts);
        Channel& c = b->chans[i];
        c.timestamp = row.timestamp;
        c.nsl_id = row.nsl_id;
        c.nsl_text = row.nsl_text;
        c.network = row.network;
        c.station = row.station;
        c.location = row.location;
        c.component = row.component;
        c.stla = hd.f[SF_STLA];
        c.stlo = hd.f[SF_STLO];
      }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < io_; ++t) pool.emplace_back(work);
    work();
    for (std::thread& t : pool) t.join();
    return ok;
  }

  void read_loop() {
    for (;;) {
      const size_t k = r_->next_batch++;
      const size_t g0 = k * r_->groups_per_batch;
      Batch* b = free_.pop();
      if (g0 >= r_->groups || r_->failed) {
        b->last = true;
        full_.push(b);
        return;
      }
      b->start_group = g0;
      b->group_count = std::min(r_->groups_per_batch, r_->groups - g0);
      b->seq = seq_++;
      b->last = false;
      b->ok = read_rows(b);
      full_.push(b);
    }
  }

  void gpu_loop() {
    fxc_ctx* ctx = nullptr;
    void *d_series = nullptr, *d_out = nullptr, *d_resp = nullptr;
    const size_t npts = (size_t)r_->plan.npts, nspec = (size_t)r_->plan.nspec, ns = r_->steps.size();
    const size_t cap_rows = r_->groups_per_batch * (size_t)r_->args.num_ch;
    if (fxc_ctx_create(gpu_, nullptr, &ctx) != FXC_OK ||
        fxc_device_alloc(ctx, cap_rows * npts * 4, &d_series) != FXC_OK ||
        fxc_device_alloc(ctx, ns * cap_rows * nspec * 8, &d_out) != FXC_OK ||
        fxc_device_alloc(ctx, r_->responses.size() * 4, &d_resp) != FXC_OK ||
        fxc_memcpy(ctx, d_resp, r_->responses.data(), r_->responses.size() * 4, FXC_COPY_H2D) != FXC_OK) {
      FXLOG_ERROR("gpu_worker_init_failed", "worker=%d gpu=%d error=\"%s\"", index_, gpu_, fxc_last_error());
      ok = false;
      r_->failed = 1;
    }
    for (;;) {
      Batch* b = full_.pop();
      if (b->last) break;
      if (ok && !b->ok) {
        ok = false;
        r_->failed = 1;
      }
      if (ok) {
        const int32_t nrows = (int32_t)(b->group_count * r_->args.num_ch);
        int rc = fxc_memcpy(ctx, d_series, b->h_series, (size_t)nrows * npts * 4, FXC_COPY_H2D);
        if (rc == FXC_OK)
          rc = fxc_s2s_run(ctx, &r_->plan, (const float*)d_series, (int64_t)npts, (int64_t)npts, nrows,
                           r_->args.num_ch, r_->steps.data(), (int32_t)ns, (const float*)d_resp, (float*)d_out,
                           (int64_t)nspec);
        if (rc == FXC_OK) rc = fxc_memcpy(ctx, b->h_out, d_out, ns * nrows * nspec * 8, FXC_COPY_D2H);
        if (rc == FXC_OK) rc = fxc_ctx_synchronize(ctx);
        if (rc != FXC_OK) {
          FXLOG_ERROR("worker_batch_compute_failed", "gpu=%d start_group=%zu count=%zu error=\"%s\"", gpu_,
                      b->start_group, b->group_count, fxc_last_error());
          ok = false;
          r_->failed = 1;
        } else if (stepack_write_batch(r_->stepack_root, index_, b->seq, b->start_group, b->group_count, b->chans,
                                       (int)ns, (int)nspec, r_->plan.delta, r_->df_out, b->h_out) != 0 ||
                   r_->tracker.mark_done(b->start_group, b->group_count) != 0) {
          FXLOG_ERROR("worker_output_write_failed", "gpu=%d start_group=%zu count=%zu", gpu_, b->start_group,
                      b->group_count);
          ok = false;
          r_->failed = 1;
        } else {
          r_->progress.add((size_t)nrows, gpu_, b->start_group, b->group_count);
        }
      }
      free_.push(b);
    }
    if (ctx) {
      fxc_device_free(ctx, d_series);
      fxc_device_free(ctx, d_out);
      fxc_device_free(ctx, d_resp);
      fxc_ctx_destroy(ctx);
    }
  }
};

bool dir_empty(const std::string& path) {
  DIR* d = opendir(path.c_str());
  if (!d) {
    FXLOG_ERROR("open_stepack_dir_failed", "path=\"%s\"", path.c_str());
    return false;
  }
  bool empty = true;
  while (dirent* e = readdir(d)) {
    if (!strcmp(e->d_name, ".") || !strcmp(e->d_name, "..")) continue;
    FXLOG_ERROR("stepack_dir_not_empty", "path=\"%s\" entry=\"%s\" action=clean_or_choose_new_output",
                path.c_str(), e->d_name);
    empty = false;
    break;
  }
  closedir(d);
  return empty;
}

}  // namespace

int main(int argc, char** argv) {
  Run run;
  run.args = parse_args(argc, argv);
  const Args& a = run.args;
  const std::string root = a.out;
  run.stepack_root = root + (root.empty() || root.back() == '/' ? "" : "/") + "stepack";
  const std::string prog_dir = root + (root.empty() || root.back() == '/' ? "" : "/") + "progress";
  if (mkdir_p(run.stepack_root) != 0 || mkdir_p(prog_dir) != 0) {
    FXLOG_ERROR("create_output_dirs_failed", "output_root=\"%s\"", root.c_str());
    return 1;
  }
  if (!dir_empty(run.stepack_root)) return 1;
  if (read_sac_index(a.input, a.num_ch, &run.rows) != 0) return 1;
  if (run.rows.size() % (size_t)a.num_ch != 0) {
    FXLOG_ERROR("sac_index_component_count_invalid", "component_count=%zu num_ch=%d", run.rows.size(), a.num_ch);
    return 1;
  }
  if (a.normalize < 0 || a.normalize > 3) {
    FXLOG_ERROR("invalid_normalize_type", "value=%d", a.normalize);
    return 1;
  }
  run.groups = run.rows.size() / (size_t)a.num_ch;
  SacHeader h0;
  if (sac_read(run.rows[0].sac_path.c_str(), &h0, nullptr, 0) != 0) {
    FXLOG_ERROR("read_first_sachead_failed", "path=\"%s\"", run.rows[0].sac_path.c_str());
    return 1;
  }
  const float delta = h0.f[SF_DELTA];
  if (!(delta > 0.0f)) {
    FXLOG_ERROR("invalid_first_sac_delta", "path=\"%s\" delta=%.9g", run.rows[0].sac_path.c_str(), delta);
    return 1;
  }
  FilterSet flt;
  if (read_filter_file(a.filter, &flt) != 0 || flt.count() <= 0) {
    FXLOG_ERROR("filter_file_empty", "path=\"%s\" filter_count=%d", a.filter, flt.count());
    return 1;
  }
  if (flt.freq_low[0] <= 0.0f || flt.freq_high[0] <= flt.freq_low[0]) {
    FXLOG_ERROR("filter_broad_band_invalid", "path=\"%s\" freq_low=%.8g freq_high=%.8g", a.filter,
                flt.freq_low[0], flt.freq_high[0]);
    return 1;
  }
  if (fxc_s2s_plan_init(a.sac_len, a.win_len, a.shift_len, a.lag, delta, flt.b.data(), flt.a.data(),
                        flt.freq_low.data(), flt.freq_high.data(), flt.count(), a.whiten, a.normalize,
                        a.phase_only, &run.plan) != FXC_OK) {
    FXLOG_ERROR("plan_failed", "error=\"%s\"", fxc_last_error());
    return 1;
  }
  run.responses.resize((size_t)flt.count() * (size_t)(run.plan.filter_nfft / 2 + 1));
  if (fxc_s2s_filter_response(&run.plan, flt.b.data(), flt.a.data(), flt.count(), run.responses.data()) != FXC_OK) {
    FXLOG_ERROR("filter_response_build_failed", "error=\"%s\"", fxc_last_error());
    return 1;
  }
  run.df_out = 1.0f / ((float)run.plan.output_nfft * delta);
  std::vector<char> skipped((size_t)run.plan.nstep, 0);
  for (int s : a.skip) {
    if (s >= 0 && s < run.plan.nstep)
      skipped[s] = 1;
    else
      FXLOG_WARN("segment_step_skip_out_of_range", "step=%d nstep=%d ignored=1", s, run.plan.nstep);
  }
  for (int i = 0; i < run.plan.nstep; ++i)
    if (!skipped[i]) run.steps.push_back(i);
  if (run.steps.empty()) {
    FXLOG_ERROR("no_valid_segment_steps", "nstep=%d skip_count=%zu", run.plan.nstep, a.skip.size());
    return 1;
  }
  // batch size: series + output + the row workspace of fxc_s2s_run (about
  // 5 floats per sample per window, more with multi-band RAM) within the
  // -M cap (x0.7) or 16 GiB
  const size_t nb = run.plan.normalize == 1 ? (size_t)run.plan.nfilters - 1 : 0;
  const size_t per_row = (size_t)run.plan.npts * 4 +
                         run.steps.size() * ((size_t)run.plan.nspec * 8 +
                                             (size_t)run.plan.segment_pts * (14 + 8 * nb));
  double cap_mib = 0;
  for (double m : a.mem_mib) cap_mib = cap_mib == 0 ? m : std::min(cap_mib, m);
  const size_t budget = cap_mib > 0 ? (size_t)(cap_mib * 0.7 * 1048576.0) : ((size_t)16 << 30);
  run.groups_per_batch = std::max<size_t>(1, std::min(run.groups, budget / (per_row * (size_t)a.num_ch)));
  run.progress.init(prog_dir + "/sac2spec_progress.tsv", run.rows.size());
  if (run.tracker.init(run.rows, a.num_ch, run.stepack_root) != 0) {
    run.progress.finish("FAILED", false);
    return 1;
  }
  FXLOG_INFO("sac2spec_plan", "rows=%zu groups=%zu groups_per_batch=%zu npts=%d seg=%d nstep_valid=%zu nspec=%d",
             run.rows.size(), run.groups, run.groups_per_batch, run.plan.npts, run.plan.segment_pts,
             run.steps.size(), run.plan.nspec);
  std::vector<Worker*> workers;
  const int nw = (int)a.gpus.size();
  for (int i = 0; i < nw; ++i) {
    Worker* w = new Worker(&run, i, a.gpus[i], std::max(1, a.threads / nw));
    if (!w->alloc(run.groups_per_batch * (size_t)a.num_ch)) run.failed = 1;
    workers.push_back(w);
  }
  for (Worker* w : workers) w->start();
  for (Worker* w : workers) {
    w->join();
    if (!w->ok) run.failed = 1;
    delete w;
  }
  if (!run.failed) {
    const std::string p = run.stepack_root + "/_SUCCESS";
    FILE* fp = fopen(p.c_str(), "wb");
    if (!fp || fprintf(fp, "DONE\n") < 0 || fclose(fp) != 0) run.failed = 1;
  }
  if (run.failed) {
    run.progress.finish("FAILED", false);
    FXLOG_ERROR("gpu_worker_failed", "workers=%d", nw);
    return 1;
  }
  run.progress.finish("DONE", true);
  return 0;
}
