// xc_linear: stepack spectra of many timestamps -> one cross-timestamp
// linear stack per (path, component) group -> the linearstack SourcePack.
//
// Replaces the chain
//   xc_fast (one xcpack NCF per pair and timestamp)
//   -> build_sourcepack (fastxc/operators/sourcepack/builder.py:163-245)
//   -> linear_stack_sourcepack_indexes
//      (fastxc/operators/stacking/linear_stack.py:312-391)
// with one pass: every timestamp's stack rows (sum over its windows / nstep)
// are folded into a per-group stack on the device, and after the last
// timestamp each group gets ONE inverse transform, divided by the group's
// record count. The finalize is linear, so this equals the mean over
// timestamps of the per-timestamp NCFs up to float32 rounding, with one
// transform per group instead of one per group and timestamp.
//
// Outputs, as the chain writes them: <stack dir>/linearstack_sourcepack/STACK/
// {linearstack.pack, sourcepack_index.tsv, _SUCCESS}, built in STACK.tmp and
// renamed into place. Groups are keyed and ordered like the linear stack
// (path_id = src nsl_id * 10000 + rec nsl_id as 8 digits, component slot with
// the materializer's component ranks); each record's SAC header is the NCF
// header xc_fast writes for the group's first record (earliest timestamp,
// then task order) with npts, iftype, user0 = record count and the fixed
// reference time of linear_stack.py:81-92; index rows carry the xcpack TSV
// texts of that record.
//
//   xc_linear -I <stepack dir|tsv> -P <allowed_paths.tsv> -O <ncf dir> -S <stack dir> -C <cc length s>
//             [-G gpu id] [--progress|--progress-file f]
// (-O only names the records' pair paths, as xc_fast's final_pair_path.)
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <filesystem>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../csrc/hostio.h"
#include "fastxc_gb300.h"
#include "xc_app.h"

using namespace fxcio;

namespace {

struct Group {
  int64_t row = 0;
  int64_t records = 0;
  std::string first_ts;
  SacHeader header;
  Channel s, r;
  float dist = 0, az = 0, baz = 0;
  std::string final_pair;
};

int rank_of(const std::string& comp) {
  // the SourcePack materializer's ranks (builder.py:403-405)
  const char t = comp.empty() ? '\0' : (char)toupper((unsigned char)comp.back());
  switch (t) {
    case 'E': case '1': return 0;
    case 'N': case '2': return 1;
    case 'Z': case '3': return 2;
    case 'R': return 3;
    case 'T': return 4;
    default: return 100;
  }
}

std::string fmt9g(double v) {
  char b[64];
  snprintf(b, sizeof(b), "%.9g", v);
  return b;
}

// csv.writer's minimal quoting for a tab-delimited row
std::string csv_field(const std::string& s) {
  if (s.find_first_of("\t\"\r\n") == std::string::npos) return s;
  std::string o = "\"";
  for (char c : s) {
    if (c == '"') o += '"';
    o += c;
  }
  return o + "\"";
}

bool linear_output_path(const std::string& final_pair, const std::string& stack_dir, std::string* out) {
  std::string name = final_pair.substr(final_pair.find_last_of('/') == std::string::npos
                                           ? 0 : final_pair.find_last_of('/') + 1);
  std::vector<std::string> parts;
  size_t a = 0;
  for (;;) {
    const size_t d = name.find('.', a);
    parts.push_back(name.substr(a, d == std::string::npos ? std::string::npos : d - a));
    if (d == std::string::npos) break;
    a = d + 1;
  }
  if (!parts.empty()) {
    std::string last = parts.back();
    for (char& c : last) c = (char)tolower((unsigned char)c);
    if (last == "sac") parts.pop_back();
  }
  if (parts.size() < 3) return false;
  const std::string pair = parts[0] + "." + parts[1];
  *out = stack_dir + "/linearstack/" + pair + "/" + pair + "." + parts[2] + ".linearstack.sac";
  return true;
}

std::string absolute_dir(const std::string& p) {
  char buf[PATH_MAX];
  if (realpath(p.c_str(), buf)) return buf;
  return std::filesystem::absolute(p).lexically_normal().string();
}

void usage() {
  fprintf(stderr,
          "Usage: xc_linear -I <stepack dir|tsv> -P <allowed_paths.tsv> -O <ncf dir> -S <stack dir>\n"
          "                 -C <cc length s> [-G gpu_id] [--progress|--progress-file file]\n");
}

}  // namespace

int main(int argc, char** argv) {
  const char *input = nullptr, *out_dir = nullptr, *stack_arg = nullptr, *paths_file = nullptr, *progress = nullptr;
  const char* gpus = "0";
  float cclen = 0.0f;
  if (argc <= 1) {
    usage();
    return 1;
  }
  for (int i = 1; i < argc; ++i) {
    const char* o = argv[i];
    auto need = [&](const char* opt) -> const char* {
      if (i + 1 >= argc) {
        FXLOG_ERROR("argument_value_missing", "option=\"%s\"", opt);
        usage();
        exit(1);
      }
      return argv[++i];
    };
    if (!strcmp(o, "-h") || !strcmp(o, "--help")) {
      usage();
      return 0;
    } else if (!strcmp(o, "-I")) input = need(o);
    else if (!strcmp(o, "-O")) out_dir = need(o);
    else if (!strcmp(o, "-S")) stack_arg = need(o);
    else if (!strcmp(o, "-C")) cclen = (float)atof(need(o));
    else if (!strcmp(o, "-G")) gpus = need(o);
    else if (!strcmp(o, "-P")) paths_file = need(o);
    else if (!strcmp(o, "--progress") || !strcmp(o, "--progress-file")) progress = need(o);
    else {
      FXLOG_ERROR("argument_unknown", "option=\"%s\"", o);
      usage();
      return 1;
    }
  }
  if (!input || !out_dir || !stack_arg || !paths_file || cclen <= 0.0f) {
    FXLOG_ERROR("required_argument_missing", "required=\"-I,-P,-O,-S,-C\"");
    usage();
    return 1;
  }
  const int device = atoi(gpus);
  std::vector<PathRecord> paths;
  if (load_allowed_paths(paths_file, &paths) != 0) return 1;
  std::vector<TimestampInput> inputs;
  if (stepack_load_index(input, &inputs) != 0) return 1;
  if (mkdir_p(stack_arg) != 0) {
    FXLOG_ERROR("stack_dir_create_failed", "path=\"%s\"", stack_arg);
    return 1;
  }
  const std::string stack_dir = absolute_dir(stack_arg);
  const std::string out_final = stack_dir + "/linearstack_sourcepack/STACK";
  const std::string out_tmp = out_final + ".tmp";
  const std::string pack_path = out_final + "/linearstack.pack";
  const std::string index_path = out_final + "/sourcepack_index.tsv";

  fxc_ctx* ctx = nullptr;
  if (fxc_ctx_create(device, nullptr, &ctx) != FXC_OK) {
    FXLOG_ERROR("gpu_context_failed", "gpu=%d error=\"%s\"", device, fxc_last_error());
    return 1;
  }
  Progress prog;
  prog.init(progress, "xc_linear", inputs.size(), "timestamp");
  const char* menv = getenv("FASTXC_XC_METHOD");

  std::map<std::pair<std::string, int>, Group> groups;
  void *d_spec = nullptr, *d_day = nullptr, *d_glob = nullptr;
  size_t spec_cap = 0, day_cap = 0;
  int64_t glob_rows = 0, glob_cap = 0;
  fxc_xc_shape shape{};
  bool have_shape = false;
  int64_t pitch = 0;
  int failed = 0;
  size_t done = 0;
  auto fail = [&](const char* ev, const std::string& ts) {
    FXLOG_ERROR(ev, "timestamp=\"%s\" error=\"%s\"", ts.c_str(), fxc_last_error());
    failed = 1;
  };
  auto ensure = [&](void** buf, size_t* cap, size_t need) -> bool {
    if (need <= *cap) return true;
    if (*buf) fxc_device_free(ctx, *buf);
    *buf = nullptr;
    *cap = 0;
    if (fxc_device_alloc(ctx, need, buf) != FXC_OK) return false;
    *cap = need;
    return true;
  };

  for (const TimestampInput& ti : inputs) {
    std::vector<Channel> chans;
    std::vector<float> payload;
    int nstep = 0, nspec = 0;
    float dt = 0, df = 0;
    if (stepack_open_timestamp(ti, &chans, &nstep, &nspec, &dt, &df, &payload) != 0) {
      FXLOG_WARN("timestamp_open_failed", "timestamp=\"%s\" skipped=1", ti.timestamp.c_str());
      continue;
    }
    if (infer_num_channels(chans) == 0) {
      FXLOG_WARN("timestamp_channels_invalid", "timestamp=\"%s\" skipped=1", ti.timestamp.c_str());
      continue;
    }
    fxc_xc_shape sh;
    if (fxc_xc_shape_init(nspec, nstep, dt, cclen, &sh) != FXC_OK) {
      fail("shape_invalid", ti.timestamp);
      break;
    }
    if (!have_shape) {
      shape = sh;
      have_shape = true;
      pitch = ((int64_t)nspec + 3) / 4 * 4;
    } else if (sh.nspec != shape.nspec || sh.cc_size != shape.cc_size || sh.dt != shape.dt) {
      FXLOG_ERROR("timestamp_shape_mismatch", "timestamp=\"%s\" nspec=%d expected_nspec=%d", ti.timestamp.c_str(),
                  sh.nspec, shape.nspec);
      failed = 1;
      break;
    }
    const size_t nch = chans.size();
    std::vector<int> gnsl(nch);
    for (size_t c = 0; c < nch; ++c) gnsl[c] = chans[c].nsl_id;
    const std::vector<Job> jobs = build_jobs(nch, nch);
    const std::vector<Task> tasks = build_tasks(gnsl, paths, jobs[0]);
    if (tasks.empty()) {
      ++done;
      prog.update(done, "RUNNING", ti.timestamp.c_str());
      continue;
    }
    std::vector<int32_t> src(tasks.size()), rec(tasks.size());
    for (size_t k = 0; k < tasks.size(); ++k) {
      src[k] = (int32_t)tasks[k].src;
      rec[k] = (int32_t)tasks[k].rec;
    }
    // per-timestamp stack rows on the device
    const size_t spec_bytes = sizeof(float) * payload.size();
    const size_t day_bytes = sizeof(float) * 2 * (size_t)pitch * tasks.size();
    if (!ensure(&d_spec, &spec_cap, spec_bytes) || !ensure(&d_day, &day_cap, day_bytes) ||
        fxc_memcpy(ctx, d_spec, payload.data(), spec_bytes, FXC_COPY_H2D) != FXC_OK) {
      fail("xc_device_memory_failed", ti.timestamp);
      break;
    }
    int method = -1;
    if (menv && !strcmp(menv, "plain")) method = FXC_XC_PLAIN;
    if (menv && !strcmp(menv, "tensor")) method = FXC_XC_TENSOR;
    fxc_pairplan* plan = nullptr;
    int rc = fxc_pairplan_create(ctx, src.data(), rec.data(), (int64_t)tasks.size(), (int32_t)nch, &plan);
    if (rc == FXC_OK && method < 0) rc = autotune_host(ctx, plan, payload, nstep, (int32_t)nch, nspec, &method);
    if (rc == FXC_OK)
      rc = fxc_xc_stack(ctx, plan, (const float*)d_spec, nstep, (int32_t)nch, nspec, nspec, nullptr,
                        1.0f / (float)nstep, (float*)d_day, pitch, method);
    fxc_pairplan_destroy(plan);
    if (rc != FXC_OK) {
      fail("xc_gpu_failed", ti.timestamp);
      break;
    }
    // group rows: new groups take the next rows; a group's first record is
    // its earliest timestamp, then the first task
    TimeInfo tinfo;
    const bool have_time = parse_timestamp(ti.timestamp, &tinfo);
    const float cc_len_s = (float)shape.half_cc * shape.dt;
    std::vector<int64_t> rows(tasks.size());
    std::vector<char> fresh(tasks.size(), 0);
    for (size_t k = 0; k < tasks.size(); ++k) {
      const Channel& s = chans[tasks[k].src];
      const Channel& r = chans[tasks[k].rec];
      char pid[32];
      snprintf(pid, sizeof(pid), "%08d", s.nsl_id * 10000 + r.nsl_id);
      const int slot = rank_of(tsv_clean(s.component)) * 3 + rank_of(tsv_clean(r.component));
      auto it = groups.find({pid, slot});
      const bool first_ever = it == groups.end();
      if (first_ever) {
        Group g;
        g.row = glob_rows++;
        it = groups.emplace(std::make_pair(std::string(pid), slot), g).first;
      }
      Group& g = it->second;
      if (first_ever || ti.timestamp < g.first_ts) {
        g.first_ts = ti.timestamp;
        g.header = ncf_header(tasks[k], s, r, shape.dt, shape.cc_size, cc_len_s, &tinfo, have_time);
        g.s = s;
        g.r = r;
        g.dist = tasks[k].path->dist;
        g.az = tasks[k].path->az;
        g.baz = tasks[k].path->baz;
        g.final_pair = tsv_clean(final_pair_path(out_dir, s, r));
      }
      ++g.records;
      rows[k] = g.row;
      fresh[k] = first_ever;  // only a group's first task ever
    }
    // grow the cross-timestamp stack (doubling, rows kept)
    if (glob_rows > glob_cap) {
      int64_t cap = glob_cap ? glob_cap : 1024;
      while (cap < glob_rows) cap *= 2;
      void* grown = nullptr;
      const size_t row_bytes = sizeof(float) * 2 * (size_t)pitch;
      if (fxc_device_alloc(ctx, row_bytes * (size_t)cap, &grown) != FXC_OK ||
          (glob_cap && fxc_memcpy(ctx, grown, d_glob, row_bytes * (size_t)glob_cap, FXC_COPY_D2D) != FXC_OK)) {
        fail("xc_device_memory_failed", ti.timestamp);
        break;
      }
      if (d_glob) fxc_device_free(ctx, d_glob);
      d_glob = grown;
      glob_cap = cap;
    }
    // fold: rows that start a group are assigned, the rest added; a group
    // met twice in one timestamp is folded by a later call (destination rows
    // of one call are distinct)
    std::vector<char> pending(tasks.size(), 1);
    for (size_t left = tasks.size(); left > 0 && !failed;) {
      std::vector<int64_t> sa, da, sb, db;  // assign / add: source task, group row
      std::map<int64_t, int> taken;
      for (size_t k = 0; k < tasks.size(); ++k) {
        if (!pending[k] || taken.count(rows[k])) continue;
        taken[rows[k]] = 1;
        pending[k] = 0;
        --left;
        (fresh[k] ? sa : sb).push_back((int64_t)k);
        (fresh[k] ? da : db).push_back(rows[k]);
      }
      if ((!sa.empty() && fxc_xc_rows_accumulate(ctx, (const float*)d_day, (int64_t)tasks.size(), pitch, sa.data(),
                                                 da.data(), (int64_t)sa.size(), (float*)d_glob, glob_rows, pitch,
                                                 shape.nspec, 1) != FXC_OK) ||
          (!sb.empty() && fxc_xc_rows_accumulate(ctx, (const float*)d_day, (int64_t)tasks.size(), pitch, sb.data(),
                                                 db.data(), (int64_t)sb.size(), (float*)d_glob, glob_rows, pitch,
                                                 shape.nspec, 0) != FXC_OK))
        fail("xc_fold_failed", ti.timestamp);
    }
    if (failed) break;
    ++done;
    prog.update(done, "RUNNING", ti.timestamp.c_str());
    FXLOG_INFO("timestamp_done", "timestamp=\"%s\" pairs=%zu groups=%lld", ti.timestamp.c_str(), tasks.size(),
               (long long)glob_rows);
  }

  // one finalize per group, mean over its records, SourcePack out
  std::vector<float> ncf;
  if (!failed && glob_rows > 0) {
    void* d_ncf = nullptr;
    const size_t nbytes = sizeof(float) * (size_t)glob_rows * shape.cc_size;
    ncf.resize((size_t)glob_rows * shape.cc_size);
    if (fxc_device_alloc(ctx, nbytes, &d_ncf) != FXC_OK ||
        fxc_xc_finalize(ctx, (const float*)d_glob, glob_rows, pitch, &shape, (float*)d_ncf) != FXC_OK ||
        fxc_memcpy(ctx, ncf.data(), d_ncf, nbytes, FXC_COPY_D2H) != FXC_OK) {
      fail("xc_finalize_failed", "STACK");
    }
    if (d_ncf) fxc_device_free(ctx, d_ncf);
  }
  if (d_spec) fxc_device_free(ctx, d_spec);
  if (d_day) fxc_device_free(ctx, d_day);
  if (d_glob) fxc_device_free(ctx, d_glob);
  fxc_ctx_destroy(ctx);

  if (!failed && !groups.empty()) {
    std::error_code ec;
    std::filesystem::remove_all(out_tmp, ec);
    std::filesystem::create_directories(out_tmp, ec);
    FILE* pack = fopen((out_tmp + "/linearstack.pack").c_str(), "wb");
    FILE* idx = fopen((out_tmp + "/sourcepack_index.tsv").c_str(), "wb");
    if (!pack || !idx) {
      FXLOG_ERROR("stack_output_open_failed", "path=\"%s\"", out_tmp.c_str());
      failed = 1;
    } else {
      static const char* kCols[] = {"timestamp", "path_id", "component_slot", "source_key", "receiver_key",
                                    "src_id", "rec_id", "src_network", "src_station", "src_location",
                                    "src_component", "rec_network", "rec_station", "rec_location", "rec_component",
                                    "npts", "dt", "dist", "az", "baz", "record_path", "record_offset", "bytes",
                                    "storage_kind", "final_pair_path"};
      std::string line;
      for (size_t c = 0; c < sizeof(kCols) / sizeof(kCols[0]); ++c) line += (c ? "\t" : "") + std::string(kCols[c]);
      fputs((line + "\r\n").c_str(), idx);
      uint64_t off = 0;
      std::vector<float> data(shape.cc_size);
      for (const auto& kv : groups) {
        const Group& g = kv.second;
        std::string lpath;
        if (!linear_output_path(g.final_pair, stack_dir, &lpath)) {
          FXLOG_ERROR("final_pair_path_unexpected", "path=\"%s\"", g.final_pair.c_str());
          failed = 1;
          break;
        }
        const float* row = ncf.data() + (size_t)g.row * shape.cc_size;
        for (int j = 0; j < shape.cc_size; ++j) data[j] = (float)((double)row[j] / (double)g.records);
        SacHeader h = g.header;
        h.i[SI_NPTS] = shape.cc_size;
        h.i[SI_IFTYPE] = 1;
        h.f[SF_USER0] = (float)g.records;
        h.i[SI_NZYEAR] = 2010;
        h.i[SI_NZJDAY] = 214;
        h.i[SI_NZHOUR] = h.i[SI_NZMIN] = h.i[SI_NZSEC] = h.i[SI_NZMSEC] = 0;
        const uint64_t nb = sizeof(SacHeader) + sizeof(float) * (uint64_t)shape.cc_size;
        if (fwrite(&h, sizeof(h), 1, pack) != 1 || fwrite(data.data(), sizeof(float), data.size(), pack) != data.size()) {
          failed = 1;
          break;
        }
        const std::string sn = tsv_clean(g.s.network), ss = tsv_clean(g.s.station), sl = tsv_clean(g.s.location);
        const std::string rn = tsv_clean(g.r.network), rs = tsv_clean(g.r.station), rl = tsv_clean(g.r.location);
        const std::vector<std::string> f = {
            "STACK", kv.first.first, std::to_string(kv.first.second), sn + "." + ss + "." + sl,
            rn + "." + rs + "." + rl, std::to_string(g.s.nsl_id), std::to_string(g.r.nsl_id), sn, ss, sl,
            tsv_clean(g.s.component), rn, rs, rl, tsv_clean(g.r.component), std::to_string(h.i[SI_NPTS]),
            fmt9g(h.f[SF_DELTA]), fmt9g(g.dist), fmt9g(g.az), fmt9g(g.baz), pack_path, std::to_string(off),
            std::to_string(nb), "linearstack_pack", lpath};
        line.clear();
        for (size_t c = 0; c < f.size(); ++c) line += (c ? "\t" : "") + csv_field(f[c]);
        fputs((line + "\r\n").c_str(), idx);
        off += nb;
      }
    }
    if (pack && fclose(pack) != 0) failed = 1;
    if (idx && fclose(idx) != 0) failed = 1;
    if (!failed) {
      FILE* ok = fopen((out_tmp + "/_SUCCESS").c_str(), "wb");
      if (!ok) {
        failed = 1;
      } else {
        fprintf(ok, "records\t%zu\npack\t%s\nindex\t%s\n", groups.size(), pack_path.c_str(), index_path.c_str());
        if (fclose(ok) != 0) failed = 1;
      }
    }
    if (!failed) {
      std::filesystem::remove_all(out_final, ec);
      std::filesystem::rename(out_tmp, out_final, ec);
      if (ec) {
        FXLOG_ERROR("stack_output_rename_failed", "path=\"%s\"", out_final.c_str());
        failed = 1;
      }
    }
  }
  prog.update(done, failed ? "FAILED" : "DONE");
  FXLOG_INFO("linear_stack_done", "groups=%zu failed=%d", groups.size(), failed);
  return failed ? 1 : 0;
}
