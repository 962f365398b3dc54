// xc_fast drop-in: stepack spectra -> per-pair correlation stacked over the
// timestamp's windows -> +-max_lag NCFs -> xcpack records.
//
// Command line of the reference (native/xc/arguproc.c:165-235):
//   xc_fast -I <stepack dir|tsv> -P <allowed_paths.tsv> -O <ncf dir> -C <max_lag s>
//           [-G gpu ids] [-M mem MiB] [-J lazy depth] [--progress|--progress-file f] [--debug]
// Output (native/xc/pack_io/pack_writer.cu): <ncf>/xcpack/<ts>.iAAAAAA.jBBBBBB.wWWW.pPPP.{xcpack,tsv},
// <ts>.done per timestamp, _SUCCESS at the end; exit code 0 / 1.
//
// Memory: each timestamp's pairs run in blocks whose device footprint
// (fxc_xc_host_bytes) fits the budget: -M MiB when given, else 0.9 x the free
// device memory at start (the reference's pair-block sizing,
// native/xc/memory/memory.cu:112-399, over this library's buffers).
//
// Option of this build: --sourcepack <dir> writes each timestamp's SourcePack
// index (<dir>/<ts>/{sourcepack_index.tsv,_SUCCESS}, the files the
// reference's build_sourcepack makes afterwards) as soon as the timestamp's
// records and .done marker are on disk.
//
// Environment: FASTXC_XC_METHOD=plain|tensor (default: method and
// contraction layout autotuned per timestamp shape with
// fxc_xc_autotune_layout), FASTXC_XC_BLOCK=<files per block>
// (default: the whole timestamp in one block), FASTXC_LOG_LEVEL.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>

#include <string>
#include <vector>

#include "../csrc/hostio.h"
#include "fastxc_gb300.h"
#include "xc_app.h"

using namespace fxcio;

static void usage() {
  fprintf(stderr,
          "Usage: xc_fast -I <stepack dir|tsv> -P <allowed_paths.tsv> -O <ncf dir> -C <cc length s>\n"
          "               [-G gpu_ids] [-M gpu_mem_mib] [-J lazy_write_depth]\n"
          "               [--progress|--progress-file file] [--sourcepack dir] [--debug]\n");
}

int main(int argc, char** argv) {
  const char *input = nullptr, *out_dir = nullptr, *paths_file = nullptr, *progress = nullptr;
  const char* sourcepack_dir = nullptr;
  const char* gpus = "0";
  const char* mem_mib = nullptr;
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
    else if (!strcmp(o, "-C")) cclen = (float)atof(need(o));
    else if (!strcmp(o, "-G")) gpus = need(o);
    else if (!strcmp(o, "-M")) mem_mib = need(o);
    else if (!strcmp(o, "-P")) paths_file = need(o);
    else if (!strcmp(o, "-J")) (void)need(o);
    else if (!strcmp(o, "--progress") || !strcmp(o, "--progress-file")) progress = need(o);
    else if (!strcmp(o, "--sourcepack")) sourcepack_dir = need(o);
    else if (!strcmp(o, "--debug")) {
    } else {
      FXLOG_ERROR("argument_unknown", "option=\"%s\"", o);
      usage();
      return 1;
    }
  }
  if (!out_dir || cclen <= 0.0f || !paths_file) {
    FXLOG_ERROR("required_argument_missing", "required=\"-O,-C,-P\"");
    usage();
    return 1;
  }
  if (!input) {
    FXLOG_ERROR("timestamp_input_missing", "required=\"-I\"");
    usage();
    return 1;
  }
  const int device = atoi(gpus);  // one GPU per process; further ids are other processes

  std::vector<PathRecord> paths;
  if (load_allowed_paths(paths_file, &paths) != 0) return 1;
  std::vector<TimestampInput> inputs;
  if (stepack_load_index(input, &inputs) != 0) return 1;
  FXLOG_INFO("stepack_index_loaded", "timestamps=%zu", inputs.size());

  fxc_ctx* ctx = nullptr;
  if (fxc_ctx_create(device, nullptr, &ctx) != FXC_OK) {
    FXLOG_ERROR("gpu_context_failed", "gpu=%d error=\"%s\"", device, fxc_last_error());
    return 1;
  }
  int64_t budget = 0;
  if (mem_mib && atoll(mem_mib) > 0) {
    budget = (int64_t)atoll(mem_mib) << 20;
  } else {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      FXLOG_ERROR("gpu_memory_query_failed", "gpu=%d", device);
      return 1;
    }
    budget = (int64_t)((double)free_b * 0.9);
  }
  FXLOG_INFO("xc_memory_budget", "gpu=%d budget_mib=%lld", device, (long long)(budget >> 20));
  Progress prog;
  prog.init(progress, "xc", inputs.size(), "timestamp");
  const std::string root = std::string(out_dir) + "/xcpack";
  if (mkdir_p(root) != 0) {
    FXLOG_ERROR("xcpack_dir_create_failed", "path=\"%s\"", root.c_str());
    return 1;
  }
  const char* menv = getenv("FASTXC_XC_METHOD");
  const char* benv = getenv("FASTXC_XC_BLOCK");
  int failed = 0;
  size_t done = 0;
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
    fxc_xc_shape shape;
    if (fxc_xc_shape_init(nspec, nstep, dt, cclen, &shape) != FXC_OK) {
      FXLOG_ERROR("shape_invalid", "timestamp=\"%s\" error=\"%s\"", ti.timestamp.c_str(), fxc_last_error());
      failed = 1;
      break;
    }
    const size_t nch = chans.size();
    size_t bs = benv ? (size_t)atol(benv) : nch;
    if (bs == 0 || bs > nch) bs = nch;
    std::vector<int> gnsl(nch);
    for (size_t c = 0; c < nch; ++c) gnsl[c] = chans[c].nsl_id;
    std::vector<Job> jobs = build_jobs(nch, bs);
    std::vector<std::vector<Task>> job_tasks(jobs.size());
    std::vector<int32_t> src, rec;
    for (size_t j = 0; j < jobs.size(); ++j) {
      job_tasks[j] = build_tasks(gnsl, paths, jobs[j]);
      for (const Task& t : job_tasks[j]) {
        src.push_back((int32_t)t.src);
        rec.push_back((int32_t)t.rec);
      }
    }
    std::vector<float> ncf((size_t)src.size() * shape.cc_size);
    if (!src.empty()) {
      int method = -1;  // autotuned unless FASTXC_XC_METHOD names one
      if (menv && !strcmp(menv, "plain")) method = FXC_XC_PLAIN;
      if (menv && !strcmp(menv, "tensor")) method = FXC_XC_TENSOR;
      const int64_t npairs = (int64_t)src.size();
      fxc_pairplan* plan = nullptr;
      int rc = FXC_OK;
      int32_t layout = FXC_XC_LAYOUT_AUTO;
      if (method < 0) {
        // the autotuner samples a few bins of every pair: its plan is the whole list
        rc = fxc_pairplan_create(ctx, src.data(), rec.data(), npairs, (int32_t)nch, &plan);
        if (rc == FXC_OK) rc = autotune_host(ctx, plan, payload, nstep, (int32_t)nch, nspec, &method, &layout);
        fxc_pairplan_destroy(plan);
        plan = nullptr;
      }
      int64_t block = npairs;
      if (rc == FXC_OK)
        rc = fxc_plan_xc_pairs(npairs, nstep, (int32_t)nch, nspec, &shape, method, 0, budget, &block, nullptr);
      if (rc == FXC_OK && block < npairs)
        FXLOG_INFO("xc_pair_blocks", "timestamp=\"%s\" pairs=%lld per_block=%lld", ti.timestamp.c_str(),
                   (long long)npairs, (long long)block);
      for (int64_t p0 = 0; rc == FXC_OK && p0 < npairs; p0 += block) {
        const int64_t np = std::min(block, npairs - p0);
        rc = fxc_pairplan_create(ctx, src.data() + p0, rec.data() + p0, np, (int32_t)nch, &plan);
        // the layout tuned on the whole list, where a block's plan admits it
        if (rc == FXC_OK && method == FXC_XC_TENSOR) rc = fxc_pairplan_set_layout(plan, layout);
        if (rc == FXC_OK)
          rc = fxc_xc_run_host(ctx, plan, payload.data(), nstep, (int32_t)nch, nspec, nullptr, 1.0f / (float)nstep,
                               &shape, ncf.data() + (size_t)p0 * shape.cc_size, method);
        fxc_pairplan_destroy(plan);
        plan = nullptr;
      }
      if (rc != FXC_OK) {
        FXLOG_ERROR("xc_gpu_failed", "timestamp=\"%s\" error=\"%s\"", ti.timestamp.c_str(), fxc_last_error());
        failed = 1;
        break;
      }
    }
    TimeInfo tinfo;
    const bool have_time = parse_timestamp(ti.timestamp, &tinfo);
    const float cc_len_s = (float)shape.half_cc * shape.dt;
    size_t k = 0;
    for (size_t j = 0; j < jobs.size(); ++j) {
      if (job_tasks[j].empty()) continue;
      XcPackWriter w;
      if (w.open(root, ti.timestamp, 0, jobs[j]) != 0) {
        FXLOG_ERROR("xcpack_writer_open_failed", "timestamp=\"%s\"", ti.timestamp.c_str());
        failed = 1;
        break;
      }
      for (const Task& t : job_tasks[j]) {
        const Channel& s = chans[t.src];
        const Channel& r = chans[t.rec];
        SacHeader hd = ncf_header(t, s, r, shape.dt, shape.cc_size, cc_len_s, &tinfo, have_time);
        if (w.append(t, s, r, hd, ncf.data() + k * shape.cc_size, shape.cc_size, shape.dt,
                     final_pair_path(out_dir, s, r)) != 0) {
          failed = 1;
          break;
        }
        ++k;
      }
      if (w.close() != 0) failed = 1;
      if (failed) break;
    }
    if (failed) break;
    if (write_marker(root + "/" + ti.timestamp + ".done") != 0) {
      failed = 1;
      break;
    }
    if (sourcepack_dir &&
        fxc_sourcepack_build(root.c_str(), sourcepack_dir, ti.timestamp.c_str(), 1, nullptr, nullptr, nullptr, 0,
                             nullptr, 0) != FXC_OK) {
      FXLOG_ERROR("sourcepack_index_failed", "timestamp=\"%s\" error=\"%s\"", ti.timestamp.c_str(),
                  fxc_last_error());
      failed = 1;
      break;
    }
    ++done;
    prog.update(done, "RUNNING", ti.timestamp.c_str());
    FXLOG_INFO("timestamp_done", "timestamp=\"%s\" pairs=%zu", ti.timestamp.c_str(), src.size());
  }
  fxc_ctx_destroy(ctx);
  if (!failed && write_marker(root + "/_SUCCESS") != 0) failed = 1;
  prog.update(done, failed ? "FAILED" : "DONE");
  return failed ? 1 : 0;
}
