// Test shim around the reference's own xc scheduler, compiled on the CPU from
// the reference sources by oracle/build_ref.py (TEST INFRASTRUCTURE ONLY).
//
// ref_xc_tasks() builds the RowBatchJob list with build_jobs() and the
// XcTask list of every job with build_tasks_for_job()
// (native/xc/worker/scheduler.cu:43-148) for a timestamp whose channels have
// the given NSL ids, against an allowed-path table holding the given
// (src, rec) NSL pairs (native/xc/io/path_table.c), and returns the tasks
// in execution order.
#include <cstdlib>
#include <vector>

#include "worker/scheduler.hpp"

extern "C" {
#include "io/path_table.h"
}

static int cmp_path(const void* a, const void* b) {
  const AllowedPathRecord* x = static_cast<const AllowedPathRecord*>(a);
  const AllowedPathRecord* y = static_cast<const AllowedPathRecord*>(b);
  return (x->path_id > y->path_id) - (x->path_id < y->path_id);
}

extern "C" int ref_xc_tasks(const int* gnsl, int nfiles, const int* path_src, const int* path_rec,
                            int npaths, int block_size, int* out_src, int* out_rec, int* out_path,
                            int* out_auto, int* out_job, int max_out) {
  TimestampWork work;
  work.specs.resize((size_t)nfiles);
  for (int i = 0; i < nfiles; ++i) work.specs[i].gnsl_id = gnsl[i];
  AllowedPathTable table;
  init_allowed_path_table(&table);
  table.records = static_cast<AllowedPathRecord*>(calloc((size_t)(npaths > 0 ? npaths : 1), sizeof(AllowedPathRecord)));
  table.count = (size_t)npaths;
  for (int i = 0; i < npaths; ++i) {
    AllowedPathRecord& r = table.records[i];
    r.src_gnsl_id = path_src[i];
    r.rec_gnsl_id = path_rec[i];
    r.path_id = make_allowed_path_id(path_src[i], path_rec[i]);
  }
  if (npaths > 1) qsort(table.records, table.count, sizeof(AllowedPathRecord), cmp_path);
  std::vector<RowBatchJob> jobs = build_jobs((size_t)nfiles, (size_t)block_size);
  std::vector<size_t> loaded;
  int n = 0;
  for (size_t j = 0; j < jobs.size(); ++j) {
    std::vector<XcTask> tasks = build_tasks_for_job(&work, &table, &jobs[j], &loaded);
    for (const XcTask& t : tasks) {
      if (n >= max_out) {
        free_allowed_path_table(&table);
        return -1;
      }
      out_src[n] = (int)t.src_meta_idx;
      out_rec[n] = (int)t.rec_meta_idx;
      out_path[n] = t.path_id;
      out_auto[n] = t.is_autocorr ? 1 : 0;
      out_job[n] = (int)j;
      ++n;
    }
  }
  free_allowed_path_table(&table);
  return n;
}
