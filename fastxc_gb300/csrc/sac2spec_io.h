// Host inputs and bookkeeping of the sac2spec drop-in.
//
// Restated from the reference (native/sac2spec/):
//   read_sac_index      readSacIndexPaths (io/sac_index.c:33-365): rows
//                       "timestamp nsl_id network station location component
//                       sac_path" (tab separated; header, blank and '#'
//                       lines skipped; fields trimmed, inner whitespace runs
//                       -> '_'), consecutive rows of one (nsl_id, timestamp)
//                       form a group that is kept when num_ch == 1 or it has
//                       exactly num_ch rows; nsl_id must be 0..9999.
//   read_filter_file    readButterworthFilters (core/filter_response.c:118-184).
//   sac_delta_matches   sacDeltaMatches (io/parallel_io.c:26-49): |d - e| <=
//                       max(|e| 1e-5, 1e-6).
//   timestamp_leaf      PathSafeTimestampLeaf / PathTimestampLeafIsSafe
//                       (path_utils.c:141-181).
//   S2sProgress         the progress sidecar of progress.cu:13-120.
//   TimestampTracker    timestamp_tracker.cu: <stepack>/<ts>/_SUCCESS once
//                       every group of a timestamp is written.
#pragma once

#include <mutex>
#include <string>
#include <vector>

#include "hostio.h"

namespace fxcio {

struct SacIndexRow {
  std::string timestamp, nsl_text, network, station, location, component, sac_path;
  int nsl_id = 0;
};
// Kept rows in file order (groups of num_ch consecutive rows); -1 on a fatal
// format error (logged), 0 otherwise.
int read_sac_index(const char* path, int num_ch, std::vector<SacIndexRow>* rows);

struct FilterSet {
  std::vector<float> freq_low, freq_high;
  std::vector<double> b, a;  // [n][5]
  int count() const { return (int)freq_low.size(); }
};
int read_filter_file(const char* path, FilterSet* out);

bool sac_delta_matches(float observed, float expected);
std::string timestamp_leaf(const std::string& ts);
bool timestamp_leaf_is_safe(const std::string& ts);

class S2sProgress {
 public:
  void init(const std::string& path, size_t total_rows);
  void add(size_t rows, int gpu_id, size_t start_group, size_t group_count);
  void finish(const char* status, bool complete);

 private:
  void write_locked(const char* status, int gpu_id, size_t batch_rows, size_t start_group,
                    size_t group_count);
  std::mutex mu_;
  std::string path_;
  size_t total_ = 0, done_ = 0;
  bool enabled_ = false;
};

class TimestampTracker {
 public:
  // groups: group g holds rows [g*num_ch, (g+1)*num_ch); their timestamps
  // must agree and be path-safe.
  int init(const std::vector<SacIndexRow>& rows, int num_ch, const std::string& stepack_root);
  int mark_done(size_t start_group, size_t group_count);

 private:
  struct Entry {
    std::string timestamp;
    size_t group_count = 0, done = 0;
  };
  std::mutex mu_;
  std::string root_;
  std::vector<Entry> entries_;
  std::vector<int> group_entry_;
};

}  // namespace fxcio
