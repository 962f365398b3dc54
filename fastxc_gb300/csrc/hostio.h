// Host-side formats and scheduling shared by the drop-in executables.
//
// Byte layouts follow the reference so that its callers and readers keep
// working: SAC headers (native/xc/include/sac.h), stepack v3 batches and
// their TSV sidecars (native/sac2spec/io/stepack_writer.c), xcpack records
// and TSV rows (native/xc/pack_io/pack_writer.cu), the allowed-path table
// (native/xc/io/path_table.c), the structured stderr log
// (native/xc/logger.c:66-86) and the progress sidecar
// (native/progress_sidecar.hpp:189).
#pragma once

#include <stdint.h>
#include <stdio.h>

#include <string>
#include <vector>

namespace fxcio {

// ---- logging ---------------------------------------------------------------
enum LogLevel { LOG_ERROR = 0, LOG_WARN = 1, LOG_INFO = 2, LOG_DEBUG = 3 };
void log_msg(LogLevel lvl, const char* event, const char* file, int line, const char* fmt, ...);
#define FXLOG_ERROR(ev, ...) fxcio::log_msg(fxcio::LOG_ERROR, ev, __FILE__, __LINE__, __VA_ARGS__)
#define FXLOG_WARN(ev, ...) fxcio::log_msg(fxcio::LOG_WARN, ev, __FILE__, __LINE__, __VA_ARGS__)
#define FXLOG_INFO(ev, ...) fxcio::log_msg(fxcio::LOG_INFO, ev, __FILE__, __LINE__, __VA_ARGS__)

// ---- progress sidecar (task status completed total unit detail) ------------
struct Progress {
  std::string path;
  std::string task, unit;
  size_t total = 0, completed = 0;
  void init(const char* p, const char* task_name, size_t tot, const char* unit_name);
  void update(size_t done, const char* status, const char* detail = "");
};

// ---- SAC --------------------------------------------------------------------
#pragma pack(push, 1)
struct SacHeader {
  float f[70];
  int32_t i[40];
  char kstnm[8];
  char kevnm[16];
  char khole[8], ko[8], ka[8];
  char kt[10][8];
  char kf[8];
  char kuser[3][8];
  char kcmpnm[8], knetwk[8], kdatrd[8], kinst[8];
};
#pragma pack(pop)
static_assert(sizeof(SacHeader) == 632, "SAC header is 632 bytes");

enum SacFloat { SF_DELTA = 0, SF_B = 5, SF_E = 6, SF_O = 7, SF_STLA = 31, SF_STLO = 32,
                SF_EVLA = 35, SF_EVLO = 36, SF_USER0 = 40, SF_USER1 = 41, SF_USER2 = 42,
                SF_DIST = 50, SF_AZ = 51, SF_BAZ = 52, SF_GCARC = 53 };
enum SacInt { SI_NZYEAR = 0, SI_NZJDAY = 1, SI_NZHOUR = 2, SI_NZMIN = 3, SI_NZSEC = 4,
              SI_NZMSEC = 5, SI_NVHDR = 6, SI_NPTS = 9, SI_IFTYPE = 15, SI_LEVEN = 35,
              SI_UNUSED27 = 39 };

SacHeader sac_null();
void sac_text(char* dst, size_t size, const std::string& s);  // space padded, no NUL
int sac_read(const char* path, SacHeader* hd, std::vector<float>* data, int target_npts);

struct TimeInfo {
  int year = 0, jday = 0, hour = 0, minute = 0;
};
bool parse_timestamp(const std::string& ts, TimeInfo* t);

// ---- allowed paths ------------------------------------------------------------
struct PathRecord {
  int path_id, src, rec;
  float gcarc, dist, az, baz;
};
int make_path_id(int src, int rec);
int load_allowed_paths(const char* path, std::vector<PathRecord>* out);  // sorted by path_id
const PathRecord* find_path_canonical(const std::vector<PathRecord>& t, int a, int b);

// ---- xc row-batch jobs and tasks ---------------------------------------------------
struct Job {
  size_t anchor_block, target_begin_block, target_end_block, block_size, file_count;
  size_t anchor_begin, anchor_end, target_begin, target_end;
};
struct Task {
  size_t src, rec;  // channel (meta) indices
  int path_id;
  const PathRecord* path;
  bool autocorr;
};
std::vector<Job> build_jobs(size_t file_count, size_t block_size);
std::vector<Task> build_tasks(const std::vector<int>& gnsl, const std::vector<PathRecord>& paths,
                              const Job& job);

// ---- stepack ---------------------------------------------------------------------
#pragma pack(push, 1)
struct StepackHeader {
  char magic[8];
  uint32_t version, header_size, nslc_entry_size, layout;
  uint64_t batch_seq, start_group, group_count;
  uint32_t worker_id, nstep, nslc_count, nspec;
  float dt, df;
  uint64_t nslc_table_bytes, payload_offset, payload_bytes, pitch_step_bytes;
  char first_timestamp[64];
  unsigned char reserved[64];
};
struct StepackNslc {
  uint32_t file_index, nsl_id;
  float stla, stlo;
  char network[16], station[32], location[16], component[16];
  unsigned char reserved[32];
};
#pragma pack(pop)
static_assert(sizeof(StepackHeader) == 232, "stepack header is 232 bytes");
static_assert(sizeof(StepackNslc) == 128, "stepack NSLC entry is 128 bytes");

struct Channel {
  std::string timestamp, network, station, location, component;
  std::string nsl_text;  // nsl_id as written in the SAC index (stepack TSV first/last_nsl_id)
  int nsl_id = 0;
  float stla = 0, stlo = 0;
};

// Writes w<worker>.b<seq>.stepack + .tsv for one batch (nodes in payload
// order, payload [nstep][nslc][nspec] complex). group_count > 0 gives num_ch.
int stepack_write_batch(const std::string& root, int worker_id, size_t batch_seq,
                        size_t start_group, size_t group_count,
                        const std::vector<Channel>& nslc, int nstep, int nspec, float dt,
                        float df, const float* payload);

struct StepackFragment {
  std::string timestamp, pack_path;
  size_t batch_seq = 0, start_group = 0, nslc_start = 0, nslc_count = 0, batch_nslc_count = 0;
  size_t nstep = 0, nspec = 0, payload_offset = 0, pitch_step_bytes = 0, nslc_step_bytes = 0;
  float dt = 0, df = 0;
};
struct TimestampInput {
  std::string timestamp;
  std::vector<StepackFragment> fragments;
};
// Groups every stepack TSV row (directory of .tsv files or one .tsv) by
// timestamp, sorted like load_stepack_timestamp_inputs_from_tsvs.
int stepack_load_index(const std::string& input, std::vector<TimestampInput>* out);
// Channels of a timestamp (merged, stable-sorted by NSL id) and the payload
// [nstep][nchan][nspec] complex assembled from the fragments.
int stepack_open_timestamp(const TimestampInput& in, std::vector<Channel>* chans, int* nstep,
                           int* nspec, float* dt, float* df, std::vector<float>* payload);
size_t infer_num_channels(const std::vector<Channel>& chans);

// ---- xcpack ------------------------------------------------------------------------
struct XcPackWriter {
  std::string root, timestamp, pack_path, tsv_path;
  size_t worker_id = 0, part = 0;
  Job job{};
  uint64_t bytes = 0, max_bytes = 4ull << 30;
  FILE* pack = nullptr;
  FILE* tsv = nullptr;
  int open(const std::string& root_dir, const std::string& ts, size_t worker, const Job& j);
  int append(const Task& t, const Channel& src, const Channel& rec, const SacHeader& hd,
             const float* trace, int npts, float dt, const std::string& final_pair_path);
  int close();
};
int write_marker(const std::string& path);
std::string final_pair_path(const std::string& ncf_dir, const Channel& src, const Channel& rec);
SacHeader ncf_header(const Task& t, const Channel& src, const Channel& rec, float dt, int cc_size,
                     float cc_len, const TimeInfo* ti, bool have_time);

int mkdir_p(const std::string& path);
// TSV field text: tabs, CR and LF become spaces (the xcpack and progress TSVs)
std::string tsv_clean(const std::string& s);

}  // namespace fxcio
