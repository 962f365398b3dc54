// SourcePack input/output of the stacking executables (ncf_pws, ncf_tfpws).
//
// A SourcePack is a set of index TSVs whose rows point at SAC records
// (632-byte header + f32 samples) inside pack files. The stacking stages
// read every index of a list, merge their rows into groups of one
// (path_id, component_slot) each, stack every group into one trace and
// write the stacks as shard packs + a merged index.
//
// Semantics restated from native/pws/io/sourcepack_io.cu (identical in
// native/tfpws/io/sourcepack_io.cu): the index header and required fields
// (:70-76, :131-147), the list file (:94-117), the k-way merge into groups
// ordered by (path_id as a string, component_slot, arrival sequence) with
// each group's records sorted by (timestamp, record_path, record_offset)
// (:201-280), the record checks (:325-383), the shard writer
// (<prefix>.wNNN.{pack,tsv}, :480-624), the merge of shard indexes sorted
// by (path_id, component_slot, worker, row) (:626-706) and the _SUCCESS
// marker (native/pws/worker/sourcepack_pipeline.cu:443-455).
#pragma once

#include <stdio.h>

#include <fstream>
#include <map>
#include <queue>
#include <string>
#include <vector>

#include "hostio.h"

namespace fxcio {

struct SourcePackRecord {
  std::string timestamp, path_id, source_key, receiver_key, src_id, rec_id;
  std::string src_network, src_station, src_location, src_component;
  std::string rec_network, rec_station, rec_location, rec_component;
  std::string dist, az, baz, final_pair_path, record_path;
  int component_slot = 0;
  long long record_offset = 0, record_bytes = 0;
};

const char* sourcepack_index_header();
std::string join_path(const std::string& dir, const char* name);
std::string absolute_path(const std::string& path);
int read_sourcepack_list(const char* path, std::vector<std::string>* indexes);

class SourcePackStream {
 public:
  explicit SourcePackStream(const std::string& path) : path_(path) {}
  int open();
  bool next(SourcePackRecord* r);

 private:
  std::string value(const std::vector<std::string>& row, const char* name) const;
  std::string path_;
  std::ifstream in_;
  std::map<std::string, int> fields_;
};

class SourcePackGroupReader {
 public:
  explicit SourcePackGroupReader(const std::vector<std::string>& paths) : paths_(paths) {}
  ~SourcePackGroupReader();
  int open();
  bool next_group(std::vector<SourcePackRecord>* records);

 private:
  struct Item {
    SourcePackRecord record;
    size_t stream = 0, seq = 0;
  };
  struct Later {
    bool operator()(const Item& a, const Item& b) const;
  };
  void push(const SourcePackRecord& r, size_t stream);
  std::vector<std::string> paths_;
  std::vector<SourcePackStream*> streams_;
  std::priority_queue<Item, std::vector<Item>, Later> heap_;
  size_t seq_ = 0;
};

size_t count_sourcepack_groups(const std::vector<std::string>& indexes);

// Open pack files by path (at most 256 at a time).
class PackFileCache {
 public:
  ~PackFileCache() { close_all(); }
  FILE* get(const std::string& path);
  void close_all();

 private:
  std::map<std::string, FILE*> files_;
};

// Sample count of a SAC header (2 x npts for x-y files).
unsigned sac_data_count(const SacHeader& hd);
// Reads one record; checks its sample count and byte size against the index.
int read_sourcepack_record(PackFileCache* cache, const SourcePackRecord& r, SacHeader* hd,
                           float* data, unsigned expected_samples);
// Header of the first record of a group.
int read_sourcepack_header(PackFileCache* cache, const SourcePackRecord& r, SacHeader* hd);

class StackShardWriter {
 public:
  // prefix "pws" or "tfpws": files <prefix>.wNNN.pack / .tsv, storage kind
  // <prefix>_pack, final pair path suffix .<prefix>.sac.
  int open(const std::string& output_dir, const std::string& prefix, size_t worker);
  int append(const SourcePackRecord& r, const SacHeader& hd, const float* data);
  int close();
  ~StackShardWriter() { close(); }
  std::string final_pair_path(const SourcePackRecord& r) const;
  const std::string& pack_path() const { return pack_path_; }

 private:
  std::string dir_, prefix_, pack_path_, index_path_;
  FILE* pack_ = nullptr;
  std::ofstream index_;
};

int merge_shard_indexes(const std::string& output_dir, const std::string& prefix, size_t workers,
                        const std::string& final_index);
int write_stack_success(const std::string& output_dir, const std::string& prefix,
                        size_t records, size_t workers, const std::string& index_path);

}  // namespace fxcio
