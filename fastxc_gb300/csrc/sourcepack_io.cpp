// SourcePack readers / shard writers of the stacking executables; the
// semantics and their reference lines are listed in sourcepack_io.h.
#include "sourcepack_io.h"

#include <limits.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cstdlib>

namespace fxcio {

namespace {

std::vector<std::string> split_tabs(const std::string& line) {
  std::vector<std::string> out;
  size_t start = 0;
  for (;;) {
    const size_t pos = line.find('\t', start);
    if (pos == std::string::npos) {
      out.push_back(line.substr(start));
      return out;
    }
    out.push_back(line.substr(start, pos - start));
    start = pos + 1;
  }
}

std::string trim_ws(const std::string& s) {
  size_t a = 0, b = s.size();
  auto ws = [](char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n'; };
  while (a < b && ws(s[a])) ++a;
  while (b > a && ws(s[b - 1])) --b;
  return s.substr(a, b - a);
}

}  // namespace

const char* sourcepack_index_header() {
  return "timestamp\tpath_id\tcomponent_slot\tsource_key\treceiver_key\tsrc_id\trec_id\t"
         "src_network\tsrc_station\tsrc_location\tsrc_component\t"
         "rec_network\trec_station\trec_location\trec_component\t"
         "npts\tdt\tdist\taz\tbaz\trecord_path\trecord_offset\tbytes\tstorage_kind\tfinal_pair_path";
}

std::string join_path(const std::string& dir, const char* name) {
  if (dir.empty() || dir.back() == '/') return dir + name;
  return dir + "/" + name;
}

std::string absolute_path(const std::string& path) {
  if (path.empty() || path[0] == '/') return path;
  char cwd[PATH_MAX];
  if (!getcwd(cwd, sizeof(cwd))) return path;
  return join_path(cwd, path.c_str());
}

int read_sourcepack_list(const char* path, std::vector<std::string>* indexes) {
  std::ifstream in(path);
  if (!in) {
    FXLOG_ERROR("sourcepack_list_open_failed", "path=\"%s\"", path);
    return 1;
  }
  std::string line;
  while (std::getline(in, line)) {
    line = trim_ws(line);
    if (line.empty() || line[0] == '#') continue;
    indexes->push_back(line);
  }
  if (indexes->empty()) {
    FXLOG_ERROR("sourcepack_list_empty", "path=\"%s\"", path);
    return 1;
  }
  return 0;
}

int SourcePackStream::open() {
  in_.open(path_.c_str());
  if (!in_) {
    FXLOG_ERROR("sourcepack_index_open_failed", "path=\"%s\"", path_.c_str());
    return 1;
  }
  std::string header;
  if (!std::getline(in_, header)) {
    FXLOG_ERROR("sourcepack_index_empty", "path=\"%s\"", path_.c_str());
    return 1;
  }
  const std::vector<std::string> names = split_tabs(header);
  for (size_t i = 0; i < names.size(); ++i) fields_[trim_ws(names[i])] = (int)i;
  static const char* required[] = {
      "timestamp",     "path_id",     "component_slot", "source_key",   "receiver_key",
      "src_id",        "rec_id",      "src_network",    "src_station",  "src_location",
      "src_component", "rec_network", "rec_station",    "rec_location", "rec_component",
      "npts",          "dt",          "dist",           "az",           "baz",
      "record_path",   "record_offset", "bytes",        "final_pair_path"};
  for (const char* f : required) {
    if (!fields_.count(f)) {
      FXLOG_ERROR("sourcepack_index_field_missing", "path=\"%s\" field=\"%s\"", path_.c_str(), f);
      return 1;
    }
  }
  return 0;
}

std::string SourcePackStream::value(const std::vector<std::string>& row, const char* name) const {
  auto it = fields_.find(name);
  if (it == fields_.end() || it->second < 0 || (size_t)it->second >= row.size()) return "";
  return trim_ws(row[(size_t)it->second]);
}

bool SourcePackStream::next(SourcePackRecord* r) {
  std::string line;
  while (std::getline(in_, line)) {
    if (line.empty()) continue;
    std::vector<std::string> row = split_tabs(line);
    if (row.size() < fields_.size()) row.resize(fields_.size());
    r->timestamp = value(row, "timestamp");
    r->path_id = value(row, "path_id");
    r->component_slot = atoi(value(row, "component_slot").c_str());
    r->source_key = value(row, "source_key");
    r->receiver_key = value(row, "receiver_key");
    r->src_id = value(row, "src_id");
    r->rec_id = value(row, "rec_id");
    r->src_network = value(row, "src_network");
    r->src_station = value(row, "src_station");
    r->src_location = value(row, "src_location");
    r->src_component = value(row, "src_component");
    r->rec_network = value(row, "rec_network");
    r->rec_station = value(row, "rec_station");
    r->rec_location = value(row, "rec_location");
    r->rec_component = value(row, "rec_component");
    r->dist = value(row, "dist");
    r->az = value(row, "az");
    r->baz = value(row, "baz");
    r->final_pair_path = value(row, "final_pair_path");
    r->record_path = value(row, "record_path");
    r->record_offset = strtoll(value(row, "record_offset").c_str(), nullptr, 10);
    r->record_bytes = strtoll(value(row, "bytes").c_str(), nullptr, 10);
    return true;
  }
  return false;
}

bool SourcePackGroupReader::Later::operator()(const Item& a, const Item& b) const {
  if (a.record.path_id != b.record.path_id) return a.record.path_id > b.record.path_id;
  if (a.record.component_slot != b.record.component_slot)
    return a.record.component_slot > b.record.component_slot;
  return a.seq > b.seq;
}

SourcePackGroupReader::~SourcePackGroupReader() {
  for (SourcePackStream* s : streams_) delete s;
}

void SourcePackGroupReader::push(const SourcePackRecord& r, size_t stream) {
  Item it;
  it.record = r;
  it.stream = stream;
  it.seq = seq_++;
  heap_.push(it);
}

int SourcePackGroupReader::open() {
  for (size_t i = 0; i < paths_.size(); ++i) {
    SourcePackStream* s = new SourcePackStream(paths_[i]);
    if (s->open() != 0) {
      delete s;
      return 1;
    }
    streams_.push_back(s);
    SourcePackRecord r;
    if (s->next(&r)) push(r, i);
  }
  return 0;
}

bool SourcePackGroupReader::next_group(std::vector<SourcePackRecord>* records) {
  records->clear();
  if (heap_.empty()) return false;
  const std::string pid = heap_.top().record.path_id;
  const int slot = heap_.top().record.component_slot;
  while (!heap_.empty() && heap_.top().record.path_id == pid &&
         heap_.top().record.component_slot == slot) {
    Item it = heap_.top();
    heap_.pop();
    records->push_back(it.record);
    SourcePackRecord nx;
    if (streams_[it.stream]->next(&nx)) push(nx, it.stream);
  }
  std::sort(records->begin(), records->end(),
            [](const SourcePackRecord& a, const SourcePackRecord& b) {
              if (a.timestamp != b.timestamp) return a.timestamp < b.timestamp;
              if (a.record_path != b.record_path) return a.record_path < b.record_path;
              return a.record_offset < b.record_offset;
            });
  return true;
}

size_t count_sourcepack_groups(const std::vector<std::string>& indexes) {
  SourcePackGroupReader rd(indexes);
  if (rd.open() != 0) return 0;
  std::vector<SourcePackRecord> g;
  size_t n = 0;
  while (rd.next_group(&g)) ++n;
  return n;
}

FILE* PackFileCache::get(const std::string& path) {
  auto it = files_.find(path);
  if (it != files_.end()) return it->second;
  if (files_.size() >= 256) close_all();
  FILE* fp = fopen(path.c_str(), "rb");
  if (!fp) {
    FXLOG_ERROR("sourcepack_record_open_failed", "path=\"%s\" error=\"%s\"", path.c_str(),
                strerror(errno));
    return nullptr;
  }
  files_[path] = fp;
  return fp;
}

void PackFileCache::close_all() {
  for (auto& kv : files_) fclose(kv.second);
  files_.clear();
}

unsigned sac_data_count(const SacHeader& hd) {
  const int npts = hd.i[SI_NPTS];
  return hd.i[SI_IFTYPE] == 4 ? (unsigned)(npts * 2) : (unsigned)npts;
}

int read_sourcepack_header(PackFileCache* cache, const SourcePackRecord& r, SacHeader* hd) {
  FILE* fp = cache->get(r.record_path);
  if (!fp) return 1;
  if (fseeko(fp, (off_t)r.record_offset, SEEK_SET) != 0 || fread(hd, sizeof(SacHeader), 1, fp) != 1) {
    FXLOG_ERROR("sourcepack_first_header_read_failed", "path=\"%s\"", r.record_path.c_str());
    return 1;
  }
  return 0;
}

int read_sourcepack_record(PackFileCache* cache, const SourcePackRecord& r, SacHeader* hd,
                           float* data, unsigned expected) {
  FILE* fp = cache->get(r.record_path);
  if (!fp) return 1;
  if (fseeko(fp, (off_t)r.record_offset, SEEK_SET) != 0) {
    FXLOG_ERROR("sourcepack_record_seek_failed", "path=\"%s\" offset=%lld", r.record_path.c_str(),
                r.record_offset);
    return 1;
  }
  if (fread(hd, sizeof(SacHeader), 1, fp) != 1) {
    FXLOG_ERROR("sourcepack_record_header_read_failed", "path=\"%s\"", r.record_path.c_str());
    return 1;
  }
  const unsigned n = sac_data_count(*hd);
  if (n != expected) {
    FXLOG_ERROR("sourcepack_record_sample_count_mismatch", "path=\"%s\" samples=%u expected_samples=%u",
                r.record_path.c_str(), n, expected);
    return 1;
  }
  const long long want = (long long)sizeof(SacHeader) + (long long)n * 4;
  if (r.record_bytes != want) {
    FXLOG_ERROR("sourcepack_record_size_mismatch", "path=\"%s\" record_bytes=%lld expected_bytes=%lld",
                r.record_path.c_str(), r.record_bytes, want);
    return 1;
  }
  if (fread(data, sizeof(float), n, fp) != n) {
    FXLOG_ERROR("sourcepack_record_data_read_failed", "path=\"%s\"", r.record_path.c_str());
    return 1;
  }
  return 0;
}

int StackShardWriter::open(const std::string& output_dir, const std::string& prefix, size_t worker) {
  dir_ = output_dir;
  prefix_ = prefix;
  char pn[64], in[64];
  snprintf(pn, sizeof(pn), "%s.w%03zu.pack", prefix.c_str(), worker);
  snprintf(in, sizeof(in), "%s.w%03zu.tsv", prefix.c_str(), worker);
  pack_path_ = join_path(dir_, pn);
  index_path_ = join_path(dir_, in);
  if (mkdir_p(dir_) != 0) {
    FXLOG_ERROR("stack_output_dir_create_failed", "path=\"%s\" error=\"%s\"", dir_.c_str(), strerror(errno));
    return 1;
  }
  pack_ = fopen(pack_path_.c_str(), "wb");
  if (!pack_) {
    FXLOG_ERROR("stack_pack_open_failed", "path=\"%s\" error=\"%s\"", pack_path_.c_str(), strerror(errno));
    return 1;
  }
  index_.open(index_path_.c_str());
  if (!index_) {
    FXLOG_ERROR("stack_shard_index_open_failed", "path=\"%s\"", index_path_.c_str());
    close();
    return 1;
  }
  index_ << sourcepack_index_header() << '\n';
  return 0;
}

std::string StackShardWriter::final_pair_path(const SourcePackRecord& r) const {
  std::string p = r.final_pair_path;
  if (p.empty())
    p = r.src_network + "-" + r.rec_network + "." + r.src_station + "-" + r.rec_station + "." +
        r.src_component + "-" + r.rec_component;
  const std::string sfx = ".sac", rep = "." + prefix_ + ".sac";
  const size_t pos = p.rfind(sfx);
  if (pos != std::string::npos && pos + sfx.size() == p.size())
    p.replace(pos, sfx.size(), rep);
  else
    p += rep;
  return p;
}

int StackShardWriter::append(const SourcePackRecord& r, const SacHeader& hd, const float* data) {
  if (!pack_ || !index_) return 1;
  const long long off = (long long)ftello(pack_);
  if (off < 0) {
    FXLOG_ERROR("stack_pack_tell_failed", "path=\"%s\" error=\"%s\"", pack_path_.c_str(), strerror(errno));
    return 1;
  }
  const unsigned n = sac_data_count(hd);
  if (fwrite(&hd, sizeof(SacHeader), 1, pack_) != 1 || fwrite(data, sizeof(float), n, pack_) != n) {
    FXLOG_ERROR("stack_pack_write_failed", "path=\"%s\"", pack_path_.c_str());
    return 1;
  }
  const long long bytes = (long long)sizeof(SacHeader) + (long long)n * 4;
  index_ << "STACK" << '\t' << r.path_id << '\t' << r.component_slot << '\t' << r.source_key << '\t'
         << r.receiver_key << '\t' << r.src_id << '\t' << r.rec_id << '\t' << r.src_network << '\t'
         << r.src_station << '\t' << r.src_location << '\t' << r.src_component << '\t'
         << r.rec_network << '\t' << r.rec_station << '\t' << r.rec_location << '\t'
         << r.rec_component << '\t' << hd.i[SI_NPTS] << '\t' << hd.f[SF_DELTA] << '\t' << r.dist
         << '\t' << r.az << '\t' << r.baz << '\t' << pack_path_ << '\t' << off << '\t' << bytes
         << '\t' << prefix_ << "_pack" << '\t' << final_pair_path(r) << '\n';
  return index_ ? 0 : 1;
}

int StackShardWriter::close() {
  int rc = 0;
  if (pack_) {
    if (fclose(pack_) != 0) rc = 1;
    pack_ = nullptr;
  }
  if (index_.is_open()) index_.close();
  return rc;
}

int merge_shard_indexes(const std::string& output_dir, const std::string& prefix, size_t workers,
                        const std::string& final_index) {
  struct Row {
    std::string path_id, line;
    int slot;
    size_t worker, seq;
  };
  std::vector<Row> rows;
  for (size_t w = 0; w < workers; ++w) {
    char name[64];
    snprintf(name, sizeof(name), "%s.w%03zu.tsv", prefix.c_str(), w);
    const std::string sp = join_path(output_dir, name);
    std::ifstream in(sp.c_str());
    if (!in) {
      FXLOG_ERROR("stack_shard_index_read_failed", "path=\"%s\"", sp.c_str());
      return 1;
    }
    std::string line;
    if (!std::getline(in, line)) continue;
    size_t seq = 0;
    while (std::getline(in, line)) {
      line = trim_ws(line);
      if (line.empty()) continue;
      const std::vector<std::string> f = split_tabs(line);
      if (f.size() < 3) {
        FXLOG_ERROR("stack_shard_index_row_malformed", "path=\"%s\"", sp.c_str());
        return 1;
      }
      rows.push_back(Row{trim_ws(f[1]), line, atoi(trim_ws(f[2]).c_str()), w, seq++});
    }
  }
  std::sort(rows.begin(), rows.end(), [](const Row& a, const Row& b) {
    if (a.path_id != b.path_id) return a.path_id < b.path_id;
    if (a.slot != b.slot) return a.slot < b.slot;
    if (a.worker != b.worker) return a.worker < b.worker;
    return a.seq < b.seq;
  });
  std::ofstream out(final_index.c_str());
  if (!out) {
    FXLOG_ERROR("stack_final_index_open_failed", "path=\"%s\"", final_index.c_str());
    return 1;
  }
  out << sourcepack_index_header() << '\n';
  for (const Row& r : rows) out << r.line << '\n';
  return out ? 0 : 1;
}

int write_stack_success(const std::string& output_dir, const std::string& prefix, size_t records,
                        size_t workers, const std::string& index_path) {
  const std::string p = join_path(output_dir, "_SUCCESS");
  std::ofstream s(p.c_str());
  if (!s) {
    FXLOG_ERROR("success_marker_open_failed", "path=\"%s\"", p.c_str());
    return 1;
  }
  s << "records\t" << records << "\n"
    << "workers\t" << workers << "\n"
    << "index\t" << index_path << "\n";
  for (size_t w = 0; w < workers; ++w) {
    char name[64];
    snprintf(name, sizeof(name), "%s.w%03zu.pack", prefix.c_str(), w);
    s << "pack\t" << join_path(output_dir, name) << "\n";
  }
  return s ? 0 : 1;
}

}  // namespace fxcio
