// SourcePack index emission over xc_fast's xcpack output (host code).
//
// A SourcePack index lists, per timestamp, where each NCF record lives inside
// the xcpack files (file, byte offset, size) together with its pair metadata,
// ordered so that all records of one station pair and component slot are
// adjacent. No NCF bytes move: the xcpack files stay the storage.
//
// Output contract (what readers of the index depend on, kept identical to
// fastxc/operators/sourcepack/builder.py:163-436 and
// fastxc/io/sourcepack.py:30-56,118-150 of the reference):
//   <out>/<safe ts>/sourcepack_index.tsv  25 tab-separated columns, CRLF rows,
//                                         minimal quoting
//   <out>/<safe ts>/_SUCCESS              timestamp/records/sources/bytes_indexed
//   <out>/_SUCCESS (async finish only)    timestamps/records/sources/bytes_indexed
//   progress sidecar                      task status completed total unit detail
// Row order with sorting on: (path id text, component slot, source key,
// receiver key, input sequence), the sequence numbering the rows of the TSVs
// read in file-name order. A timestamp's folder is written under a
// dot-prefixed temporary name and renamed into place.
//
// Design: one pass over the TSV text builds compact records (the 25 output
// fields are computed once, at parse time), a stable sort on a precomputed
// key orders them, and one buffered write emits each index. The same
// routine serves three callers: the whole-output build, the per-timestamp
// build, and xc_fast itself, which indexes each timestamp right after
// writing its `.done` marker; a polling thread (fxc_sourcepack_async_*)
// covers pipelines that run the materializer beside an external xc_fast.

#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <map>
#include <mutex>
#include <set>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "fastxc_gb300.h"

namespace fxc {
void set_error(const char* fmt, ...);
}
using fxc::set_error;

namespace fs = std::filesystem;

namespace {

// ---- small text helpers -----------------------------------------------------

// One TSV line split into fields with the quoting rules of a CSV dialect
// whose delimiter is a tab: a field that starts with '"' runs to the closing
// quote, and "" inside it is one quote character.
std::vector<std::string> split_tsv(const std::string& line) {
  std::vector<std::string> out;
  std::string cur;
  size_t i = 0;
  const size_t n = line.size();
  bool field_start = true;
  bool quoted = false;
  while (i < n) {
    char c = line[i];
    if (quoted) {
      if (c == '"') {
        if (i + 1 < n && line[i + 1] == '"') {
          cur.push_back('"');
          i += 2;
          continue;
        }
        quoted = false;
        ++i;
        continue;
      }
      cur.push_back(c);
      ++i;
      continue;
    }
    if (field_start && c == '"') {
      quoted = true;
      field_start = false;
      ++i;
      continue;
    }
    if (c == '\t') {
      out.push_back(cur);
      cur.clear();
      field_start = true;
      ++i;
      continue;
    }
    cur.push_back(c);
    field_start = false;
    ++i;
  }
  out.push_back(cur);
  return out;
}

// A field as a minimally quoted TSV cell: quoted only when it holds a tab, a
// quote or a line break.
void put_cell(std::string& out, const std::string& v) {
  if (v.find_first_of("\t\"\r\n") == std::string::npos) {
    out += v;
    return;
  }
  out.push_back('"');
  for (char c : v) {
    if (c == '"') out.push_back('"');
    out.push_back(c);
  }
  out.push_back('"');
}

std::string strip(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && isspace((unsigned char)s[a])) ++a;
  while (b > a && isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

bool all_digits(const std::string& s) {
  if (s.empty()) return false;
  for (char c : s)
    if (c < '0' || c > '9') return false;
  return true;
}

// Whole-string integer (surrounding blanks allowed); false on anything else.
bool parse_int(const std::string& s, long long* v) {
  std::string t = strip(s);
  if (t.empty()) return false;
  size_t i = (t[0] == '+' || t[0] == '-') ? 1 : 0;
  if (i == t.size()) return false;
  for (size_t k = i; k < t.size(); ++k)
    if (t[k] < '0' || t[k] > '9') return false;
  errno = 0;
  *v = strtoll(t.c_str(), nullptr, 10);
  return errno == 0;
}

// Folder name of a timestamp: runs of characters outside [0-9A-Za-z._:-]
// become one '-', leading and trailing '-' are dropped, "" becomes "item".
std::string safe_name(const std::string& ts) {
  std::string out;
  bool in_run = false;
  for (char c : ts) {
    const bool ok = isalnum((unsigned char)c) || c == '.' || c == '_' || c == ':' || c == '-';
    if (ok && (unsigned char)c < 0x80) {
      out.push_back(c);
      in_run = false;
    } else if (!in_run) {
      out.push_back('-');
      in_run = true;
    }
  }
  size_t a = out.find_first_not_of('-');
  if (a == std::string::npos) return "item";
  size_t b = out.find_last_not_of('-');
  return out.substr(a, b - a + 1);
}

// Component rank of the pair slot: the last character of the component code,
// E/1 -> 0, N/2 -> 1, Z/3 -> 2, R -> 3, T -> 4, anything else 100.
int component_rank(const std::string& comp) {
  if (comp.empty()) return 100;
  switch (toupper((unsigned char)comp.back())) {
    case 'E': case '1': return 0;
    case 'N': case '2': return 1;
    case 'Z': case '3': return 2;
    case 'R': return 3;
    case 'T': return 4;
    default: return 100;
  }
}

// ---- paths --------------------------------------------------------------------

std::string expand_user(const std::string& p) {
  if (p.empty() || p[0] != '~') return p;
  if (p.size() > 1 && p[1] != '/') return p;  // ~user is left to the shell
  const char* home = getenv("HOME");
  return std::string(home ? home : "") + p.substr(1);
}

// Lexical normal form of a POSIX path: repeated separators and "." parts
// removed, no trailing separator, ".." kept (as pure path arithmetic does).
std::string lexical_norm(const std::string& p) {
  if (p.empty()) return ".";
  std::string lead;
  size_t i = 0;
  if (p[0] == '/') {
    lead = (p.size() > 1 && p[1] == '/' && (p.size() == 2 || p[2] != '/')) ? "//" : "/";
    while (i < p.size() && p[i] == '/') ++i;
  }
  std::vector<std::string> parts;
  while (i < p.size()) {
    size_t j = p.find('/', i);
    if (j == std::string::npos) j = p.size();
    std::string part = p.substr(i, j - i);
    if (!part.empty() && part != ".") parts.push_back(part);
    i = j + 1;
  }
  std::string out = lead;
  for (size_t k = 0; k < parts.size(); ++k) {
    if (k) out.push_back('/');
    out += parts[k];
  }
  return out.empty() ? "." : out;
}

// Absolute, symlink-resolved path that need not exist yet (the existing
// prefix is resolved, the rest appended).
std::string resolve_path(const std::string& p) {
  std::error_code ec;
  fs::path a = fs::absolute(fs::path(expand_user(p)), ec);
  if (ec) return lexical_norm(p);
  fs::path r = fs::weakly_canonical(a, ec);
  if (ec) return lexical_norm(a.string());
  return lexical_norm(r.string());
}

bool is_dir(const std::string& p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

bool is_file(const std::string& p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

std::string parent_of(const std::string& p) {
  size_t k = p.find_last_of('/');
  if (k == std::string::npos) return ".";
  if (k == 0) return "/";
  return p.substr(0, k);
}

std::string base_of(const std::string& p) {
  size_t k = p.find_last_of('/');
  return k == std::string::npos ? p : p.substr(k + 1);
}

// Names in `dir` ending with `suffix`, in byte order.
std::vector<std::string> names_with_suffix(const std::string& dir, const char* suffix) {
  std::vector<std::string> out;
  std::error_code ec;
  const size_t sl = strlen(suffix);
  for (fs::directory_iterator it(dir, ec), end; !ec && it != end; it.increment(ec)) {
    std::string n = it->path().filename().string();
    if (n.size() >= sl && n.compare(n.size() - sl, sl, suffix) == 0) out.push_back(n);
  }
  std::sort(out.begin(), out.end());
  return out;
}

bool read_text(const std::string& path, std::string* out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  *out = ss.str();
  if (out->size() >= 3 && (unsigned char)(*out)[0] == 0xEF && (unsigned char)(*out)[1] == 0xBB &&
      (unsigned char)(*out)[2] == 0xBF)
    out->erase(0, 3);
  return true;
}

// Lines of a text file with "\n", "\r\n" or "\r" endings.
std::vector<std::string> lines_of(const std::string& text) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < text.size()) {
    size_t j = text.find_first_of("\r\n", i);
    if (j == std::string::npos) {
      out.push_back(text.substr(i));
      break;
    }
    out.push_back(text.substr(i, j - i));
    i = j + 1;
    if (text[j] == '\r' && i < text.size() && text[i] == '\n') ++i;
  }
  return out;
}

bool write_file(const std::string& path, const std::string& data) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return false;
  const bool ok = fwrite(data.data(), 1, data.size(), f) == data.size();
  return (fclose(f) == 0) && ok;
}

// ---- records ------------------------------------------------------------------

enum Err { OK = 0, NOT_FOUND = 1, BAD_FORMAT = 2, IO = 3 };

const char* const kIndexHeader[25] = {
    "timestamp", "path_id", "component_slot", "source_key", "receiver_key", "src_id", "rec_id",
    "src_network", "src_station", "src_location", "src_component", "rec_network", "rec_station",
    "rec_location", "rec_component", "npts", "dt", "dist", "az", "baz", "record_path", "record_offset",
    "bytes", "storage_kind", "final_pair_path"};

// xcpack TSV columns the index needs
const char* const kRequired[] = {"timestamp", "pack_path", "offset", "bytes", "src_id", "rec_id",
                                 "src_network", "src_station", "src_location", "src_component",
                                 "rec_network", "rec_station", "rec_location", "rec_component",
                                 "npts", "dt", "dist", "az", "baz"};

struct Record {
  std::string timestamp;
  std::string cells;  // the index row, already joined and terminated
  std::string path_id, source_key, receiver_key;
  int slot = 0;
  int64_t bytes = 0;
  size_t seq = 0;
};

struct Failure {
  Err code = OK;
  std::string msg;
};

// Records of one xcpack TSV; `seq` numbers them on from its current value.
// `want_ts` (non-null) keeps only that timestamp's rows (they still consume
// sequence numbers).
Err read_tsv(const std::string& tsv, size_t* seq, const std::string* want_ts, std::vector<Record>* out,
             Failure* fail) {
  std::string text;
  if (!read_text(tsv, &text)) {
    fail->msg = "cannot read xcpack TSV " + tsv;
    return fail->code = IO;
  }
  std::vector<std::string> lines = lines_of(text);
  size_t li = 0;
  while (li < lines.size() && lines[li].empty()) ++li;
  if (li == lines.size()) return OK;  // no header: no rows
  std::vector<std::string> head = split_tsv(lines[li++]);
  std::unordered_map<std::string, size_t> col;
  for (size_t k = 0; k < head.size(); ++k) col[head[k]] = k;  // a repeated name: its last column
  std::string missing;
  for (const char* r : kRequired)
    if (!col.count(r)) missing += std::string(missing.empty() ? "" : ", ") + r;
  if (!missing.empty()) {
    fail->msg = "xcpack TSV " + tsv + " lacks the missing fields " + missing;
    return fail->code = BAD_FORMAT;
  }
  const std::string tsv_dir = parent_of(tsv);
  std::unordered_map<std::string, std::string> pack_cache;
  auto field = [&](const std::vector<std::string>& f, const char* name) -> std::string {
    auto it = col.find(name);
    if (it == col.end() || it->second >= f.size()) return std::string();
    return f[it->second];
  };
  for (; li < lines.size(); ++li) {
    if (lines[li].empty()) continue;
    std::vector<std::string> f = split_tsv(lines[li]);
    const std::string ptxt = field(f, "pack_path");
    auto pc = pack_cache.find(ptxt);
    if (pc == pack_cache.end()) {
      std::string p = expand_user(ptxt);
      if (p.empty() || p[0] != '/') p = tsv_dir + "/" + p;
      p = lexical_norm(p);
      if (!is_file(p)) {
        fail->msg = "xcpack TSV " + tsv + " points at a pack file that does not exist: " + p;
        return fail->code = NOT_FOUND;
      }
      pc = pack_cache.emplace(ptxt, p).first;
    }
    long long off = 0, nb = 0;
    if (!parse_int(field(f, "offset"), &off) || !parse_int(field(f, "bytes"), &nb)) {
      fail->msg = "xcpack TSV " + tsv + ": row " + std::to_string(li + 1) + " has a non-integer offset or size";
      return fail->code = BAD_FORMAT;
    }
    if (off < 0 || nb <= 0) {
      fail->msg = "xcpack TSV " + tsv + ": row " + std::to_string(li + 1) + " has offset < 0 or size <= 0";
      return fail->code = BAD_FORMAT;
    }
    const size_t my_seq = (*seq)++;
    const std::string ts = field(f, "timestamp");
    if (want_ts && ts != *want_ts) continue;
    Record r;
    r.timestamp = ts;
    r.seq = my_seq;
    r.bytes = nb;
    r.source_key = field(f, "src_network") + "." + field(f, "src_station") + "." + field(f, "src_location");
    r.receiver_key = field(f, "rec_network") + "." + field(f, "rec_station") + "." + field(f, "rec_location");
    r.slot = component_rank(field(f, "src_component")) * 3 + component_rank(field(f, "rec_component"));
    const std::string pid = strip(field(f, "path_id"));
    if (!pid.empty()) {
      r.path_id = all_digits(pid) && pid.size() < 8 ? std::string(8 - pid.size(), '0') + pid : pid;
    } else {
      long long s = 0, q = 0;
      if (!parse_int(field(f, "src_id"), &s) || !parse_int(field(f, "rec_id"), &q)) {
        fail->msg = "xcpack TSV " + tsv + ": row " + std::to_string(li + 1) + " has no path_id and non-integer ids";
        return fail->code = BAD_FORMAT;
      }
      char buf[32];
      snprintf(buf, sizeof buf, "%08lld", s * 10000 + q);
      r.path_id = buf;
    }
    const std::string vals[25] = {
        ts, r.path_id, std::to_string(r.slot), r.source_key, r.receiver_key, field(f, "src_id"),
        field(f, "rec_id"), field(f, "src_network"), field(f, "src_station"), field(f, "src_location"),
        field(f, "src_component"), field(f, "rec_network"), field(f, "rec_station"), field(f, "rec_location"),
        field(f, "rec_component"), field(f, "npts"), field(f, "dt"), field(f, "dist"), field(f, "az"),
        field(f, "baz"), pc->second, std::to_string(off), std::to_string(nb), "xcpack", field(f, "final_pair_path")};
    for (int k = 0; k < 25; ++k) {
      if (k) r.cells.push_back('\t');
      put_cell(r.cells, vals[k]);
    }
    r.cells += "\r\n";
    out->push_back(std::move(r));
  }
  return OK;
}

struct Totals {
  int64_t timestamps = 0, records = 0, sources = 0, bytes = 0;
};

// Writes one timestamp's folder from its records (any order on input).
Err emit_timestamp(const std::string& ts, std::vector<Record> recs, const std::string& out_dir, bool sorted,
                   Totals* t, Failure* fail) {
  const std::string name = safe_name(ts);
  const std::string target = out_dir + "/" + name;
  const std::string tmp = out_dir + "/." + name + ".tmp";
  std::error_code ec;
  fs::remove_all(tmp, ec);
  fs::create_directories(tmp, ec);
  if (ec) {
    fail->msg = "cannot create " + tmp + ": " + ec.message();
    return fail->code = IO;
  }
  if (sorted) {
    std::stable_sort(recs.begin(), recs.end(), [](const Record& a, const Record& b) {
      if (a.path_id != b.path_id) return a.path_id < b.path_id;
      if (a.slot != b.slot) return a.slot < b.slot;
      if (a.source_key != b.source_key) return a.source_key < b.source_key;
      if (a.receiver_key != b.receiver_key) return a.receiver_key < b.receiver_key;
      return a.seq < b.seq;
    });
  } else {
    std::stable_sort(recs.begin(), recs.end(), [](const Record& a, const Record& b) { return a.seq < b.seq; });
  }
  std::string body;
  for (int k = 0; k < 25; ++k) {
    if (k) body.push_back('\t');
    body += kIndexHeader[k];
  }
  body += "\r\n";
  std::set<std::string> sources;
  int64_t nbytes = 0;
  for (const Record& r : recs) {
    body += r.cells;
    sources.insert(r.source_key);
    nbytes += r.bytes;
  }
  const std::string ok = "timestamp\t" + ts + "\nrecords\t" + std::to_string(recs.size()) + "\nsources\t" +
                         std::to_string(sources.size()) + "\nbytes_indexed\t" + std::to_string(nbytes) + "\n";
  if (!write_file(tmp + "/sourcepack_index.tsv", body) || !write_file(tmp + "/_SUCCESS", ok)) {
    fail->msg = "cannot write the index files under " + tmp;
    return fail->code = IO;
  }
  fs::remove_all(target, ec);
  fs::rename(tmp, target, ec);
  if (ec) {
    fail->msg = "cannot move " + tmp + " to " + target + ": " + ec.message();
    return fail->code = IO;
  }
  t->timestamps += 1;
  t->records += (int64_t)recs.size();
  t->sources += (int64_t)sources.size();
  t->bytes += nbytes;
  return OK;
}

// The xcpack folder of an xc output root: the root itself when it is named
// "xcpack", else <root>/xcpack.
Err find_xcpack(const char* root, std::string* dir, Failure* fail) {
  if (!root || !*root) {
    fail->msg = "no xc output folder given";
    return fail->code = NOT_FOUND;
  }
  const std::string r = resolve_path(root);
  const std::string cand = base_of(r) == "xcpack" ? r : r + "/xcpack";
  if (!is_dir(cand)) {
    fail->msg = "no xcpack folder at " + r + " (looked for " + cand + ")";
    return fail->code = NOT_FOUND;
  }
  *dir = cand;
  return OK;
}

// Timestamps a workspace lists in manifest/timestamp_index.tsv (the
// workspace is the xcpack folder's parent, or its grandparent under "ncf").
std::vector<std::string> inventory_timestamps(const std::string& xcpack_dir) {
  const std::string parent = parent_of(xcpack_dir);
  const std::string ws = base_of(parent) == "ncf" ? parent_of(parent) : parent;
  std::string text;
  std::set<std::string> out;
  if (!is_file(ws + "/manifest/timestamp_index.tsv") || !read_text(ws + "/manifest/timestamp_index.tsv", &text))
    return {};
  std::vector<std::string> lines = lines_of(text);
  size_t li = 0;
  while (li < lines.size() && lines[li].empty()) ++li;
  if (li == lines.size()) return {};
  std::vector<std::string> head = split_tsv(lines[li++]);
  size_t c = std::find(head.begin(), head.end(), std::string("timestamp")) - head.begin();
  if (c == head.size()) return {};
  for (; li < lines.size(); ++li) {
    if (lines[li].empty()) continue;
    std::vector<std::string> f = split_tsv(lines[li]);
    if (c < f.size()) {
      std::string ts = strip(f[c]);
      if (!ts.empty()) out.insert(ts);
    }
  }
  return std::vector<std::string>(out.begin(), out.end());
}

std::vector<std::string> done_timestamps(const std::string& xcpack_dir) {
  std::vector<std::string> out;
  for (const std::string& n : names_with_suffix(xcpack_dir, ".done"))
    if (n[0] != '_') out.push_back(n.substr(0, n.size() - 5));
  return out;
}

void write_progress(const char* file, const char* status, int64_t done, int64_t total, const std::string& detail) {
  if (!file || !*file) return;
  const std::string p = resolve_path(file);
  std::error_code ec;
  fs::create_directories(parent_of(p), ec);
  auto clean = [](std::string s) {
    for (char& c : s)
      if (c == '\t' || c == '\r' || c == '\n') c = ' ';
    return s;
  };
  const std::string body = "task\tstatus\tcompleted\ttotal\tunit\tdetail\noverall\t" + clean(status) + "\t" +
                           std::to_string(done) + "\t" + std::to_string(total) + "\ttimestamps\t" + clean(detail) +
                           "\n";
  const std::string tmp = p + ".tmp";
  if (write_file(tmp, body)) fs::rename(tmp, p, ec);
}

int status_of(Err e) { return e == NOT_FOUND ? FXC_ERR_NOTFOUND : e == BAD_FORMAT ? FXC_ERR_IO : FXC_ERR_IO; }

// Index one timestamp from the TSVs whose names start with it (all TSVs when
// none does); sequence numbers run over those files only.
Err index_one(const std::string& xcpack_dir, const std::string& out_dir, const std::string& ts, bool sorted,
              Totals* t, Failure* fail) {
  std::vector<std::string> all = names_with_suffix(xcpack_dir, ".tsv");
  std::vector<std::string> mine;
  for (const std::string& n : all)
    if (n.compare(0, ts.size(), ts) == 0) mine.push_back(n);
  if (mine.empty()) mine = all;
  std::vector<Record> recs;
  size_t seq = 0;
  for (const std::string& n : mine) {
    Err e = read_tsv(xcpack_dir + "/" + n, &seq, &ts, &recs, fail);
    if (e != OK) return e;
  }
  return emit_timestamp(ts, std::move(recs), out_dir, sorted, t, fail);
}

}  // namespace

// ---- C ABI ----------------------------------------------------------------------

extern "C" int fxc_sourcepack_build(const char* xc_root, const char* out_dir, const char* timestamp,
                                    int sort_within_source, const char* progress_file, fxc_sourcepack_totals* out,
                                    char* out_path, size_t out_path_cap, char* names, size_t names_cap) {
  Failure fail;
  std::string xdir;
  if (find_xcpack(xc_root, &xdir, &fail) != OK) {
    set_error("%s", fail.msg.c_str());
    return status_of(fail.code);
  }
  if (timestamp && !(out_dir && *out_dir)) {
    set_error("a single-timestamp build needs an output folder");
    return FXC_ERR_INVALID;
  }
  const std::string odir = (out_dir && *out_dir) ? resolve_path(out_dir) : parent_of(xdir) + "/sourcepack";
  std::error_code ec;
  fs::create_directories(odir, ec);
  if (ec) {
    set_error("cannot create %s: %s", odir.c_str(), ec.message().c_str());
    return FXC_ERR_IO;
  }
  Totals t;
  std::string folders;  // indexed timestamp folders, one per line
  if (timestamp) {
    folders = safe_name(timestamp) + "\n";
    if (index_one(xdir, odir, timestamp, sort_within_source != 0, &t, &fail) != OK) {
      set_error("%s", fail.msg.c_str());
      return status_of(fail.code);
    }
  } else {
    std::map<std::string, std::vector<Record>> by_ts;
    std::vector<Record> recs;
    size_t seq = 0;
    for (const std::string& n : names_with_suffix(xdir, ".tsv")) {
      if (read_tsv(xdir + "/" + n, &seq, nullptr, &recs, &fail) != OK) {
        set_error("%s", fail.msg.c_str());
        return status_of(fail.code);
      }
    }
    for (Record& r : recs) by_ts[r.timestamp].push_back(std::move(r));
    std::set<std::string> stamps;
    for (auto& kv : by_ts) stamps.insert(kv.first);
    for (const std::string& s : inventory_timestamps(xdir)) stamps.insert(s);
    for (const std::string& s : done_timestamps(xdir)) stamps.insert(s);
    if (stamps.empty()) {
      set_error("the xcpack folder %s holds no timestamps", xdir.c_str());
      return FXC_ERR_NOTFOUND;
    }
    const int64_t total = (int64_t)stamps.size();
    write_progress(progress_file, "RUNNING", 0, total, "source index build");
    int64_t k = 0;
    for (const std::string& s : stamps) {
      auto it = by_ts.find(s);
      std::vector<Record> mine = it == by_ts.end() ? std::vector<Record>() : std::move(it->second);
      const int64_t before = t.records;
      if (emit_timestamp(s, std::move(mine), odir, sort_within_source != 0, &t, &fail) != OK) {
        set_error("%s", fail.msg.c_str());
        return status_of(fail.code);
      }
      write_progress(progress_file, "RUNNING", ++k, total, s + ": " + std::to_string(t.records - before) + " records");
      folders += safe_name(s) + "\n";
    }
    write_progress(progress_file, "DONE", total, total, "source index ready");
  }
  if (out) {
    out->timestamps = t.timestamps;
    out->records = t.records;
    out->sources = t.sources;
    out->bytes_indexed = t.bytes;
  }
  if (out_path && out_path_cap) snprintf(out_path, out_path_cap, "%s", odir.c_str());
  if (names && names_cap) snprintf(names, names_cap, "%s", folders.c_str());
  return FXC_OK;
}

// ---- polling materializer -----------------------------------------------------------

struct fxc_sourcepack_async {
  std::string xdir, odir, progress;
  bool sorted = true;
  double poll_s = 5.0;
  int64_t expected = 0;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;
  bool stop = false;
  std::set<std::string> done;
  Totals t;
  std::string error;
  Err error_code = OK;

  // indexes every timestamp with a .done marker not indexed yet
  Err scan() {
    if (!is_dir(xdir)) return OK;
    for (const std::string& ts : done_timestamps(xdir)) {
      {
        std::lock_guard<std::mutex> g(mu);
        if (done.count(ts)) continue;
      }
      Totals one;
      Failure f;
      if (index_one(xdir, odir, ts, sorted, &one, &f) != OK) {
        std::lock_guard<std::mutex> g(mu);
        error = f.msg;
        error_code = f.code;
        return f.code;
      }
      int64_t n;
      {
        std::lock_guard<std::mutex> g(mu);
        done.insert(ts);
        t.records += one.records;
        t.sources += one.sources;
        t.bytes += one.bytes;
        n = (int64_t)done.size();
      }
      write_progress(progress.c_str(), "RUNNING", n, expected, ts + ": " + std::to_string(one.records) + " records");
    }
    return OK;
  }

  void run() {
    std::unique_lock<std::mutex> lk(mu);
    while (!stop) {
      lk.unlock();
      const Err e = scan();
      lk.lock();
      if (e != OK) return;
      cv.wait_for(lk, std::chrono::duration<double>(poll_s), [this] { return stop; });
    }
  }
};

extern "C" int fxc_sourcepack_async_start(const char* xc_root, const char* out_dir, int sort_within_source,
                                          const char* progress_file, double poll_interval_s,
                                          fxc_sourcepack_async** out) {
  if (!out || !out_dir || !*out_dir || !xc_root) {
    set_error("fxc_sourcepack_async_start: xc root, output folder and handle are required");
    return FXC_ERR_INVALID;
  }
  auto* a = new fxc_sourcepack_async();
  const std::string r = resolve_path(xc_root);
  a->xdir = base_of(r) == "xcpack" ? r : r + "/xcpack";
  a->odir = resolve_path(out_dir);
  a->progress = progress_file ? progress_file : "";
  a->sorted = sort_within_source != 0;
  a->poll_s = std::max(0.5, poll_interval_s);
  std::vector<std::string> inv = inventory_timestamps(a->xdir);
  a->expected = !inv.empty() ? (int64_t)inv.size() : is_dir(a->xdir) ? (int64_t)done_timestamps(a->xdir).size() : 0;
  std::error_code ec;
  fs::create_directories(a->odir, ec);
  if (ec) {
    set_error("cannot create %s: %s", a->odir.c_str(), ec.message().c_str());
    delete a;
    return FXC_ERR_IO;
  }
  write_progress(a->progress.c_str(), "RUNNING", 0, a->expected, "async source index build");
  a->th = std::thread([a] { a->run(); });
  *out = a;
  return FXC_OK;
}

extern "C" int fxc_sourcepack_async_finish(fxc_sourcepack_async* a, int mark_success, const char* status_message,
                                           fxc_sourcepack_totals* out) {
  if (!a) {
    set_error("fxc_sourcepack_async_finish: null handle");
    return FXC_ERR_INVALID;
  }
  {
    std::lock_guard<std::mutex> g(a->mu);
    a->stop = true;
  }
  a->cv.notify_all();
  if (a->th.joinable()) a->th.join();
  if (a->error_code == OK) a->scan();
  std::vector<std::string> dirs;
  std::error_code ec;
  for (fs::directory_iterator it(a->odir, ec), end; !ec && it != end; it.increment(ec)) {
    if (is_file(it->path().string() + "/sourcepack_index.tsv")) dirs.push_back(it->path().filename().string());
  }
  const int64_t npaths = (int64_t)dirs.size();
  const int64_t total = a->expected ? a->expected : npaths;
  int rc = FXC_OK;
  if (a->error_code != OK) {
    write_progress(a->progress.c_str(), "FAILED", (int64_t)a->done.size(), a->expected, a->error);
    set_error("asynchronous SourcePack indexing failed: %s", a->error.c_str());
    rc = status_of(a->error_code);
  } else if (mark_success) {
    const std::string ok = "timestamps\t" + std::to_string(npaths) + "\nrecords\t" + std::to_string(a->t.records) +
                           "\nsources\t" + std::to_string(a->t.sources) + "\nbytes_indexed\t" +
                           std::to_string(a->t.bytes) + "\n";
    if (!write_file(a->odir + "/_SUCCESS", ok)) {
      set_error("cannot write %s/_SUCCESS", a->odir.c_str());
      rc = FXC_ERR_IO;
    }
    write_progress(a->progress.c_str(), "DONE", npaths, total, "source index ready");
  } else {
    fs::remove(a->odir + "/_SUCCESS", ec);
    write_progress(a->progress.c_str(), "FAILED", npaths, total,
                   status_message && *status_message ? status_message
                                                     : "upstream XC did not complete; global success marker withheld");
  }
  if (out) {
    out->timestamps = npaths;
    out->records = a->t.records;
    out->sources = a->t.sources;
    out->bytes_indexed = a->t.bytes;
  }
  delete a;
  return rc;
}
