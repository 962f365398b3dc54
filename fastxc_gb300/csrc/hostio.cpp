// Host-side formats and scheduling of the drop-in executables (see hostio.h).
#include "hostio.h"

#include <dirent.h>
#include <errno.h>
#include <fcntl.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <map>

namespace fxcio {

// ---------------------------------------------------------------------------
// logging: "LEVEL event=<e> file=<f> line=<n> k=v ..." on stderr, level from
// FASTXC_LOG_LEVEL (error|warn|info|debug)
// ---------------------------------------------------------------------------

static int g_level = -1;

static int log_level() {
  if (g_level < 0) {
    g_level = LOG_INFO;
    const char* v = getenv("FASTXC_LOG_LEVEL");
    if (v) {
      if (!strcasecmp(v, "error")) g_level = LOG_ERROR;
      else if (!strcasecmp(v, "warn") || !strcasecmp(v, "warning")) g_level = LOG_WARN;
      else if (!strcasecmp(v, "info")) g_level = LOG_INFO;
      else if (!strcasecmp(v, "debug")) g_level = LOG_DEBUG;
    }
  }
  return g_level;
}

void log_msg(LogLevel lvl, const char* event, const char* file, int line, const char* fmt, ...) {
  if ((int)lvl > log_level()) return;
  static const char* names[] = {"ERROR", "WARN", "INFO", "DEBUG"};
  flockfile(stderr);
  fprintf(stderr, "%s event=%s file=%s line=%d ", names[lvl], event ? event : "unknown",
          file ? file : "unknown", line);
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  fputc('\n', stderr);
  fflush(stderr);
  funlockfile(stderr);
}

static std::string clean_field(const std::string& s) {
  std::string o = s;
  for (char& c : o)
    if (c == '\t' || c == '\n' || c == '\r') c = ' ';
  return o;
}

std::string tsv_clean(const std::string& s) { return clean_field(s); }

void Progress::init(const char* p, const char* task_name, size_t tot, const char* unit_name) {
  path = (p && strcmp(p, "NONE") != 0) ? p : "";
  task = task_name;
  unit = unit_name;
  total = tot;
  completed = 0;
  update(0, "RUNNING");
}

void Progress::update(size_t done, const char* status, const char* detail) {
  completed = done;
  if (path.empty()) return;
  std::string tmp = path + ".tmp";
  FILE* fp = fopen(tmp.c_str(), "w");
  if (!fp) return;
  fprintf(fp, "task\tstatus\tcompleted\ttotal\tunit\tdetail\n");
  fprintf(fp, "%s\t%s\t%zu\t%zu\t%s\t%s\n", clean_field(task).c_str(), clean_field(status).c_str(),
          completed, total, clean_field(unit).c_str(), clean_field(detail).c_str());
  if (fclose(fp) == 0) rename(tmp.c_str(), path.c_str());
}

int mkdir_p(const std::string& path) {
  if (path.empty()) return -1;
  std::string cur;
  size_t pos = 0;
  while (pos != std::string::npos) {
    pos = path.find('/', pos + 1);
    cur = path.substr(0, pos);
    if (cur.empty()) continue;
    if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return -1;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// SAC
// ---------------------------------------------------------------------------

SacHeader sac_null() {
  // sac_null (native/xc/io/sacio.c:28): floats and ints -12345, nvhdr 6,
  // strings "-12345" padded with blanks
  SacHeader h;
  for (float& v : h.f) v = -12345.0f;
  for (int32_t& v : h.i) v = -12345;
  h.i[SI_NVHDR] = 6;
  char* s = reinterpret_cast<char*>(&h) + 70 * 4 + 40 * 4;
  const size_t nchar = sizeof(SacHeader) - 70 * 4 - 40 * 4;
  memset(s, ' ', nchar);
  auto put = [](char* d) { memcpy(d, "-12345", 6); };
  put(h.kstnm);
  put(h.kevnm);
  put(h.khole);
  put(h.ko);
  put(h.ka);
  for (auto& k : h.kt) put(k);
  put(h.kf);
  for (auto& k : h.kuser) put(k);
  put(h.kcmpnm);
  put(h.knetwk);
  put(h.kdatrd);
  put(h.kinst);
  return h;
}

void sac_text(char* dst, size_t size, const std::string& s) {
  memset(dst, ' ', size);
  memcpy(dst, s.data(), std::min(size, s.size()));
}

int sac_read(const char* path, SacHeader* hd, std::vector<float>* data, int target_npts) {
  // read_sac_buffer (native/sac2spec/io/sacio.c:158-210): truncate to, or
  // zero-pad up to, target_npts samples
  FILE* fp = fopen(path, "rb");
  if (!fp) {
    FXLOG_ERROR("open_sac_failed", "path=\"%s\"", path);
    return -1;
  }
  if (fread(hd, sizeof(SacHeader), 1, fp) != 1 || hd->i[SI_NPTS] < 0) {
    fclose(fp);
    FXLOG_ERROR("read_sac_header_failed", "path=\"%s\"", path);
    return -1;
  }
  if (data && target_npts > 0) {
    data->assign((size_t)target_npts, 0.0f);
    const size_t n = (size_t)std::min(hd->i[SI_NPTS], target_npts);
    if (n > 0 && fread(data->data(), n * sizeof(float), 1, fp) != 1) {
      fclose(fp);
      FXLOG_ERROR("read_sac_data_failed", "path=\"%s\"", path);
      return -1;
    }
  }
  fclose(fp);
  return 0;
}

static int days_in_year(int y) { return ((y % 4 == 0 && y % 100 != 0) || y % 400 == 0) ? 366 : 365; }

static bool digits(const std::string& s, size_t pos, size_t n, int* out) {
  if (pos + n > s.size()) return false;
  int v = 0;
  for (size_t k = 0; k < n; ++k) {
    if (s[pos + k] < '0' || s[pos + k] > '9') return false;
    v = v * 10 + (s[pos + k] - '0');
  }
  *out = v;
  return true;
}

bool parse_timestamp(const std::string& ts, TimeInfo* t) {
  // parse_timestamp_text (native/xc/io/sac_record.cu:64-148): "YYYY.JJJ.HHMM"
  // or "YYYYMMDDTHHMM[SS]" / "YYYY-MM-DDTHH:MM"
  *t = TimeInfo();
  int y = 0, j = 0, hm = 0, used = 0;
  if (sscanf(ts.c_str(), "%d.%d.%d%n", &y, &j, &hm, &used) == 3 && used == (int)ts.size()) {
    const int h = hm / 100, m = hm % 100;
    if (y > 0 && j >= 1 && j <= days_in_year(y) && h >= 0 && h <= 23 && m >= 0 && m <= 59) {
      *t = TimeInfo{y, j, h, m};
      return true;
    }
  }
  int mo = 0, d = 0, h = 0, m = 0;
  size_t tp;
  if (ts.size() >= 13 && (ts[8] == 'T' || ts[8] == 't')) {
    if (!digits(ts, 0, 4, &y) || !digits(ts, 4, 2, &mo) || !digits(ts, 6, 2, &d)) return false;
    tp = 9;
  } else if (ts.size() >= 15 && ts[4] == '-' && ts[7] == '-' && (ts[10] == 'T' || ts[10] == 't')) {
    if (!digits(ts, 0, 4, &y) || !digits(ts, 5, 2, &mo) || !digits(ts, 8, 2, &d)) return false;
    tp = 11;
  } else {
    return false;
  }
  if (tp + 5 <= ts.size() && ts[tp + 2] == ':') {
    if (!digits(ts, tp, 2, &h) || !digits(ts, tp + 3, 2, &m)) return false;
  } else if (tp + 4 <= ts.size()) {
    if (!digits(ts, tp, 2, &h) || !digits(ts, tp + 2, 2, &m)) return false;
  } else {
    return false;
  }
  static const int mdays[12] = {31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31};
  if (mo < 1 || mo > 12) return false;
  int dim = mdays[mo - 1] + ((mo == 2 && days_in_year(y) == 366) ? 1 : 0);
  if (d < 1 || d > dim) return false;
  int jd = d;
  for (int k = 0; k < mo - 1; ++k) jd += mdays[k] + ((k == 1 && days_in_year(y) == 366) ? 1 : 0);
  if (y <= 0 || h < 0 || h > 23 || m < 0 || m > 59) return false;
  *t = TimeInfo{y, jd, h, m};
  return true;
}

// ---------------------------------------------------------------------------
// allowed paths (native/xc/io/path_table.c)
// ---------------------------------------------------------------------------

int make_path_id(int src, int rec) {
  if (src <= 0 || src > 9999 || rec <= 0 || rec > 9999) return -1;
  return src * 10000 + rec;
}

int load_allowed_paths(const char* path, std::vector<PathRecord>* out) {
  out->clear();
  FILE* fp = fopen(path, "r");
  if (!fp) {
    FXLOG_ERROR("allowed_path_table_open_failed", "path=\"%s\" error=\"%s\"", path, strerror(errno));
    return -1;
  }
  char line[4096];
  while (fgets(line, sizeof(line), fp)) {
    if (line[0] == '\0' || line[0] == '\n' || line[0] == '#') continue;
    if (strncmp(line, "path_id", 7) == 0) continue;
    char* f[9] = {0};
    int nf = 0;
    char* save = nullptr;
    for (char* tok = strtok_r(line, "\t\r\n", &save); tok && nf < 9; tok = strtok_r(nullptr, "\t\r\n", &save))
      f[nf++] = tok;
    if (nf < 8) continue;
    PathRecord r;
    r.path_id = atoi(f[0]);
    r.src = atoi(f[1]);
    r.rec = atoi(f[2]);
    if (nf >= 9) {
      r.gcarc = (float)atof(f[5]);
      r.dist = (float)atof(f[6]);
      r.az = (float)atof(f[7]);
      r.baz = (float)atof(f[8]);
    } else {
      r.gcarc = (float)(atof(f[5]) / 111.195);
      r.dist = (float)atof(f[5]);
      r.az = (float)atof(f[6]);
      r.baz = (float)atof(f[7]);
    }
    if (r.path_id <= 0 || r.path_id != make_path_id(r.src, r.rec) || r.src > r.rec) {
      FXLOG_WARN("allowed_path_row_skipped",
                 "path=\"%s\" path_id=%d src=%d rec=%d reason=malformed_or_noncanonical", path,
                 r.path_id, r.src, r.rec);
      continue;
    }
    out->push_back(r);
  }
  fclose(fp);
  std::stable_sort(out->begin(), out->end(),
                   [](const PathRecord& a, const PathRecord& b) { return a.path_id < b.path_id; });
  return 0;
}

const PathRecord* find_path_canonical(const std::vector<PathRecord>& t, int a, int b) {
  const int s = std::min(a, b), r = std::max(a, b);
  const int id = make_path_id(s, r);
  if (id <= 0) return nullptr;
  auto it = std::lower_bound(t.begin(), t.end(), id,
                             [](const PathRecord& x, int v) { return x.path_id < v; });
  return (it != t.end() && it->path_id == id) ? &*it : nullptr;
}

// ---------------------------------------------------------------------------
// row-batch jobs / tasks (native/xc/worker/scheduler.cu:25-148)
// ---------------------------------------------------------------------------

static Job fill_job(size_t files, size_t bs, size_t anchor, size_t tb, size_t te) {
  Job j;
  j.anchor_block = anchor;
  j.target_begin_block = tb;
  j.target_end_block = te;
  j.block_size = bs;
  j.file_count = files;
  j.anchor_begin = anchor * bs;
  j.anchor_end = std::min(files, j.anchor_begin + bs);
  j.target_begin = tb * bs;
  j.target_end = std::min(files, te * bs);
  return j;
}

std::vector<Job> build_jobs(size_t files, size_t bs) {
  std::vector<Job> jobs;
  if (bs == 0) return jobs;
  const size_t nb = (files + bs - 1) / bs;
  for (size_t a = 0; a < nb; ++a) {
    jobs.push_back(fill_job(files, bs, a, a, a + 1));
    for (size_t t = a + 1; t < nb; t += 1) jobs.push_back(fill_job(files, bs, a, t, std::min(nb, t + 1)));
  }
  return jobs;
}

std::vector<Task> build_tasks(const std::vector<int>& g, const std::vector<PathRecord>& paths,
                              const Job& job) {
  std::vector<Task> tasks;
  auto push = [&](size_t s, size_t r, const PathRecord* pr, bool au) {
    tasks.push_back(Task{s, r, pr->path_id, pr, au});
  };
  auto try_pair = [&](size_t a, size_t b, bool same) {
    const bool au = g[a] == g[b];
    if (same && !au && b <= a) return;
    const PathRecord* pr = find_path_canonical(paths, g[a], g[b]);
    if (!pr) return;
    if (au) {
      push(a, b, pr, true);
      if (!same) push(b, a, pr, true);
      return;
    }
    if (g[a] < g[b])
      push(a, b, pr, false);
    else
      push(b, a, pr, false);
  };
  for (size_t tb = job.target_begin_block; tb < job.target_end_block; ++tb) {
    size_t begin = tb * job.block_size, end = std::min(job.file_count, begin + job.block_size);
    const bool same = tb == job.anchor_block;
    if (same) {
      begin = job.anchor_begin;
      end = job.anchor_end;
    }
    for (size_t a = job.anchor_begin; a < job.anchor_end; ++a)
      for (size_t b = begin; b < end; ++b) try_pair(a, b, same);
  }
  return tasks;
}

// ---------------------------------------------------------------------------
// stepack v3 (native/sac2spec/io/stepack_writer.c)
// ---------------------------------------------------------------------------

static const char kStepackTsvHeader[] =
    "timestamp\tworker_id\tbatch_seq\tstart_group\tgroup_count\t"
    "pack_path\toffset\tbytes\tversion\tlayout\tnstep\tnslc_start\t"
    "nslc_count\tbatch_nslc_count\tnspec\tdt\tdf\tnslc_table_bytes\t"
    "payload_offset\tpayload_bytes\tbatch_payload_bytes\tstep_bytes\t"
    "pitch_step_bytes\tnslc_step_bytes\tfirst_nsl_id\tlast_nsl_id\n";

static void fixed_copy(char* dst, size_t size, const std::string& s) {
  memset(dst, 0, size);
  for (size_t i = 0; i + 1 < size && i < s.size(); ++i) {
    const char c = s[i];
    dst[i] = (c == '\t' || c == '\n' || c == '\r') ? ' ' : c;
  }
}

static std::string abs_path(const std::string& p) {
  if (!p.empty() && p[0] == '/') return p;
  char cwd[4096];
  if (!getcwd(cwd, sizeof(cwd))) return p;
  return std::string(cwd) + "/" + p;
}

int stepack_write_batch(const std::string& root_in, int worker_id, size_t batch_seq,
                        size_t start_group, size_t group_count, const std::vector<Channel>& nodes,
                        int nstep, int nspec, float dt, float df, const float* payload) {
  if (nodes.empty()) return 0;
  const std::string root = abs_path(root_in);
  if (mkdir_p(root) != 0) return -1;
  char leaf[64];
  snprintf(leaf, sizeof(leaf), "w%03d.b%06zu.", worker_id, batch_seq);
  const std::string pack_path = root + "/" + leaf + "stepack";
  const std::string tsv_path = root + "/" + leaf + "tsv";
  const uint64_t n = nodes.size();
  const uint64_t table = n * sizeof(StepackNslc);
  const uint64_t nslc_step = (uint64_t)nspec * 8;
  const uint64_t pitch = n * nslc_step;
  const uint64_t pay = (uint64_t)nstep * pitch;
  const uint64_t rec = sizeof(StepackHeader) + table + pay;
  StepackHeader h;
  memset(&h, 0, sizeof(h));
  memcpy(h.magic, "FXCSTPK", 7);
  h.version = 3;
  h.header_size = sizeof(StepackHeader);
  h.nslc_entry_size = sizeof(StepackNslc);
  h.layout = 2;
  h.batch_seq = batch_seq;
  h.start_group = start_group;
  h.group_count = group_count;
  h.worker_id = (uint32_t)worker_id;
  h.nstep = (uint32_t)nstep;
  h.nslc_count = (uint32_t)n;
  h.nspec = (uint32_t)nspec;
  h.dt = dt;
  h.df = df;
  h.nslc_table_bytes = table;
  h.payload_offset = sizeof(StepackHeader) + table;
  h.payload_bytes = pay;
  h.pitch_step_bytes = pitch;
  fixed_copy(h.first_timestamp, sizeof(h.first_timestamp), nodes[0].timestamp);
  std::vector<StepackNslc> tab(n);
  for (size_t i = 0; i < n; ++i) {
    StepackNslc& e = tab[i];
    memset(&e, 0, sizeof(e));
    e.file_index = (uint32_t)i;
    e.nsl_id = (uint32_t)nodes[i].nsl_id;
    e.stla = nodes[i].stla;
    e.stlo = nodes[i].stlo;
    fixed_copy(e.network, sizeof(e.network), nodes[i].network);
    fixed_copy(e.station, sizeof(e.station), nodes[i].station);
    fixed_copy(e.location, sizeof(e.location), nodes[i].location);
    fixed_copy(e.component, sizeof(e.component), nodes[i].component);
  }
  FILE* pf = fopen(pack_path.c_str(), "wb");
  FILE* tf = fopen(tsv_path.c_str(), "w");
  int st = -1;
  if (pf && tf && fwrite(&h, sizeof(h), 1, pf) == 1 && fwrite(tab.data(), table, 1, pf) == 1 &&
      (pay == 0 || fwrite(payload, pay, 1, pf) == 1)) {
    fputs(kStepackTsvHeader, tf);
    const size_t num_ch = (group_count > 0 && n % group_count == 0) ? n / group_count : 0;
    size_t b = 0;
    while (b < n) {
      size_t e = b + 1;
      while (e < n && nodes[e].timestamp == nodes[b].timestamp) ++e;
      const size_t rc = e - b;
      size_t rsg = start_group, rgc = group_count;
      if (num_ch > 0 && b % num_ch == 0 && rc % num_ch == 0) {
        rsg = start_group + b / num_ch;
        rgc = rc / num_ch;
      }
      const uint64_t rstep = rc * nslc_step, rpay = (uint64_t)nstep * rstep;
      fputs(clean_field(nodes[b].timestamp).c_str(), tf);
      fprintf(tf, "\t%d\t%zu\t%zu\t%zu\t", worker_id, batch_seq, rsg, rgc);
      fputs(clean_field(pack_path).c_str(), tf);
      fprintf(tf,
              "\t%llu\t%llu\t%u\t%u\t%d\t%zu\t%zu\t%zu\t%d\t%.9g\t%.9g\t%llu\t%llu\t%llu\t%llu\t%llu\t"
              "%llu\t%llu\t",
              0ull, (unsigned long long)rec, 3u, 2u, nstep, b, rc, (size_t)n, nspec, dt, df,
              (unsigned long long)table, (unsigned long long)h.payload_offset,
              (unsigned long long)rpay, (unsigned long long)pay, (unsigned long long)rstep,
              (unsigned long long)pitch, (unsigned long long)nslc_step);
      auto nsl = [](const Channel& c) {
        return c.nsl_text.empty() ? std::to_string(c.nsl_id) : clean_field(c.nsl_text);
      };
      fprintf(tf, "%s\t%s\n", nsl(nodes[b]).c_str(), nsl(nodes[e - 1]).c_str());
      b = e;
    }
    st = 0;
  } else {
    FXLOG_ERROR("stepack_batch_write_failed", "path=\"%s\" errno=%d", pack_path.c_str(), errno);
  }
  if (pf && fclose(pf) != 0) st = -1;
  if (tf && fclose(tf) != 0) st = -1;
  return st;
}

static std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\r' || s[a] == '\n')) ++a;
  while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r' || s[b - 1] == '\n')) --b;
  return s.substr(a, b - a);
}

static std::vector<std::string> split_tab(const std::string& s) {
  std::vector<std::string> out;
  size_t p = 0;
  while (true) {
    size_t q = s.find('\t', p);
    out.push_back(s.substr(p, q == std::string::npos ? std::string::npos : q - p));
    if (q == std::string::npos) break;
    p = q + 1;
  }
  return out;
}

static bool is_dir(const std::string& p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

int stepack_load_index(const std::string& input, std::vector<TimestampInput>* out) {
  std::vector<std::string> tsvs;
  if (is_dir(input)) {
    std::string dir = input;
    if (is_dir(dir + "/stepack")) dir += "/stepack";
    DIR* d = opendir(dir.c_str());
    if (!d) return -1;
    while (dirent* e = readdir(d)) {
      std::string n = e->d_name;
      if (n.size() > 4 && n.compare(n.size() - 4, 4, ".tsv") == 0) tsvs.push_back(dir + "/" + n);
    }
    closedir(d);
    std::sort(tsvs.begin(), tsvs.end());
  } else {
    tsvs.push_back(input);
  }
  if (tsvs.empty()) {
    FXLOG_ERROR("stepack_tsv_not_found", "path=\"%s\"", input.c_str());
    return -1;
  }
  std::map<std::string, size_t> by_ts;
  out->clear();
  for (const std::string& t : tsvs) {
    FILE* fp = fopen(t.c_str(), "r");
    if (!fp) return -1;
    std::string base = t.substr(0, t.find_last_of('/'));
    std::vector<std::string> hdr;
    char line[16384];
    while (fgets(line, sizeof(line), fp)) {
      std::string text = trim(line);
      if (text.empty() || text[0] == '#') continue;
      std::vector<std::string> f = split_tab(text);
      if (hdr.empty()) {
        hdr = f;
        continue;
      }
      auto col = [&](const char* name) -> int {
        for (size_t i = 0; i < hdr.size(); ++i)
          if (hdr[i] == name) return (int)i;
        return -1;
      };
      auto get = [&](const char* name) -> std::string {
        const int c = col(name);
        return (c >= 0 && c < (int)f.size()) ? f[c] : std::string();
      };
      StepackFragment fr;
      fr.timestamp = get("timestamp");
      fr.pack_path = get("pack_path");
      if (!fr.pack_path.empty() && fr.pack_path[0] != '/') fr.pack_path = base + "/" + fr.pack_path;
      fr.batch_seq = strtoull(get("batch_seq").c_str(), nullptr, 10);
      fr.start_group = strtoull(get("start_group").c_str(), nullptr, 10);
      fr.nstep = strtoull(get("nstep").c_str(), nullptr, 10);
      fr.nslc_start = strtoull(get("nslc_start").c_str(), nullptr, 10);
      fr.nslc_count = strtoull(get("nslc_count").c_str(), nullptr, 10);
      fr.batch_nslc_count = strtoull(get("batch_nslc_count").c_str(), nullptr, 10);
      fr.nspec = strtoull(get("nspec").c_str(), nullptr, 10);
      fr.dt = strtof(get("dt").c_str(), nullptr);
      fr.df = strtof(get("df").c_str(), nullptr);
      fr.payload_offset = strtoull(get("payload_offset").c_str(), nullptr, 10);
      fr.pitch_step_bytes = strtoull(get("pitch_step_bytes").c_str(), nullptr, 10);
      fr.nslc_step_bytes = strtoull(get("nslc_step_bytes").c_str(), nullptr, 10);
      if (fr.timestamp.empty() || fr.pack_path.empty() || fr.nstep == 0 || fr.nspec < 2) {
        FXLOG_ERROR("stepack_tsv_row_malformed", "path=\"%s\" row=\"%s\"", t.c_str(), text.c_str());
        fclose(fp);
        return -1;
      }
      auto it = by_ts.find(fr.timestamp);
      if (it == by_ts.end()) {
        by_ts[fr.timestamp] = out->size();
        out->push_back(TimestampInput{fr.timestamp, {}});
        it = by_ts.find(fr.timestamp);
      }
      (*out)[it->second].fragments.push_back(fr);
    }
    fclose(fp);
  }
  std::sort(out->begin(), out->end(),
            [](const TimestampInput& a, const TimestampInput& b) { return a.timestamp < b.timestamp; });
  for (TimestampInput& ti : *out)
    std::sort(ti.fragments.begin(), ti.fragments.end(),
              [](const StepackFragment& a, const StepackFragment& b) {
                if (a.batch_seq != b.batch_seq) return a.batch_seq < b.batch_seq;
                if (a.start_group != b.start_group) return a.start_group < b.start_group;
                if (a.nslc_start != b.nslc_start) return a.nslc_start < b.nslc_start;
                return a.pack_path < b.pack_path;
              });
  return 0;
}

static int pread_all(int fd, size_t off, void* dst, size_t n) {
  char* o = static_cast<char*>(dst);
  size_t done = 0;
  while (done < n) {
    ssize_t r = pread(fd, o + done, std::min(n - done, (size_t)1 << 30), (off_t)(off + done));
    if (r < 0 && errno == EINTR) continue;
    if (r <= 0) return -1;
    done += (size_t)r;
  }
  return 0;
}

static std::string fixed_str(const char* s, size_t n) {
  size_t k = 0;
  while (k < n && s[k] != '\0') ++k;
  return std::string(s, k);
}

int stepack_open_timestamp(const TimestampInput& in, std::vector<Channel>* chans, int* nstep,
                           int* nspec, float* dt, float* df, std::vector<float>* payload) {
  struct Tmp {
    Channel c;
    size_t frag, local, order;
  };
  std::vector<Tmp> all;
  std::vector<int> fds;
  *nstep = 0;
  for (size_t fi = 0; fi < in.fragments.size(); ++fi) {
    const StepackFragment& fr = in.fragments[fi];
    int fd = open(fr.pack_path.c_str(), O_RDONLY);
    if (fd < 0) {
      FXLOG_ERROR("stepack_open_failed", "path=\"%s\"", fr.pack_path.c_str());
      for (int x : fds) close(x);
      return -1;
    }
    fds.push_back(fd);
    StepackHeader h;
    if (pread_all(fd, 0, &h, sizeof(h)) != 0 || memcmp(h.magic, "FXCSTPK", 7) != 0 ||
        h.version != 3 || h.header_size != sizeof(StepackHeader) ||
        h.nslc_entry_size != sizeof(StepackNslc) || h.layout != 2 || h.nstep != fr.nstep ||
        h.nspec != fr.nspec || h.nslc_count != fr.batch_nslc_count ||
        fr.nslc_start + fr.nslc_count > fr.batch_nslc_count) {
      FXLOG_ERROR("stepack_format_unsupported", "path=\"%s\"", fr.pack_path.c_str());
      for (int x : fds) close(x);
      return -1;
    }
    if (fi == 0) {
      *nstep = (int)h.nstep;
      *nspec = (int)h.nspec;
      *dt = h.dt;
      *df = h.df;
    } else if ((int)h.nstep != *nstep || (int)h.nspec != *nspec) {
      FXLOG_ERROR("stepack_shape_mismatch", "path=\"%s\"", fr.pack_path.c_str());
      for (int x : fds) close(x);
      return -1;
    }
    std::vector<StepackNslc> tab(fr.nslc_count);
    if (fr.nslc_count && pread_all(fd, sizeof(StepackHeader) + fr.nslc_start * sizeof(StepackNslc),
                                   tab.data(), fr.nslc_count * sizeof(StepackNslc)) != 0) {
      for (int x : fds) close(x);
      return -1;
    }
    for (size_t i = 0; i < fr.nslc_count; ++i) {
      Tmp t;
      t.c.timestamp = in.timestamp;
      t.c.network = fixed_str(tab[i].network, 16);
      t.c.station = fixed_str(tab[i].station, 32);
      t.c.location = fixed_str(tab[i].location, 16);
      t.c.component = fixed_str(tab[i].component, 16);
      t.c.nsl_id = (int)tab[i].nsl_id;
      t.c.stla = tab[i].stla;
      t.c.stlo = tab[i].stlo;
      t.frag = fi;
      t.local = i;
      t.order = all.size();
      all.push_back(t);
    }
  }
  std::stable_sort(all.begin(), all.end(), [](const Tmp& a, const Tmp& b) {
    if (a.c.nsl_id != b.c.nsl_id) return a.c.nsl_id < b.c.nsl_id;
    return a.order < b.order;
  });
  chans->clear();
  for (const Tmp& t : all) chans->push_back(t.c);
  const size_t nch = all.size(), ns = (size_t)*nspec;
  payload->assign((size_t)*nstep * nch * ns * 2, 0.0f);
  for (size_t c = 0; c < nch; ++c) {
    const StepackFragment& fr = in.fragments[all[c].frag];
    const int fd = fds[all[c].frag];
    for (int s = 0; s < *nstep; ++s) {
      const size_t off = fr.payload_offset + (size_t)s * fr.pitch_step_bytes +
                         (fr.nslc_start + all[c].local) * fr.nslc_step_bytes;
      if (pread_all(fd, off, payload->data() + ((size_t)s * nch + c) * ns * 2, ns * 8) != 0) {
        for (int x : fds) close(x);
        return -1;
      }
    }
  }
  for (int x : fds) close(x);
  return 0;
}

size_t infer_num_channels(const std::vector<Channel>& ch) {
  size_t expected = 0, i = 0;
  int last = 0;
  while (i < ch.size()) {
    const int id = ch[i].nsl_id;
    if (id <= last) return 0;
    const size_t b = i;
    while (i < ch.size() && ch[i].nsl_id == id) ++i;
    if (expected == 0)
      expected = i - b;
    else if (i - b != expected)
      return 0;
    last = id;
  }
  return expected;
}

// ---------------------------------------------------------------------------
// xcpack (native/xc/pack_io/pack_writer.cu, io/sac_record.cu)
// ---------------------------------------------------------------------------

static const char kXcpackTsvHeader[] =
    "timestamp\tworker_id\tanchor_block\ttarget_begin_block\ttarget_end_block\t"
    "block_size\tanchor_begin\tanchor_end\ttarget_begin\ttarget_end\t"
    "pack_path\toffset\tbytes\t"
    "src_id\trec_id\tsrc_network\tsrc_station\tsrc_location\tsrc_component\t"
    "rec_network\trec_station\trec_location\trec_component\t"
    "npts\tdt\tdist\taz\tbaz\tfinal_pair_path\n";

int XcPackWriter::open(const std::string& root_dir, const std::string& ts, size_t worker,
                       const Job& j) {
  root = root_dir;
  timestamp = ts;
  worker_id = worker;
  job = j;
  part = 0;
  if (mkdir_p(root) != 0) return -1;
  char name[512];
  snprintf(name, sizeof(name), "%s.i%06zu.j%06zu.w%03zu.p%03zu", ts.c_str(), j.anchor_block,
           j.target_begin_block, worker, part);
  pack_path = root + "/" + name + ".xcpack";
  tsv_path = root + "/" + name + ".tsv";
  pack = fopen(pack_path.c_str(), "ab");
  tsv = fopen(tsv_path.c_str(), "ab");
  if (!pack || !tsv) return -1;
  fseeko(pack, 0, SEEK_END);
  fseeko(tsv, 0, SEEK_END);
  if (ftello(tsv) == 0) fputs(kXcpackTsvHeader, tsv);
  bytes = (uint64_t)ftello(pack);
  return 0;
}

int XcPackWriter::append(const Task& t, const Channel& src, const Channel& rec, const SacHeader& hd,
                         const float* trace, int npts, float dt, const std::string& fpp) {
  const uint64_t rb = sizeof(SacHeader) + (uint64_t)npts * 4;
  if (bytes > 0 && bytes + rb > max_bytes) {
    fclose(pack);
    fclose(tsv);
    ++part;
    char name[512];
    snprintf(name, sizeof(name), "%s.i%06zu.j%06zu.w%03zu.p%03zu", timestamp.c_str(),
             job.anchor_block, job.target_begin_block, worker_id, part);
    pack_path = root + "/" + name + ".xcpack";
    tsv_path = root + "/" + name + ".tsv";
    pack = fopen(pack_path.c_str(), "ab");
    tsv = fopen(tsv_path.c_str(), "ab");
    if (!pack || !tsv) return -1;
    fseeko(pack, 0, SEEK_END);
    fseeko(tsv, 0, SEEK_END);
    if (ftello(tsv) == 0) fputs(kXcpackTsvHeader, tsv);
    bytes = (uint64_t)ftello(pack);
  }
  const uint64_t off = bytes;
  if (fwrite(&hd, sizeof(hd), 1, pack) != 1 || fwrite(trace, (size_t)npts * 4, 1, pack) != 1)
    return -1;
  bytes += rb;
  fprintf(tsv,
          "%s\t%zu\t%zu\t%zu\t%zu\t%zu\t%zu\t%zu\t%zu\t%zu\t%s\t%llu\t%llu\t%d\t%d\t%s\t%s\t%s\t%s\t%s\t%s\t%s\t"
          "%s\t%d\t%.9g\t%.9g\t%.9g\t%.9g\t%s\n",
          clean_field(timestamp).c_str(), worker_id, job.anchor_block, job.target_begin_block,
          job.target_end_block, job.block_size, job.anchor_begin, job.anchor_end, job.target_begin,
          job.target_end, clean_field(pack_path).c_str(), (unsigned long long)off,
          (unsigned long long)rb, src.nsl_id, rec.nsl_id, clean_field(src.network).c_str(),
          clean_field(src.station).c_str(), clean_field(src.location).c_str(),
          clean_field(src.component).c_str(), clean_field(rec.network).c_str(),
          clean_field(rec.station).c_str(), clean_field(rec.location).c_str(),
          clean_field(rec.component).c_str(), npts, dt, t.path->dist, t.path->az, t.path->baz,
          clean_field(fpp).c_str());
  return 0;
}

int XcPackWriter::close() {
  int st = 0;
  if (pack && fclose(pack) != 0) st = -1;
  if (tsv && fclose(tsv) != 0) st = -1;
  pack = tsv = nullptr;
  return st;
}

int write_marker(const std::string& path) {
  FILE* fp = fopen(path.c_str(), "w");
  if (!fp) return -1;
  fprintf(fp, "DONE\n");
  return fclose(fp) == 0 ? 0 : -1;
}

std::string final_pair_path(const std::string& ncf_dir, const Channel& s, const Channel& r) {
  // build_output_path (native/xc/io/sac_record.cu:158-186)
  return ncf_dir + "/" + s.network + "." + s.station + "/" + r.network + "." + r.station + "/" +
         s.network + "-" + r.network + "." + s.station + "-" + r.station + "." + s.component + "-" +
         r.component + ".sac";
}

SacHeader ncf_header(const Task& t, const Channel& src, const Channel& rec, float dt, int cc_size,
                     float cc_len, const TimeInfo* ti, bool have_time) {
  // SacheadProcess (native/xc/io/sac_header.c:3-39) + build_sac_header_for_task
  // (native/xc/io/sac_record.cu:188-213)
  SacHeader h = sac_null();
  h.f[SF_STLA] = rec.stla;
  h.f[SF_STLO] = rec.stlo;
  h.f[SF_EVLA] = src.stla;
  h.f[SF_EVLO] = src.stlo;
  h.f[SF_GCARC] = t.path->gcarc;
  h.f[SF_AZ] = t.path->az;
  h.f[SF_BAZ] = t.path->baz;
  h.f[SF_DIST] = t.path->dist;
  h.i[SI_IFTYPE] = 1;
  h.i[SI_LEVEN] = 1;
  h.f[SF_DELTA] = dt;
  h.i[SI_NPTS] = cc_size;
  h.f[SF_B] = -1.0f * cc_len;
  h.f[SF_E] = cc_len;
  h.i[SI_UNUSED27] = 1;
  h.f[SF_O] = 0.0f;
  if (have_time) {
    h.i[SI_NZYEAR] = ti->year;
    h.i[SI_NZJDAY] = ti->jday;
    h.i[SI_NZHOUR] = ti->hour;
    h.i[SI_NZMIN] = ti->minute;
    h.i[SI_NZSEC] = 0;
    h.i[SI_NZMSEC] = 0;
  }
  sac_text(h.kstnm, sizeof(h.kstnm), rec.station);
  sac_text(h.knetwk, sizeof(h.knetwk), rec.network);
  sac_text(h.kcmpnm, sizeof(h.kcmpnm), src.component + "-" + rec.component);
  sac_text(h.kevnm, sizeof(h.kevnm), src.network + "." + src.station);
  h.f[SF_USER0] = (float)src.nsl_id;
  h.f[SF_USER1] = (float)rec.nsl_id;
  h.f[SF_USER2] = (float)t.path_id;
  return h;
}

}  // namespace fxcio
