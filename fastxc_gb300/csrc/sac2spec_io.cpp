// sac2spec host inputs and bookkeeping; the reference lines each piece
// restates are listed in sac2spec_io.h.
#include "sac2spec_io.h"

#include <ctype.h>
#include <errno.h>
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

namespace fxcio {

namespace {

std::string trim_space(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && isspace((unsigned char)s[a])) ++a;
  while (b > a && isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

// copyCleanField: whitespace runs inside a field become one '_', a trailing
// '_' is dropped; at most 254 characters are kept.
std::string clean_field(const std::string& s) {
  std::string out;
  bool last_space = false;
  for (char c : s) {
    if (out.size() + 1 >= 255) break;
    if (isspace((unsigned char)c)) {
      if (!out.empty() && !last_space) out.push_back('_');
      last_space = true;
    } else {
      out.push_back(c);
      last_space = false;
    }
  }
  if (!out.empty() && out.back() == '_') out.pop_back();
  return out;
}

}  // namespace

int read_sac_index(const char* path, int num_ch, std::vector<SacIndexRow>* rows) {
  FILE* fp = fopen(path, "r");
  if (!fp) {
    FXLOG_ERROR("open_sac_index_failed", "path=\"%s\"", path);
    return -1;
  }
  rows->clear();
  std::vector<SacIndexRow> group;
  std::string cur_nsl, cur_ts;
  // appendPathPair parses nsl_id (0..9999) of the groups it keeps
  auto flush = [&]() -> bool {
    if (group.empty()) return true;
    if (num_ch == 1 || group.size() == (size_t)num_ch) {
      for (SacIndexRow& r : group) {
        char* end = nullptr;
        errno = 0;
        const long v = strtol(r.nsl_text.c_str(), &end, 10);
        if (errno != 0 || end == r.nsl_text.c_str() || *end != '\0' || v < 0 || v > 9999) {
          FXLOG_ERROR("sac_index_nsl_id_invalid", "nsl_id=\"%s\" path=\"%s\" expected=0000..9999",
                      r.nsl_text.c_str(), r.sac_path.c_str());
          return false;
        }
        r.nsl_id = (int)v;
      }
      rows->insert(rows->end(), group.begin(), group.end());
    } else {
      FXLOG_WARN("sac_index_group_skipped",
                 "timestamp=%s nsl_id=%s path=\"%s\" expected_components=%d got_components=%zu",
                 cur_ts.c_str(), group[0].nsl_text.c_str(), path, num_ch, group.size());
    }
    group.clear();
    return true;
  };
  char buf[8192];
  int line_no = 0;
  while (fgets(buf, sizeof(buf), fp)) {
    ++line_no;
    const std::string t = trim_space(buf);
    if (t.empty() || t[0] == '#') continue;
    if (t.compare(0, 9, "timestamp") == 0 || t.compare(0, 6, "nsl_id") == 0) continue;
    std::vector<std::string> f;
    size_t start = 0;
    for (int i = 0; i < 6; ++i) {
      const size_t tab = t.find('\t', start);
      if (tab == std::string::npos) break;
      f.push_back(trim_space(t.substr(start, tab - start)));
      start = tab + 1;
    }
    if (f.size() != 6) {
      FXLOG_ERROR("sac_index_row_malformed_tsv", "path=\"%s\" line=%d expected=7_tab_separated_fields",
                  path, line_no);
      fclose(fp);
      return -1;
    }
    f.push_back(trim_space(t.substr(start)));
    SacIndexRow r;
    r.timestamp = clean_field(f[0]);
    r.nsl_text = clean_field(f[1]);
    r.network = clean_field(f[2]);
    r.station = clean_field(f[3]);
    r.location = clean_field(f[4]);
    r.component = clean_field(f[5]);
    r.sac_path = f[6];
    if (r.timestamp.empty() || r.nsl_text.empty() || r.network.empty() || r.station.empty() ||
        r.location.empty() || r.component.empty() || r.sac_path.empty()) {
      FXLOG_ERROR("sac_index_row_incomplete", "path=\"%s\" line=%d", path, line_no);
      fclose(fp);
      return -1;
    }
    if (!cur_nsl.empty() && (cur_nsl != r.nsl_text || cur_ts != r.timestamp) && !flush()) {
      fclose(fp);
      return -1;
    }
    cur_nsl = r.nsl_text;
    cur_ts = r.timestamp;
    group.push_back(r);
  }
  fclose(fp);
  if (!flush()) return -1;
  if (rows->empty()) {
    FXLOG_ERROR("sac_index_empty", "path=\"%s\"", path);
    return -1;
  }
  FXLOG_INFO("sac_index_loaded", "rows=%zu path=\"%s\"", rows->size(), path);
  return 0;
}

int read_filter_file(const char* path, FilterSet* out) {
  FILE* fp = fopen(path, "r");
  if (!fp) {
    FXLOG_ERROR("open_filter_file_failed", "path=\"%s\"", path);
    return -1;
  }
  *out = FilterSet();
  char line[1024];
  int state = 0;
  float lo = 0, hi = 0;
  double b[5] = {0}, a[5] = {0};
  while (fgets(line, sizeof(line), fp)) {
    if (line[0] == '#') {
      if (sscanf(line, "# %f/%f", &lo, &hi) != 2) {
        FXLOG_WARN("filter_band_malformed", "path=\"%s\"", path);
        continue;
      }
      state = 1;
      continue;
    }
    if (state == 1) {
      if (sscanf(line, "%lf %lf %lf %lf %lf", &b[0], &b[1], &b[2], &b[3], &b[4]) != 5) continue;
      state = 2;
      continue;
    }
    if (state == 2) {
      if (sscanf(line, "%lf %lf %lf %lf %lf", &a[0], &a[1], &a[2], &a[3], &a[4]) != 5) {
        state = 0;
        continue;
      }
      out->freq_low.push_back(lo);
      out->freq_high.push_back(hi);
      out->b.insert(out->b.end(), b, b + 5);
      out->a.insert(out->a.end(), a, a + 5);
      lo = hi = 0;
      for (int i = 0; i < 5; ++i) b[i] = a[i] = 0;
      state = 0;
    }
  }
  fclose(fp);
  return 0;
}

bool sac_delta_matches(float observed, float expected) {
  float tol = fabsf(expected) * 1.0e-5f;
  if (tol < 1.0e-6f) tol = 1.0e-6f;
  return fabsf(observed - expected) <= tol;
}

static bool safe_char(char c) {
  return (c >= '0' && c <= '9') || (c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z') || c == '.' ||
         c == '_' || c == ':' || c == '-';
}

std::string timestamp_leaf(const std::string& ts) {
  std::string o;
  for (char c : ts) {
    if (o.size() + 1 >= 255) break;
    o.push_back(safe_char(c) ? c : '-');
  }
  while (!o.empty() && o.back() == '-') o.pop_back();
  if (o.empty()) o = "timestamp";
  return o;
}

bool timestamp_leaf_is_safe(const std::string& ts) {
  const std::string leaf = timestamp_leaf(ts);
  return leaf == ts && leaf != "." && leaf != "..";
}

void S2sProgress::init(const std::string& path, size_t total_rows) {
  std::lock_guard<std::mutex> lk(mu_);
  path_ = path;
  enabled_ = !path.empty() && path != "NONE";
  total_ = total_rows;
  done_ = 0;
  write_locked("RUNNING", -1, 0, 0, 0);
}

void S2sProgress::add(size_t rows, int gpu_id, size_t start_group, size_t group_count) {
  std::lock_guard<std::mutex> lk(mu_);
  done_ += rows;
  if (done_ > total_) done_ = total_;
  write_locked("RUNNING", gpu_id, rows, start_group, group_count);
}

void S2sProgress::finish(const char* status, bool complete) {
  std::lock_guard<std::mutex> lk(mu_);
  if (complete) done_ = total_;
  write_locked(status, -1, 0, 0, 0);
}

void S2sProgress::write_locked(const char* status, int gpu_id, size_t batch_rows, size_t start_group,
                               size_t group_count) {
  if (!enabled_) return;
  const std::string tmp = path_ + ".tmp";
  FILE* fp = fopen(tmp.c_str(), "w");
  if (!fp) {
    enabled_ = false;
    return;
  }
  fprintf(fp, "task\tstatus\tcompleted\ttotal\tunit\tdetail\n");
  fprintf(fp, "overall\t%s\t%zu\t%zu\tsac_rows\tgpu_id=%d last_batch_rows=%zu start_group=%zu group_count=%zu\n",
          status, done_, total_, gpu_id, batch_rows, start_group, group_count);
  if (fclose(fp) != 0 || rename(tmp.c_str(), path_.c_str()) != 0) enabled_ = false;
}

int TimestampTracker::init(const std::vector<SacIndexRow>& rows, int num_ch, const std::string& root) {
  root_ = root;
  entries_.clear();
  const size_t groups = rows.size() / (size_t)num_ch;
  group_entry_.assign(groups, 0);
  for (size_t g = 0; g < groups; ++g) {
    const std::string& ts = rows[g * num_ch].timestamp;
    if (!timestamp_leaf_is_safe(ts)) {
      FXLOG_ERROR("timestamp_unsafe_for_path", "timestamp=%s group=%zu action=fix_sac_index_timestamp",
                  ts.c_str(), g);
      return -1;
    }
    for (int c = 1; c < num_ch; ++c) {
      if (rows[g * num_ch + c].timestamp != ts) {
        FXLOG_ERROR("timestamp_group_mismatch", "group=%zu ch0=%s ch%d=%s", g, ts.c_str(), c,
                    rows[g * num_ch + c].timestamp.c_str());
        return -1;
      }
    }
    if (entries_.empty() || entries_.back().timestamp != ts) {
      for (const Entry& e : entries_) {
        if (e.timestamp == ts) {
          FXLOG_ERROR("timestamp_not_contiguous", "timestamp=%s group=%zu", ts.c_str(), g);
          return -1;
        }
      }
      entries_.push_back(Entry{ts, 0, 0});
    }
    ++entries_.back().group_count;
    group_entry_[g] = (int)entries_.size() - 1;
  }
  return 0;
}

int TimestampTracker::mark_done(size_t start_group, size_t group_count) {
  std::lock_guard<std::mutex> lk(mu_);
  if (start_group + group_count > group_entry_.size()) {
    FXLOG_ERROR("timestamp_batch_range_invalid", "start_group=%zu group_count=%zu total_groups=%zu",
                start_group, group_count, group_entry_.size());
    return -1;
  }
  for (size_t g = start_group; g < start_group + group_count; ++g) {
    Entry& e = entries_[group_entry_[g]];
    if (++e.done != e.group_count) continue;
    const std::string dir = root_ + "/" + timestamp_leaf(e.timestamp);
    if (mkdir_p(dir) != 0) return -1;
    const std::string p = dir + "/_SUCCESS";
    FILE* fp = fopen(p.c_str(), "wb");
    if (!fp) {
      FXLOG_ERROR("write_timestamp_success_failed", "path=\"%s\" errno=%d", p.c_str(), errno);
      return -1;
    }
    fprintf(fp, "timestamp\t%s\ngroups\t%zu\n", e.timestamp.c_str(), e.group_count);
    if (fclose(fp) != 0) return -1;
  }
  return 0;
}

}  // namespace fxcio
