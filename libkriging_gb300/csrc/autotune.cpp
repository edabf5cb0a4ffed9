// autotune.cpp -- the measured-choice table (autotune.hpp) and its C ABI.
#include "autotune.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace lkg {

void set_last_error(const char* msg);

int autotune_select(const std::vector<double>& costs) {
  int best = -1;
  for (int i = 0; i < (int)costs.size(); ++i)
    if (std::isfinite(costs[i]) && (best < 0 || costs[i] < costs[best])) best = i;
  return best;
}

Autotuner& Autotuner::instance() {
  static Autotuner t;
  return t;
}

Autotuner::Autotuner() {
  const char* off = std::getenv("LKG_AUTOTUNE");
  if (off && std::strcmp(off, "0") == 0) enabled_ = false;
  const char* f = std::getenv("LKG_TUNE_FILE");
  if (f && *f) {
    file_ = f;
    load_file(file_);
  }
}

int Autotuner::lookup(const std::string& key, int fallback) const {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = table_.find(key);
  return it == table_.end() ? fallback : it->second.choice;
}

int Autotuner::record(const std::string& key, const std::vector<int>& candidates, const std::vector<double>& costs) {
  const int i = autotune_select(costs);
  if (i < 0) return -1;
  {
    std::lock_guard<std::mutex> lk(mu_);
    table_[key] = Entry{candidates[i], costs[i]};
  }
  if (!file_.empty()) save_file(file_);
  return candidates[i];
}

int Autotuner::choose(const std::string& key, const std::vector<int>& candidates, int fallback,
                      const std::function<double(int)>& cost) {
  if (!enabled_ || candidates.empty()) return fallback;
  {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = table_.find(key);
    if (it != table_.end()) return it->second.choice;
  }
  std::vector<double> costs;
  costs.reserve(candidates.size());
  for (int c : candidates) costs.push_back(cost(c));
  const int r = record(key, candidates, costs);
  return r < 0 ? fallback : r;
}

std::string Autotuner::report() const {
  std::lock_guard<std::mutex> lk(mu_);
  std::ostringstream o;
  o.precision(9);
  for (const auto& kv : table_) o << kv.first << "\t" << kv.second.choice << "\t" << kv.second.cost << "\n";
  return o.str();
}

void Autotuner::clear() {
  std::lock_guard<std::mutex> lk(mu_);
  table_.clear();
}

void Autotuner::clear_key(const std::string& key) {
  std::lock_guard<std::mutex> lk(mu_);
  table_.erase(key);
}

bool Autotuner::save_file(const std::string& path) const {
  std::ostringstream o;
  o.precision(17);
  {
    std::lock_guard<std::mutex> lk(mu_);
    o << "{";
    bool first = true;
    for (const auto& kv : table_) {
      o << (first ? "\n" : ",\n") << "  \"" << kv.first << "\": [" << kv.second.choice << ", "
        << (std::isfinite(kv.second.cost) ? kv.second.cost : -1.0) << "]";
      first = false;
    }
    o << "\n}\n";
  }
  const std::string tmp = path + ".tmp";
  {
    std::ofstream f(tmp, std::ios::trunc);
    if (!f) return false;
    f << o.str();
    if (!f) return false;
  }
  return std::rename(tmp.c_str(), path.c_str()) == 0;
}

// the file format written above: a flat object of "key": [int, number]; keys hold no quotes or backslashes
bool Autotuner::load_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) return false;
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string s = ss.str();
  std::map<std::string, Entry> parsed;
  size_t p = s.find('{');
  if (p == std::string::npos) return false;
  for (;;) {
    const size_t q0 = s.find('"', p + 1);
    if (q0 == std::string::npos) break;
    const size_t q1 = s.find('"', q0 + 1);
    const size_t b0 = s.find('[', q1);
    const size_t b1 = s.find(']', b0);
    if (q1 == std::string::npos || b0 == std::string::npos || b1 == std::string::npos) return false;
    const std::string key = s.substr(q0 + 1, q1 - q0 - 1);
    int choice = 0;
    double cost = 0.0;
    if (std::sscanf(s.substr(b0 + 1, b1 - b0 - 1).c_str(), "%d , %lf", &choice, &cost) != 2) return false;
    parsed[key] = Entry{choice, cost < 0.0 ? std::numeric_limits<double>::infinity() : cost};
    p = b1;
  }
  std::lock_guard<std::mutex> lk(mu_);
  for (auto& kv : parsed) table_[kv.first] = kv.second;
  return true;
}

}  // namespace lkg

extern "C" {

void lkg_autotune_enable(int on) { lkg::Autotuner::instance().set_enabled(on != 0); }

int lkg_autotune_report(char* out, int cap) {
  const std::string s = lkg::Autotuner::instance().report();
  if (out && cap > 0) {
    std::strncpy(out, s.c_str(), cap - 1);
    out[cap - 1] = 0;
  }
  return (int)s.size() + 1;
}

int lkg_autotune_record(const char* key, const int* candidates, const double* costs, int n) {
  if (!key || n <= 0 || !candidates || !costs) {
    lkg::set_last_error("lkg_autotune_record: empty key or candidate list");
    return -1;
  }
  const int r = lkg::Autotuner::instance().record(key, std::vector<int>(candidates, candidates + n),
                                                  std::vector<double>(costs, costs + n));
  if (r < 0) lkg::set_last_error("lkg_autotune_record: no candidate has a finite cost");
  return r;
}

int lkg_autotune_lookup(const char* key, int fallback) {
  return key ? lkg::Autotuner::instance().lookup(key, fallback) : fallback;
}

int lkg_autotune_save(const char* path) {
  if (!path || !lkg::Autotuner::instance().save_file(path)) {
    lkg::set_last_error("lkg_autotune_save: cannot write the file");
    return -1;
  }
  return 0;
}

int lkg_autotune_load(const char* path) {
  if (!path || !lkg::Autotuner::instance().load_file(path)) {
    lkg::set_last_error("lkg_autotune_load: cannot read or parse the file");
    return -1;
  }
  return 0;
}

void lkg_autotune_clear(void) { lkg::Autotuner::instance().clear(); }

}  // extern "C"
