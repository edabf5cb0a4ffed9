// autotune.hpp -- choices of schedule and precision made by measurement, kept in a table and persisted.
//
// A tuning key names one decision for one problem shape (for example "vecchia_wpb:k=0:d=3:m=30:n=1048576").
// choose() returns the tabled choice for the key, or measures every candidate with the caller's cost function
// (lower is better; +inf marks a candidate that is not allowed, e.g. one that misses an error budget), tables the
// cheapest (ties to the earlier candidate) and returns it.  The table is loaded from and saved to a small JSON
// object file: $LKG_TUNE_FILE when set, else no file (the table lives for the process).  Tuning is on unless
// disabled (lkg_autotune_enable(0) or LKG_AUTOTUNE=0), in which case choose() returns the caller's default.
#pragma once
#include <functional>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace lkg {

class Autotuner {
 public:
  static Autotuner& instance();

  int choose(const std::string& key, const std::vector<int>& candidates, int fallback,
             const std::function<double(int)>& cost);
  // the tabled choice, or `fallback` when the key is not in the table
  int lookup(const std::string& key, int fallback) const;
  // table a choice from costs measured elsewhere (same selection rule as choose)
  int record(const std::string& key, const std::vector<int>& candidates, const std::vector<double>& costs);
  void set_enabled(bool on) { enabled_ = on; }
  bool enabled() const { return enabled_; }
  // the table as "key<TAB>choice<TAB>cost<LF>" lines
  std::string report() const;
  // read / write the table as a JSON object {"key": [choice, cost], ...}; return false on I/O or parse errors
  bool load_file(const std::string& path);
  bool save_file(const std::string& path) const;
  void clear();
  void clear_key(const std::string& key);

 private:
  Autotuner();
  struct Entry {
    int choice;
    double cost;
  };
  mutable std::mutex mu_;
  std::map<std::string, Entry> table_;
  bool enabled_ = true;
  std::string file_;
};

// the selection rule: index of the lowest finite cost, ties to the earlier candidate; -1 when none is finite
int autotune_select(const std::vector<double>& costs);

}  // namespace lkg
