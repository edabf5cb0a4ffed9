// stats.cpp -- per-kernel launch counters and CUDA-event timings.
#include "stats.hpp"

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <vector>

#include "../../include/libkriging_gb300.h"
#include "common.cuh"

namespace lkg {

namespace {

struct Acc {
  long long launches = 0, timed = 0;
  double ms = 0.0, flops = 0.0, bytes = 0.0;
};

struct Pending {
  std::string name;
  cudaEvent_t e0, e1;
  double flops, bytes;
};

struct Registry {
  std::mutex mu;
  bool enabled = false;
  std::map<std::string, Acc> acc;
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  long long total = 0;

  cudaEvent_t get_event() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    LKG_CUDA(cudaEventCreate(&e));
    return e;
  }
  void drain() {  // caller holds mu
    for (auto& p : pending) {
      LKG_CUDA(cudaEventSynchronize(p.e1));
      float ms = 0.f;
      LKG_CUDA(cudaEventElapsedTime(&ms, p.e0, p.e1));
      Acc& a = acc[p.name];
      a.timed++;
      a.ms += ms;
      a.flops += p.flops;
      a.bytes += p.bytes;
      pool.push_back(p.e0);
      pool.push_back(p.e1);
    }
    pending.clear();
  }
};

Registry& reg() {
  static Registry r;
  return r;
}

}  // namespace

void stats_set_enabled(bool on) {
  std::lock_guard<std::mutex> lk(reg().mu);
  reg().enabled = on;
}

bool stats_enabled() { return reg().enabled; }

void stats_reset() {
  std::lock_guard<std::mutex> lk(reg().mu);
  reg().drain();
  reg().acc.clear();
  reg().total = 0;
}

long long stats_total_launches() {
  std::lock_guard<std::mutex> lk(reg().mu);
  return reg().total;
}

namespace {
thread_local std::map<std::string, long long> t_launches;  // this thread's launches per kernel name
}  // namespace

std::map<std::string, long long> stats_thread_launch_counts() { return t_launches; }

void stats_add_launches(const std::map<std::string, long long>& counts, int sign) {
  std::lock_guard<std::mutex> lk(reg().mu);
  for (auto& kv : counts) {
    reg().acc[kv.first].launches += sign * kv.second;
    reg().total += sign * kv.second;
  }
}

std::string stats_report() {
  std::lock_guard<std::mutex> lk(reg().mu);
  reg().drain();
  std::ostringstream o;
  o.precision(17);
  for (auto& kv : reg().acc)
    o << kv.first << "\t" << kv.second.launches << "\t" << kv.second.timed << "\t" << kv.second.ms << "\t"
      << kv.second.flops << "\t" << kv.second.bytes << "\n";
  return o.str();
}

LaunchTimer::LaunchTimer(const char* kernel, cudaStream_t st, double flops, double bytes)
    : name_(kernel), st_(st), flops_(flops), bytes_(bytes) {
  t_launches[name_]++;
  Registry& r = reg();
  std::lock_guard<std::mutex> lk(r.mu);
  r.acc[name_].launches++;
  r.total++;
  if (r.enabled) {
    e0_ = r.get_event();
    LKG_CUDA(cudaEventRecord(e0_, st_));
  }
}

LaunchTimer::~LaunchTimer() {
  if (!e0_) return;
  Registry& r = reg();
  std::lock_guard<std::mutex> lk(r.mu);
  cudaEvent_t e1 = r.get_event();
  if (cudaEventRecord(e1, st_) == cudaSuccess) r.pending.push_back({name_, e0_, e1, flops_, bytes_});
}

}  // namespace lkg

extern "C" {

void lkg_stats_enable(int on) { lkg::stats_set_enabled(on != 0); }

void lkg_stats_reset(void) { lkg::stats_reset(); }

int lkg_stats_report(char* out, int cap) {
  try {
    const std::string s = lkg::stats_report();
    if (out && cap > 0) {
      const size_t k = std::min<size_t>(s.size(), (size_t)cap - 1);
      std::memcpy(out, s.data(), k);
      out[k] = 0;
    }
    return (int)s.size() + 1;
  } catch (...) {
    return -1;
  }
}

}  // extern "C"
