// stats.hpp -- per-kernel launch counters and CUDA-event timings (measured on the launching stream).
//
// Every kernel launch of the library goes through a LaunchTimer: the launch count per kernel name is always kept;
// when timing is enabled each launch is bracketed by two events on its own stream and its algorithmic work (flops,
// bytes) is recorded, so a caller can derive achieved TFLOP/s or GB/s per kernel from live runs.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>

namespace lkg {

void stats_set_enabled(bool on);
bool stats_enabled();
void stats_reset();
// "name\tlaunches\ttimed_launches\tms\tflops\tbytes\n" per kernel (synchronises pending events)
std::string stats_report();
long long stats_total_launches();
// launch count per kernel name of the calling thread's launches, and adding (sign +1) or removing (-1) such counts:
// a replayed CUDA graph adds the launches it was captured with
std::map<std::string, long long> stats_thread_launch_counts();
void stats_add_launches(const std::map<std::string, long long>& counts, int sign);

class LaunchTimer {
 public:
  LaunchTimer(const char* kernel, cudaStream_t st, double flops, double bytes);
  ~LaunchTimer();
  LaunchTimer(const LaunchTimer&) = delete;
  LaunchTimer& operator=(const LaunchTimer&) = delete;

 private:
  const char* name_;
  cudaStream_t st_;
  double flops_, bytes_;
  cudaEvent_t e0_ = nullptr;
};

}  // namespace lkg
