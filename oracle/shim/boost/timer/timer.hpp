// Minimal project-written stand-in for boost::timer::auto_cpu_timer: elapsed().wall in
// nanoseconds, and a one-line report on destruction. Test infrastructure only.
#ifndef ORACLE_SHIM_TIMER_HPP
#define ORACLE_SHIM_TIMER_HPP
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <ctime>
namespace boost { namespace timer {
typedef std::int_least64_t nanosecond_type;
struct cpu_times { nanosecond_type wall, user, system; };
class auto_cpu_timer {
 public:
  auto_cpu_timer() : t0_(std::chrono::steady_clock::now()), c0_(std::clock()) {}
  ~auto_cpu_timer() {
    cpu_times t = elapsed();
    double cpu = double(std::clock() - c0_) / CLOCKS_PER_SEC;
    std::printf(" %.6fs wall, %.6fs CPU\n", t.wall / 1e9, cpu);
  }
  cpu_times elapsed() const {
    cpu_times t;
    t.wall = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0_).count();
    t.user = nanosecond_type(double(std::clock() - c0_) / CLOCKS_PER_SEC * 1e9);
    t.system = 0;
    return t;
  }
 private:
  std::chrono::steady_clock::time_point t0_;
  std::clock_t c0_;
};
}}  // namespace boost::timer
#endif
