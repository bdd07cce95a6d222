// Minimal project-written stand-in for boost::detail::spinlock (lock/unlock/try_lock),
// used by the reference's per-node locks. Test infrastructure only.
#ifndef ORACLE_SHIM_SPINLOCK_HPP
#define ORACLE_SHIM_SPINLOCK_HPP
#include <atomic>
namespace boost { namespace detail {
class spinlock {
 public:
  spinlock() { f_.clear(); }
  bool try_lock() { return !f_.test_and_set(std::memory_order_acquire); }
  void lock() { while (f_.test_and_set(std::memory_order_acquire)) { } }
  void unlock() { f_.clear(std::memory_order_release); }
 private:
  std::atomic_flag f_;
};
}}  // namespace boost::detail
#endif
