// Minimal project-written stand-in for the three members of boost::dynamic_bitset
// that the reference headers use (construct (n, value), test/set/reset, operator[]).
// Test infrastructure only: it lets the reference compile here without Boost.
#ifndef ORACLE_SHIM_DYNAMIC_BITSET_HPP
#define ORACLE_SHIM_DYNAMIC_BITSET_HPP
#include <cstddef>
#include <cstdint>
#include <vector>
namespace boost {
template <typename Block = unsigned long>
class dynamic_bitset {
 public:
  typedef std::size_t size_type;
  class reference {
   public:
    reference(std::uint64_t* w, std::uint64_t m) : w_(w), m_(m) {}
    operator bool() const { return (*w_ & m_) != 0; }
    reference& operator=(bool v) { if (v) *w_ |= m_; else *w_ &= ~m_; return *this; }
   private:
    std::uint64_t* w_; std::uint64_t m_;
  };
  dynamic_bitset() : n_(0) {}
  // As in Boost: the second argument is an integer whose low bits seed the first bits.
  explicit dynamic_bitset(size_type n, unsigned long value = 0) : n_(n), w_((n + 63) / 64, 0) {
    for (size_type i = 0; i < 64 && i < n; ++i) if ((value >> i) & 1UL) set(i);
  }
  size_type size() const { return n_; }
  bool test(size_type i) const { return (w_[i >> 6] >> (i & 63)) & 1ULL; }
  dynamic_bitset& set(size_type i) { w_[i >> 6] |= (1ULL << (i & 63)); return *this; }
  dynamic_bitset& set() { for (auto& x : w_) x = ~0ULL; trim(); return *this; }
  dynamic_bitset& reset(size_type i) { w_[i >> 6] &= ~(1ULL << (i & 63)); return *this; }
  dynamic_bitset& reset() { for (auto& x : w_) x = 0; return *this; }
  bool operator[](size_type i) const { return test(i); }
  reference operator[](size_type i) { return reference(&w_[i >> 6], 1ULL << (i & 63)); }
 private:
  void trim() { if (n_ & 63) w_.back() &= (1ULL << (n_ & 63)) - 1; }
  size_type n_;
  std::vector<std::uint64_t> w_;
};
}  // namespace boost
#endif
