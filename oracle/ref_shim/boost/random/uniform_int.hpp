/* Stand-in for boost/random/uniform_int.hpp.  boost's integer method for a 32-bit engine and a
 * range [min, max] narrower than the engine's: bucket = 2^32-1 div (max-min+1), plus one when
 * (2^32-1) mod (max-min+1) == max-min; the result is the engine's draw divided by the bucket,
 * drawn again while it exceeds max-min.  A full 32-bit range returns the draw itself.  (It maps
 * draws differently from std::uniform_int_distribution.)  Test infrastructure only. */
#ifndef REF_SHIM_BOOST_UNIFORM_INT_HPP
#define REF_SHIM_BOOST_UNIFORM_INT_HPP
#include <cstdint>
namespace boost {
using std::uint32_t;
template <class IntType = int>
class uniform_int {
 public:
  typedef IntType result_type;
  explicit uniform_int(IntType min_arg = 0, IntType max_arg = 9) : min_(min_arg), max_(max_arg) {}
  IntType min() const { return min_; }
  IntType max() const { return max_; }
  template <class Engine>
  IntType operator()(Engine& eng) const {
    const uint32_t range = static_cast<uint32_t>(max_) - static_cast<uint32_t>(min_);
    const uint32_t brange = 0xffffffffu;
    if (range == brange) return static_cast<IntType>(static_cast<uint32_t>(min_) + static_cast<uint32_t>(eng()));
    uint32_t bucket = brange / (range + 1u);
    if (brange % (range + 1u) == range) ++bucket;
    for (;;) {
      const uint32_t r = static_cast<uint32_t>(eng()) / bucket;
      if (r <= range) return static_cast<IntType>(static_cast<uint32_t>(min_) + r);
    }
  }
 private:
  IntType min_, max_;
};
}
#endif
