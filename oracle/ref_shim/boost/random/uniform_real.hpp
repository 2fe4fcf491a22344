/* Stand-in for boost/random/uniform_real.hpp (included by the reference, not used on its
 * reconstruction path).  Test infrastructure only. */
#ifndef REF_SHIM_BOOST_UNIFORM_REAL_HPP
#define REF_SHIM_BOOST_UNIFORM_REAL_HPP
namespace boost {
template <class RealType = double>
class uniform_real {
 public:
  typedef RealType result_type;
  explicit uniform_real(RealType a = 0, RealType b = 1) : a_(a), b_(b) {}
  template <class Engine>
  RealType operator()(Engine& eng) const {
    return a_ + (b_ - a_) * (static_cast<RealType>(eng()) / static_cast<RealType>(4294967296.0));
  }
 private:
  RealType a_, b_;
};
}
#endif
