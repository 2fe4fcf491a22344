/* Stand-in for boost/random/variate_generator.hpp: binds an engine (held by reference when the
 * template argument is a reference) to a distribution.  Test infrastructure only. */
#ifndef REF_SHIM_BOOST_VARIATE_GENERATOR_HPP
#define REF_SHIM_BOOST_VARIATE_GENERATOR_HPP
namespace boost {
template <class Engine, class Distribution>
class variate_generator {
 public:
  typedef typename Distribution::result_type result_type;
  variate_generator(Engine e, Distribution d) : eng_(e), dist_(d) {}
  result_type operator()() { return dist_(eng_); }
 private:
  Engine eng_;
  Distribution dist_;
};
}
#endif
