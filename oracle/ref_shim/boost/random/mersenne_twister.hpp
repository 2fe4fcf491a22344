/* Stand-in for boost/random/mersenne_twister.hpp.  boost::mt19937 and std::mt19937 are the same
 * generator (MT19937, Matsumoto & Nishimura 1998: same default seed 5489, same seeding from one
 * 32-bit value, same output).  Test infrastructure only. */
#ifndef REF_SHIM_BOOST_MT_HPP
#define REF_SHIM_BOOST_MT_HPP
#include <cstdint>
#include <random>
namespace boost {
using std::uint32_t;
using std::int32_t;
typedef std::mt19937 mt19937;
}
#endif
