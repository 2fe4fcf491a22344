/* Stand-in for boost/assert.hpp (reached through boost's smart-pointer headers):
 * BOOST_ASSERT is the C assert.  Test infrastructure only. */
#ifndef REF_SHIM_BOOST_ASSERT_HPP
#define REF_SHIM_BOOST_ASSERT_HPP
#include <cassert>
#ifndef BOOST_ASSERT
#define BOOST_ASSERT(expr) assert(expr)
#endif
#endif
