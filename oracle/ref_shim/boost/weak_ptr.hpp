/* Stand-in for boost/weak_ptr.hpp (std::weak_ptr).  Test infrastructure only. */
#ifndef REF_SHIM_BOOST_WEAK_PTR_HPP
#define REF_SHIM_BOOST_WEAK_PTR_HPP
#include <memory>
namespace boost {
using std::weak_ptr;
}
#endif
