/* Stand-in for boost/shared_ptr.hpp: the reference uses boost::shared_ptr only as an owning
 * reference-counted pointer, which std::shared_ptr provides.  Test infrastructure (builds the
 * reference from its own sources as the parity oracle); never part of the product. */
#ifndef REF_SHIM_BOOST_SHARED_PTR_HPP
#define REF_SHIM_BOOST_SHARED_PTR_HPP
#include <memory>
#include "boost/assert.hpp"
namespace boost {
using std::shared_ptr;
using std::weak_ptr;
using std::dynamic_pointer_cast;
using std::static_pointer_cast;
}
#endif
