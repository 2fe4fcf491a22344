/* Stand-in for boost/shared_array.hpp: a reference-counted owner of a new[] array with
 * indexing.  Test infrastructure only. */
#ifndef REF_SHIM_BOOST_SHARED_ARRAY_HPP
#define REF_SHIM_BOOST_SHARED_ARRAY_HPP
#include <cstddef>
#include <memory>
#include "boost/assert.hpp"
namespace boost {
template <class T>
class shared_array {
 public:
  shared_array() {}
  explicit shared_array(T* p) : p_(p, std::default_delete<T[]>()) {}
  T& operator[](std::ptrdiff_t i) const { return p_.get()[i]; }
  T* get() const { return p_.get(); }
  void reset() { p_.reset(); }
  void reset(T* p) { p_.reset(p, std::default_delete<T[]>()); }
  explicit operator bool() const { return p_.get() != nullptr; }
  long use_count() const { return p_.use_count(); }
 private:
  std::shared_ptr<T> p_;
};
}
#endif
