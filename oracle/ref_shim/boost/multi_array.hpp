// TEST INFRASTRUCTURE: name shim so that the reference's headers compile
// without Boost.  The reference's TYPES.h only names boost::multi_array in
// typedefs; the paths compiled here never instantiate one, so a declaration
// is enough (any use would fail to compile, not misbehave).
#ifndef RSCHOL_REF_SHIM_BOOST_MULTI_ARRAY_HPP
#define RSCHOL_REF_SHIM_BOOST_MULTI_ARRAY_HPP
#include <cstddef>
namespace boost {
template <class T, std::size_t N>
class multi_array;
}
#endif
