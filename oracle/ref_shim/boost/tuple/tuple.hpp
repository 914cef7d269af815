// TEST INFRASTRUCTURE: name shim so that the reference's headers compile
// without Boost.  Forwards boost::tuple to the standard library's tuple;
// nothing on the reference paths compiled here instantiates it.
#ifndef RSCHOL_REF_SHIM_BOOST_TUPLE_HPP
#define RSCHOL_REF_SHIM_BOOST_TUPLE_HPP
#include <tuple>
namespace boost {
using std::get;
using std::make_tuple;
using std::tie;
using std::tuple;
}  // namespace boost
#endif
