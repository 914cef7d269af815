// TEST INFRASTRUCTURE: name shim so that the reference's headers compile
// without Boost (boost::unordered_set -> std::unordered_set).
#ifndef RSCHOL_REF_SHIM_BOOST_UNORDERED_SET_HPP
#define RSCHOL_REF_SHIM_BOOST_UNORDERED_SET_HPP
#include <unordered_set>
namespace boost {
using std::unordered_set;
}
#endif
