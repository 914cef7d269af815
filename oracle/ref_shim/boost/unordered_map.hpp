// TEST INFRASTRUCTURE: name shim so that the reference's headers compile
// without Boost (boost::unordered_map -> std::unordered_map).
#ifndef RSCHOL_REF_SHIM_BOOST_UNORDERED_MAP_HPP
#define RSCHOL_REF_SHIM_BOOST_UNORDERED_MAP_HPP
#include <unordered_map>
namespace boost {
using std::unordered_map;
}
#endif
