/* Project-written stand-in for boost::container::flat_set (boost is absent). Oracle only. */
#ifndef ORACLE_SHIM_FLAT_SET
#define ORACLE_SHIM_FLAT_SET
#include <set>
namespace boost { namespace container {
template<typename T> class flat_set: public std::set<T> { };
} }
#endif
