/* Project-written stand-in for boost::container::small_vector (boost is absent);
 * only the std::vector subset that MCell4's hot-path routines use. Oracle only. */
#ifndef ORACLE_SHIM_SMALL_VECTOR
#define ORACLE_SHIM_SMALL_VECTOR
#include <vector>
namespace boost { namespace container {
template<typename T, size_t N> class small_vector: public std::vector<T> {
public:
  using std::vector<T>::vector;
};
} }
#endif
