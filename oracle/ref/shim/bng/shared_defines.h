/*
 * Project-written stand-in for libbng's bng/shared_defines.h.
 *
 * libbng (mcellteam/libbng) is an un-vendored sibling repository of the
 * reference; no version is pinned anywhere in the reference tree. MCell4's
 * src4/defines.h:36,90-113 imports the names below from it. This header supplies
 * them so that the reference's own hot-path routines can be compiled for the
 * oracle harness. Values:
 *   - EPS / SQRT_EPS / GIGANTIC follow MCell3's EPS_C, SQRT_EPS_C and GIGANTIC
 *     (src/mcell_structs.h:238-240), which MCell4 inherited;
 *   - distinguishable_* restate MCell3's distinguishable() (src/util.c:449);
 *   - the fp32 POS_EPS / POS_SQRT_EPS values are chosen here (libbng's are not
 *     in the tree) and are documented as such.
 * Test infrastructure only: nothing in the product links this.
 */
#ifndef ORACLE_SHIM_BNG_SHARED_DEFINES_H
#define ORACLE_SHIM_BNG_SHARED_DEFINES_H

#include <cmath>
#include <cstdint>
#include <cassert>
#include <climits>
#include <cfloat>
#include <set>
#include <string>
#include <sstream>
#include <vector>
#include <algorithm>

#ifndef POS_T_BYTES
#define POS_T_BYTES 8
#endif

typedef unsigned int uint;
const uint UINT_INVALID = 0xFFFFFFFFu;  // libbng's invalid value of an unsigned count

const uint ID_INVALID = UINT_MAX;
const uint INDEX_INVALID = UINT_MAX;
const uint ID_INVALID2 = UINT_MAX - 1;
const uint INDEX_INVALID2 = UINT_MAX - 1;

#define release_assert(x) assert(x)

namespace BNGCommon {

const double EPS = 1e-12;
const double SQRT_EPS = 1e-6;
const double DBL_GIGANTIC = 1e140;

#if POS_T_BYTES == 8
typedef double pos_t;
const pos_t POS_EPS = EPS;
const pos_t POS_SQRT_EPS = SQRT_EPS;
const pos_t POS_GIGANTIC = DBL_GIGANTIC;
#else
typedef float pos_t;
const pos_t POS_EPS = 1e-6f;
const pos_t POS_SQRT_EPS = 1e-3f;
const pos_t POS_GIGANTIC = FLT_MAX / 2;
#endif

// the routines multiply stime_t by Vec3, so it follows the position precision
typedef pos_t stime_t;
const stime_t STIME_EPS = POS_EPS;
const stime_t STIME_SQRT_EPS = POS_SQRT_EPS;
const stime_t STIME_GIGANTIC = POS_GIGANTIC;

static inline double fabs_f(const double x) { return std::fabs(x); }
static inline double sqrt_f(const double x) { return std::sqrt(x); }
static inline double pow_f(const double a, const double b) { return std::pow(a, b); }
static inline double floor_f(const double x) { return std::floor(x); }
static inline double round_f(const double x) { return std::round(x); }

static inline bool cmp_eq(const double a, const double b, const double eps) {
  return std::fabs(a - b) < eps;
}
static inline bool cmp_eq(const double a, const double b) {
  return cmp_eq(a, b, EPS);
}
static inline bool cmp_lt(const double a, const double b, const double eps) {
  return a < b && !cmp_eq(a, b, eps);
}

// same decision rule as MCell3 distinguishable() (src/util.c:449-462)
static inline bool distinguishable_f(double a, double b, double eps) {
  double c = std::fabs(a - b);
  a = std::fabs(a);
  if (a < 1) {
    a = 1;
  }
  b = std::fabs(b);
  if (b < a) {
    eps *= a;
  }
  else {
    eps *= b;
  }
  return c > eps;
}

static inline bool distinguishable_p(pos_t a, pos_t b, pos_t eps) {
  pos_t c = std::fabs(a - b);
  a = std::fabs(a);
  if (a < 1) {
    a = 1;
  }
  b = std::fabs(b);
  if (b < a) {
    eps *= a;
  }
  else {
    eps *= b;
  }
  return c > eps;
}

static inline std::string f_to_str(const double val, const int n = 17) {
  std::ostringstream out;
  out.precision(n);
  out << val;
  return out.str();
}

} // namespace BNGCommon

namespace BNG {
typedef uint species_id_t;
const species_id_t SPECIES_ID_INVALID = ID_INVALID;
typedef int orientation_t;
const orientation_t ORIENTATION_DOWN = -1;
const orientation_t ORIENTATION_NONE = 0;
const orientation_t ORIENTATION_UP = 1;
const orientation_t ORIENTATION_NOT_SET = 2;
const orientation_t ORIENTATION_DEPENDS_ON_SURF_COMP = 3;
} // namespace BNG

// ordered set with the small API subset MCell4 uses (vector-backed in libbng)
template<typename T>
class uint_set {
public:
  typedef typename std::set<T>::const_iterator const_iterator;
  void insert(const T& v) { s.insert(v); }
  void insert_unique(const T& v) { s.insert(v); }
  void erase_existing(const T& v) { s.erase(v); }
  size_t count(const T& v) const { return s.count(v); }
  size_t size() const { return s.size(); }
  bool empty() const { return s.empty(); }
  void clear() { s.clear(); }
  const_iterator begin() const { return s.begin(); }
  const_iterator end() const { return s.end(); }
  bool operator==(const uint_set& o) const { return s == o.s; }
private:
  std::set<T> s;
};

// hash set used for crossed subpartitions; iteration order is irrelevant to the
// routines compiled here (collisions are sorted by time afterwards)
template<typename T>
class uint_dense_hash_set {
public:
  typedef typename std::set<T>::const_iterator const_iterator;
  void insert(const T& v) { s.insert(v); }
  size_t count(const T& v) const { return s.count(v); }
  size_t size() const { return s.size(); }
  bool empty() const { return s.empty(); }
  void clear() { s.clear(); }
  void clear_no_resize() { s.clear(); }
  void resize(size_t) { }
  const_iterator begin() const { return s.begin(); }
  const_iterator end() const { return s.end(); }
private:
  std::set<T> s;
};

#endif
