/*
 * Declarations the reference routines expect from headers that are not compiled
 * here (collision_utils.inl's INLINE_ATTR, libbng's CHECK_STIME_MAX and
 * RxnClass pathway lookup, rxn_utils.inl's trigger_intersect used by
 * exact_disk). Project-written; oracle only.
 */
#ifndef ORACLE_REF_PRELUDE_H
#define ORACLE_REF_PRELUDE_H

#include <cstdio>
#include <cfloat>
#include <ostream>
#include <sstream>

// logging and fatal errors of the release and region routines
#define mcell_error(...) do { fprintf(stderr, __VA_ARGS__); } while (0)
inline std::ostream& perf() {
  static std::ostringstream sink;
  sink.str("");
  return sink;
}
#ifndef FLT_INVALID
#define FLT_INVALID FLT_MAX
#endif

#define INLINE_ATTR __attribute__((always_inline))
// only reached from find_boundaries_occluding_disk, which is dead with use_expanded_list
#define mcell_internal_error(...) do { fprintf(stderr, __VA_ARGS__); } while (0)
#ifndef CHECK_STIME_MAX
#define CHECK_STIME_MAX(x) do { } while (0)
#endif

namespace MCell {
namespace RxnUtils {
// the reference's own search, compiled further down from src4/rxn_utils.inl
static int binary_search_double(const std::vector<double>& A, double match, int max_idx, double mult);
}  // namespace RxnUtils
}  // namespace MCell

namespace BNG {
// pathway for a probability drawn below max_fixed_p. libbng is not in the tree; MCell3's
// test_bimolecular selects it with binary_search_double over the class's cumulative
// probabilities up to index n_pathways - 1 (src/react_cond.c:166-172), and so does this
// stand-in, with the reference's binary_search_double (src4/rxn_utils.inl:301)
inline int RxnClass::get_pathway_index_for_probability(const double prob, const double mult) const {
  return MCell::RxnUtils::binary_search_double(cum_probs, prob, (int)cum_probs.size() - 1, mult);
}
} // namespace BNG

namespace MCell {
namespace RxnUtils {
// surface-class lookup for a volume molecule hitting wall w (stands in for
// find_mol_reactions_with_surf_classes); only the rxn type is consulted by exact_disk
static BNG::RxnClass g_transparent_class = [] { BNG::RxnClass c; c.type = BNG::RxnType::Transparent; return c; }();
static BNG::RxnClass g_absorb_class = [] { BNG::RxnClass c; c.type = BNG::RxnType::Standard; c.cum_probs.push_back(1e140); return c; }();
static inline void trigger_intersect(
    Partition& p, const Molecule& reacA, const orientation_t, const Wall& w, const bool,
    BNG::RxnClassesVector& matching_rxns) {
  auto it = p.wall_class.find(std::make_pair(w.index, reacA.species_id));
  if (it == p.wall_class.end() || it->second == 0) {
    return;
  }
  matching_rxns.push_back(it->second == 1 ? &g_transparent_class : &g_absorb_class);
}
} // namespace RxnUtils
} // namespace MCell

#endif
