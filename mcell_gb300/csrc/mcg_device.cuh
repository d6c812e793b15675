// Device side of the volume-molecule diffuse-react step.
//
// One thread diffuses one molecule for one time step. The per-molecule work
// restates MCell4's DiffuseReactEvent::diffuse_vol_molecule / ray_trace_vol
// (src4/diffuse_react_event.cpp:367-780) and the routines they call:
//   collect_crossed_subparts / collect_neighboring_subparts  collision_utils_subparts.inl:38-300
//   get_displacement_up_to_partition_boundary                 collision_utils.inl:48-114
//   get_closest_wall_collision / collide_wall / jump_away_line collision_utils.inl:568-914
//   collide_mol                                               collision_utils.inl:464-515
//   reflect_from_wall                                         collision_utils.inl:1711-1747
//   cross_transparent_wall (non-compartment branch)           diffuse_react_event.cpp:3062-3094
//   sort_collisions_by_time                                   diffuse_react_event.cpp:341-364
//   exact_disk                                                exact_disk_utils.inl:840-1145
//   test_bimolecular / test_intersect / time_of_unimol         rxn_utils.inl:336-414, :593-626, :721-735
// with the same operation order, so the fp64 instantiation (built with
// -fmad=false) reproduces the reference's wall hits, subpartitions and reaction
// decisions exactly for identical inputs.
//
// What differs from the reference is the data layout and the parallel
// schedule: molecules are SoA records sorted by (subpartition, species) at the
// start of each iteration, partners are read from those sorted ranges (their
// start-of-iteration positions) instead of per-subpartition hash sets, walls
// of a subpartition are a CSR list, and reactions are claimed with atomics and
// resolved deterministically (see mcg_kernels.cuh).
#pragma once

#include "mcg_math.cuh"

// inlining of the fp32 side guard (run at the end of most segments)
#ifndef MCG_GUARD_INLINE
#define MCG_GUARD_INLINE __forceinline__
#endif

// occupants whose positions one thread loads together in the partner scan
#ifndef MCG_OCC_BATCH
#define MCG_OCC_BATCH 1
#endif

namespace mcg {

constexpr int MAXSP = 16;
constexpr int MAXC = 16;        // vol-vol collision candidates per page of a ray trace (earliest first)
constexpr int MAXSET = 48;      // subpartitions a ray trace's partner list holds
constexpr int MAX_REDO = 256;   // edge/vertex re-tries in one get_closest_wall_collision
constexpr int MAX_BOUNCES = 4096;
constexpr uint32_t NONE = 0xFFFFFFFFu;

// device status bits (OR-ed into a status word; the host maps them to MCG_ERR_*)
constexpr uint32_t ST_CAPACITY = 1u << 0;
constexpr uint32_t ST_ESCAPE = 1u << 1;
constexpr uint32_t ST_WATCHDOG = 1u << 2;
// exact fallbacks taken (counted, results unchanged): more candidates than one page
// holds (later pages refilled in time order), more partner subpartitions than the list
// holds (partners scanned along the walk, candidates deduplicated)
constexpr uint32_t ST_COLL_OVERFLOW = 1u << 3;
constexpr uint32_t ST_SET_OVERFLOW = 1u << 4;
// the bits that end a trace (the fallback bits only count)
constexpr uint32_t ST_ERRORS = ST_CAPACITY | ST_ESCAPE | ST_WATCHDOG;

// molecule meta word (w lane of the position record): species in bits 0-7, the
// schedule flag in bit 8, counted-volume membership in bits 9-15, the replica
// (model) the molecule belongs to in bits 16-31
constexpr uint32_t META_SPECIES_MASK = 0xFFu;
constexpr uint32_t META_SCHEDULE_UNIMOL = 1u << 8;  // MOLECULE_FLAG_SCHEDULE_UNIMOL_RXN
constexpr uint32_t META_CV_SHIFT = 9;   // bits 9-15: inside counted object k (membership, updated at crossings)
constexpr uint32_t MAX_COUNTED = 7;
constexpr uint32_t META_REP_SHIFT = 16;
constexpr uint32_t MAX_REPLICAS = 1u << 16;
__host__ __device__ __forceinline__ uint32_t make_meta(uint32_t species, uint32_t rep, uint32_t flags = 0) {
  return species | flags | (rep << META_REP_SHIFT);
}
__host__ __device__ __forceinline__ uint32_t meta_rep(uint32_t m) { return m >> META_REP_SHIFT; }
__host__ __device__ __forceinline__ uint32_t meta_cv(uint32_t m) { return (m >> META_CV_SHIFT) & 0x7Fu; }

// replica modes: advancing, frozen (finished, kept until collected), dropped at the next sort
constexpr uint32_t REP_RUN = 0, REP_FROZEN = 1, REP_DROP = 2;

template <typename T>
struct Eps;
template <>
struct Eps<double> {
  static constexpr double pos = 1e-12;       // POS_EPS (libbng; MCell3 EPS_C)
  static constexpr double pos_sqrt = 1e-6;   // POS_SQRT_EPS
  static constexpr double stime = 1e-12;     // STIME_EPS
};
template <>
struct Eps<float> {
  static constexpr float pos = 1e-6f;
  static constexpr float pos_sqrt = 1e-3f;
  static constexpr float stime = 1e-6f;
};
constexpr double EPS = 1e-12;  // time EPS (libbng EPS)
constexpr double TIME_FOREVER = 1e20;
constexpr double GIGANTIC = 1e140;
constexpr double MY_PI = 3.14159265358979323846;

template <typename T>
struct alignas(4 * sizeof(T)) P4 {
  T x, y, z, w;
};

__device__ __forceinline__ uint32_t meta_of(const P4<float>& p) { return __float_as_uint(p.w); }
__device__ __forceinline__ uint32_t meta_of(const P4<double>& p) {
  return (uint32_t)__double_as_longlong(p.w);
}
__device__ __forceinline__ void set_meta(P4<float>& p, uint32_t m) { p.w = __uint_as_float(m); }
__device__ __forceinline__ void set_meta(P4<double>& p, uint32_t m) {
  p.w = __longlong_as_double((long long)m);
}

constexpr int MAXPW = 4;  // pathways of one reaction class

// species and reaction tables (read-only on the device). A reaction class (one per
// reactant pair, one per unimolecular reactant) holds its pathways' cumulative
// probabilities (bimolecular) or rates x time step (unimolecular) and their products
// (-1 = none), as BNG::RxnClass's cum_probs.
struct Chem {
  int nsp;
  int nuni;
  double space_step[MAXSP];
  double unimol_k[MAXSP];               // k_tot per time step (last cumulative rate), < 0: none
  double uni_cum[MAXSP][MAXPW];
  double bimol_p[MAXSP][MAXSP];         // max_fixed_p (last cumulative probability), < 0: none
  double bimol_cum[MAXSP][MAXSP][MAXPW];
  uint32_t partners[MAXSP];             // bit b: species b reacts with this species
  uint32_t can_volwall[MAXSP];          // has a non-reflective wall class somewhere
  int8_t uni_npw[MAXSP];
  int8_t uni_prod[MAXSP][MAXPW][2];
  int8_t bimol_npw[MAXSP][MAXSP];
  int8_t bimol_prod[MAXSP][MAXSP][MAXPW][2];
};

template <typename T>
struct WallFace {
  V3<T> u, v, v0, v1, v2;
  T uv1u, uv2u, uv2v;
};

// One replica (independent model) as the kernels see it: its partition grid,
// walls, reaction tables, random stream and place in the shared sort-key space.
// The engine keeps one per replica in a device table; a molecule finds its own
// through the replica index in its meta word.
template <typename T>
struct Geo {
  V3<T> origin, opposite;
  T part_edge, sp_edge, sp_rcp, R;
  int nsub, nsub2, nsp;
  uint32_t n3;                // subpartitions (nsub^3)
  float rcp_n, rcp_n2;        // 1 / nsub, 1 / nsub^2 (index decoding without integer division)
  uint32_t oct_shift;         // 3: occupants binned per subpartition octant, 0: per subpartition
  uint32_t kbase;             // first sort key of the replica; keys are (species, subpartition, octant)
  uint32_t rep;               // replica index
  uint32_t it0;               // engine iteration at which the replica's own iteration 0 runs
  uint32_t mode;              // REP_RUN / REP_FROZEN / REP_DROP
  uint32_t it_end;            // engine iteration from which the replica is frozen (its iteration budget)
  uint64_t seed;              // Config.seed of the replica
  const P4<T>* wrej;          // normal xyz, distance to origin
  const WallFace<T>* wface;
  const uint32_t* wsp_off;    // CSR: walls per subpartition (ascending wall index)
  const uint32_t* wsp_list;   // wall indices
  const uint64_t* wsp_cells;  // per entry: cells of the subpartition's 4x4x4 grid the wall reaches
  // per subpartition listing 1-64 walls: the block (of 64) of wsp_cellent holding, per
  // cell of its 4x4x4 grid, the bit mask of its entries that reach the cell; NONE
  // for other subpartitions
  const uint32_t* wsp_cm;
  const uint64_t* wsp_cellent;
  const uint8_t* wall_class;  // [wall * nsp + species]: 0 reflect, 1 transparent, 2 absorptive
  const Chem* chem;
  // fp32 engines: the wall constants in fp64 for the tie-breaks, 16 per wall (normal
  // xyz, d, unit_u xyz, unit_v xyz, v0 xyz, uv_vert1_u, uv_vert2 u v); null in fp64
  const double* w64;
  const uint16_t* wall_obj;   // geometry object of each wall (releases inside objects), or null
  uint32_t n_cv;              // counted objects (volumes whose contents are counted)
  uint16_t cv_obj[MAX_COUNTED];
  // the grid in fp64 (the inside tests run in fp64 in both engines)
  double origin64[3], sp_edge64, sp_rcp64;
};

// counted-object slots a wall belongs to (walls of counted objects only)
template <typename T>
__device__ __forceinline__ uint32_t cv_bits_of_wall(const Geo<T>& g, uint32_t wi) {
  if (!g.n_cv) return 0;
  const uint16_t o = g.wall_obj[wi];
  uint32_t f = 0;
  for (uint32_t k = 0; k < g.n_cv; k++)
    if (g.cv_obj[k] == o) f |= 1u << k;
  return f;
}

// molecules at the start of the iteration, sorted by key (replica, species, subpartition, octant)
template <typename T>
struct Cells {
  const P4<T>* pos;
  const uint64_t* uid;
  const uint32_t* start;  // [nkeys + 1]
  const uint8_t* dead;    // optional: partners already used up this iteration
  int maxc, maxset;       // capacities of a candidate page and of the partner list (tests lower them)
};

template <typename T>
struct TraceOut {
  int status;  // 0 finished, 1 reacted with a partner, 2 absorbed, 3 error
  V3<T> pos;
  uint32_t subpart;
  uint32_t partner;  // index into Cells
  T t_abs;           // time of the reaction / absorption
  int pathway;       // pathway of the reaction class that fired (status 1)
  V3<T> rxn_pos;
  T elapsed, t_steps;
  uint32_t err;
  // counted-volume membership set by transparent crossings up to the reaction
  // (update_counted_volume_id_when_crossing_wall, collision_utils.inl:1637-1694: a hit
  // on a counted object's front face goes inside it, on its back face outside): the
  // objects crossed and their membership after the last crossing
  uint32_t cv_mask, cv_val;
};

// a molecule's counted-volume bits after the crossings of a trace
template <typename T>
__device__ __forceinline__ uint32_t cv_after(uint32_t cv, const TraceOut<T>& r) {
  return (cv & ~r.cv_mask) | (r.cv_val & r.cv_mask);
}

// ------------------------------------------------------------------ draws

// production: Philox stream of the molecule-step
struct PhiloxDraws {
  Philox ph;
  __device__ __forceinline__ uint32_t u32() { return ph.next_u32(); }
  __device__ __forceinline__ bool overrun() const { return false; }
};

// harness: injected 32-bit draws
struct InjectedDraws {
  const uint32_t* d;
  uint32_t n, used;
  bool over;
  __device__ __forceinline__ uint32_t u32() {
    if (used >= n) {
      over = true;
      return 0;
    }
    return d[used++];
  }
  __device__ __forceinline__ bool overrun() const { return over; }
};

// rng_dbl: 32-bit draw scaled by 2^-32 (isaac64_dbl32)
template <class D>
__device__ __forceinline__ double draw_dbl(D& d) {
  return (double)d.u32() * (1.0 / 4294967296.0);
}

// events recorded by the harness (no-op in production)
struct NoEvents {
  __device__ __forceinline__ void put(int, uint64_t, int, double, double, double, double, double) {}
};
// events of one chosen molecule in production runs (diagnostics), null = off
struct MaybeEvents {
  double* out;
  __device__ __forceinline__ void put(int kind, uint64_t index, int side, double t_rel, double t_abs, double x,
                                      double y, double z) {
    if (!out) return;
    int n = (int)out[6];
    if (n < 32) {
      double* e = out + 9 + n * 8;
      e[0] = kind;
      e[1] = (double)index;
      e[2] = side;
      e[3] = t_rel;
      e[4] = t_abs;
      e[5] = x;
      e[6] = y;
      e[7] = z;
    }
    out[6] = n + 1;
  }
};
struct EventLog {
  double* out;  // MCG_TRACE_RESULT_SIZE doubles
  __device__ void put(int kind, uint64_t index, int side, double t_rel, double t_abs, double x, double y,
                      double z) {
    int n = (int)out[6];
    if (n < 32) {
      double* e = out + 9 + n * 8;
      e[0] = kind;
      e[1] = (double)index;
      e[2] = side;
      e[3] = t_rel;
      e[4] = t_abs;
      e[5] = x;
      e[6] = y;
      e[7] = z;
    }
    out[6] = n + 1;
  }
};

// ------------------------------------------------------------------ partition helpers

template <typename T>
__device__ __forceinline__ bool in_partition(const Geo<T>& g, V3<T> p) {
  return p.x >= g.origin.x && p.y >= g.origin.y && p.z >= g.origin.z && p.x < g.opposite.x &&
         p.y < g.opposite.y && p.z < g.opposite.z;
}
// subpartition 3-D index (Partition::get_subpart_3d_indices). Clamped to the grid:
// positions a rounding step outside the partition stay addressable.
template <typename T>
__device__ __forceinline__ void sub3(const Geo<T>& g, V3<T> p, int& x, int& y, int& z) {
  V3<T> r = p - g.origin;
  x = min(max((int)(r.x * g.sp_rcp), 0), g.nsub - 1);
  y = min(max((int)(r.y * g.sp_rcp), 0), g.nsub - 1);
  z = min(max((int)(r.z * g.sp_rcp), 0), g.nsub - 1);
}
template <typename T>
__device__ __forceinline__ uint32_t sub_of3(const Geo<T>& g, int x, int y, int z) {
  return (uint32_t)(x + y * g.nsub + z * g.nsub2);
}
// subpartition index -> grid coordinates without integer division: float reciprocals
// and a +-1 correction (indices are below 300^3 < 2^25, so the estimate is off by at
// most one)
template <typename T>
__device__ __forceinline__ void decode_sp(const Geo<T>& g, uint32_t sp, int& x, int& y, int& z) {
  const int n = g.nsub, n2 = g.nsub2;
  int zz = (int)((float)sp * g.rcp_n2);
  int r = (int)sp - zz * n2;
  if (r < 0) {
    zz--;
    r += n2;
  } else if (r >= n2) {
    zz++;
    r -= n2;
  }
  int yy = (int)((float)r * g.rcp_n);
  int xx = r - yy * n;
  if (xx < 0) {
    yy--;
    xx += n;
  } else if (xx >= n) {
    yy++;
    xx -= n;
  }
  x = xx;
  y = yy;
  z = zz;
}

template <typename T>
__device__ __forceinline__ uint32_t subpart_of(const Geo<T>& g, V3<T> p) {
  int x, y, z;
  sub3(g, p, x, y, z);
  return sub_of3(g, x, y, z);
}
// octants (bit o: x half o&1, y half o&2, z half o&4) of subpartition sp that the box
// [lo, hi] overlaps
template <typename T>
__device__ __forceinline__ uint32_t octants_touched(const Geo<T>& g, uint32_t sp, V3<T> lo, V3<T> hi) {
  int ix, iy, iz;
  decode_sp(g, sp, ix, iy, iz);
  const T h = g.sp_edge * (T)0.5;
  const V3<T> mid = v3<T>(add_rn(add_rn(g.origin.x, mul_rn((T)ix, g.sp_edge)), h),
                          add_rn(add_rn(g.origin.y, mul_rn((T)iy, g.sp_edge)), h),
                          add_rn(add_rn(g.origin.z, mul_rn((T)iz, g.sp_edge)), h));
  const uint32_t ax = (lo.x < mid.x ? 1u : 0u) | (hi.x >= mid.x ? 2u : 0u);
  const uint32_t ay = (lo.y < mid.y ? 1u : 0u) | (hi.y >= mid.y ? 2u : 0u);
  const uint32_t az = (lo.z < mid.z ? 1u : 0u) | (hi.z >= mid.z ? 2u : 0u);
  // expand the per-axis half sets into the 8 octant bits
  const uint32_t mx = (ax & 1 ? 0x55u : 0u) | (ax & 2 ? 0xAAu : 0u);
  const uint32_t my = (ay & 1 ? 0x33u : 0u) | (ay & 2 ? 0xCCu : 0u);
  const uint32_t mz = (az & 1 ? 0x0Fu : 0u) | (az & 2 ? 0xF0u : 0u);
  return mx & my & mz;
}
// box around the segment p -> p + d, grown by m in each direction
// cells of subpartition sp's 4x4x4 grid (bit x + 4y + 16z) that the box [lo, hi]
// touches; the outer faces are not tested (the box may reach past the subpartition)
template <typename T>
__device__ __forceinline__ uint64_t cells_touched(const Geo<T>& g, uint32_t sp, V3<T> lo, V3<T> hi) {
  int ix, iy, iz;
  decode_sp(g, sp, ix, iy, iz);
  const T q = g.sp_edge * (T)0.25;
  const V3<T> o = g.origin + cmul(v3<T>((T)ix, (T)iy, (T)iz), v3<T>(g.sp_edge, g.sp_edge, g.sp_edge));
  auto axis = [q](T l, T h, T base) -> uint32_t {
    const T q1 = base + q, q2 = base + (T)2 * q, q3 = base + (T)3 * q;
    return (l < q1 ? 1u : 0u) | (l < q2 && h >= q1 ? 2u : 0u) | (l < q3 && h >= q2 ? 4u : 0u) | (h >= q3 ? 8u : 0u);
  };
  const uint32_t ax = axis(lo.x, hi.x, o.x), ay = axis(lo.y, hi.y, o.y), az = axis(lo.z, hi.z, o.z);
  // x: the same nibble in all 16 (y, z) positions; y: 4-bit groups per z; z: 16-bit groups
  const uint64_t mx = (uint64_t)ax * 0x1111111111111111ull;
  const uint64_t gy = (ay & 1 ? 0x000Full : 0) | (ay & 2 ? 0x00F0ull : 0) | (ay & 4 ? 0x0F00ull : 0) | (ay & 8 ? 0xF000ull : 0);
  const uint64_t my = gy * 0x0001000100010001ull;
  const uint64_t mz = (az & 1 ? 0xFFFFull : 0) | (az & 2 ? 0xFFFF0000ull : 0) | (az & 4 ? 0xFFFF00000000ull : 0) |
                      (az & 8 ? 0xFFFF000000000000ull : 0);
  return mx & my & mz;
}

template <typename T>
__device__ __forceinline__ void seg_box(V3<T> p, V3<T> d, T m, V3<T>& lo, V3<T>& hi) {
  const V3<T> e = p + d;
  lo = v3<T>(min(p.x, e.x) - m, min(p.y, e.y) - m, min(p.z, e.z) - m);
  hi = v3<T>(max(p.x, e.x) + m, max(p.y, e.y) + m, max(p.z, e.z) + m);
}
template <typename T>
__device__ __forceinline__ V3<T> guard_zero(V3<T> a) {
  const T tiny = (T)1.17549435082228750797e-38;  // FLT_MIN, as guard_zero_div uses
  if (a.x == 0) a.x = tiny;
  if (a.y == 0) a.y = tiny;
  if (a.z == 0) a.z = tiny;
  return a;
}
template <typename T>
__device__ __forceinline__ bool distinguishable(T a, T b, T eps) {
  T c = tabs(a - b);
  a = tabs(a);
  if (a < 1) a = 1;
  b = tabs(b);
  if (b < a)
    eps *= a;
  else
    eps *= b;
  return c > eps;
}
template <typename T>
__device__ __forceinline__ T abs_max_2vec(V3<T> a, V3<T> b) {
  return tmax(tmax(tmax(tabs(a.x), tabs(b.x)), tmax(tabs(a.y), tabs(b.y))), tmax(tabs(a.z), tabs(b.z)));
}

// get_displacement_up_to_partition_boundary (collision_utils.inl:48-114)
template <typename T>
__device__ __noinline__ V3<T> disp_up_to_partition_boundary(const Geo<T>& g, V3<T> pos, V3<T> disp) {
  V3<T> nz = guard_zero(disp);
  V3<T> dir = v3<T>(nz.x > 0 ? 1 : 0, nz.y > 0 ? 1 : 0, nz.z > 0 ? 1 : 0);
  V3<T> edges = g.origin + scale(dir, g.part_edge);
  V3<T> diff = edges - pos;
  T hit = 1;
  if (tabs(diff.x) < Eps<T>::pos || tabs(diff.y) < Eps<T>::pos || tabs(diff.z) < Eps<T>::pos) {
    return v3<T>(0, 0, 0);
  }
  V3<T> t = cdiv(diff, nz);
  if (t.x >= 0 && t.x < t.y && t.x <= t.z)
    hit = t.x;
  else if (t.y >= 0 && t.y <= t.z)
    hit = t.y;
  else if (t.z >= 0)
    hit = t.z;
  return scale(disp, hit - Eps<T>::stime);
}

// ------------------------------------------------------------------ subpartition walk

// Visits the subpartitions the segment pos -> pos+disp crosses, in order
// (collect_crossed_subparts, collision_utils_subparts.inl:127-300). The walk is
// re-entrant so the wall search can stop early without storing the list.
template <typename T>
struct Walk {
  V3<T> cp, disp, rcp;
  int cx, cy, cz, ax, ay, az, dx, dy, dz;
  uint32_t cur, dest;
  int steps;
  bool done;

  __device__ void start(const Geo<T>& g, V3<T> pos, uint32_t start_sp, V3<T> d) {
    disp = d;
    V3<T> dest_p = pos + d;
    V3<T> nz = guard_zero(d);
    dx = nz.x > 0;
    dy = nz.y > 0;
    dz = nz.z > 0;
    decode_sp(g, start_sp, cx, cy, cz);
    int ex, ey, ez;
    sub3(g, dest_p, ex, ey, ez);
    dest = sub_of3(g, ex, ey, ez);
    cur = start_sp;
    cp = pos;
    ax = dx ? 1 : -1;
    ay = dy ? 1 : -1;
    az = dz ? 1 : -1;
    rcp = cdiv(v3<T>(1, 1, 1), nz);
    done = (cur == dest);
    steps = 0;
  }
  // advances to the next crossed subpartition; false when the walk is over
  __device__ bool next(const Geo<T>& g) {
    if (done) return false;
    const T e = g.sp_edge;
    V3<T> edges = v3<T>(add_rn(add_rn(g.origin.x, mul_rn((T)cx, e)), mul_rn((T)dx, e)),
                        add_rn(add_rn(g.origin.y, mul_rn((T)cy, e)), mul_rn((T)dy, e)),
                        add_rn(add_rn(g.origin.z, mul_rn((T)cz, e)), mul_rn((T)dz, e)));
    V3<T> diff = edges - cp;
    V3<T> t = cmul(diff, rcp);
    if (t.x < t.y && t.x <= t.z) {
      cp = v3<T>(add_rn(cp.x, mul_rn(disp.x, t.x)), add_rn(cp.y, mul_rn(disp.y, t.x)), add_rn(cp.z, mul_rn(disp.z, t.x)));
      cx += ax;
      if (cx < 0 || cx >= g.nsub) {
        done = true;
        return false;
      }
    } else if (t.y <= t.z) {
      cp = v3<T>(add_rn(cp.x, mul_rn(disp.x, t.y)), add_rn(cp.y, mul_rn(disp.y, t.y)), add_rn(cp.z, mul_rn(disp.z, t.y)));
      cy += ay;
      if (cy < 0 || cy >= g.nsub) {
        done = true;
        return false;
      }
    } else {
      cp = v3<T>(add_rn(cp.x, mul_rn(disp.x, t.z)), add_rn(cp.y, mul_rn(disp.y, t.z)), add_rn(cp.z, mul_rn(disp.z, t.z)));
      cz += az;
      if (cz < 0 || cz >= g.nsub) {
        done = true;
        return false;
      }
    }
    cur = sub_of3(g, cx, cy, cz);
    if (cur == dest || ++steps > 3 * g.nsub) done = true;
    return true;
  }
};

struct SubSet {
  uint32_t s[MAXSET];
  int n, cap;
  uint32_t n3;  // number of subpartitions (indices are checked against it)
  bool overflow;
  __device__ __forceinline__ void insert(uint32_t v) {
    if (v >= n3) return;
    for (int i = 0; i < n; i++)
      if (s[i] == v) return;
    if (n < cap)
      s[n++] = v;
    else
      overflow = true;
  }
  template <typename T>
  __device__ __forceinline__ void insert3(const Geo<T>& g, int x, int y, int z) {
    insert(sub_of3(g, x, y, z));
  }
};

// The same set as a bit mask over a 4x4x4 window of subpartitions (registers, no
// dynamic indexing). Bit dx | dy << 2 | dz << 4 stands for subpartition
// (x0 + dx, y0 + dy, z0 + dz); an index outside the grid is skipped exactly as
// SubSet skips it, and an insertion outside the window marks the mask unusable
// (the caller then builds the list instead).
struct SubMask {
  uint64_t bits;
  int x0, y0, z0;
  uint32_t n3;
  bool bad;
  template <typename T>
  __device__ __forceinline__ void insert3(const Geo<T>& g, int x, int y, int z) {
    if (sub_of3(g, x, y, z) >= n3) return;
    const unsigned dx = (unsigned)(x - x0), dy = (unsigned)(y - y0), dz = (unsigned)(z - z0);
    if ((dx | dy | dz) > 3u) {
      bad = true;
      return;
    }
    bits |= 1ull << (dx | (dy << 2) | (dz << 4));
  }
};

// collect_neighboring_subparts (collision_utils_subparts.inl:38-122). Out of line:
// it runs at the start, at each crossing and at the end of a segment, and one copy
// instead of three keeps the diffuse kernel's instruction footprint smaller (the
// kernel stalls on instruction fetch; measured 7 % faster).
template <typename T, class Set>
__device__ __forceinline__ void collect_neighbors_body(const Geo<T>& g, V3<T> pos, int ix, int iy, int iz, T r,
                                                       Set& st) {
  T part_len = g.part_edge;
  V3<T> rel = pos - g.origin;
  V3<T> plus = rel + v3<T>(r, r, r);
  V3<T> minus = rel - v3<T>(r, r, r);
  V3<T> b = cmul(v3<T>((T)ix, (T)iy, (T)iz), v3<T>(g.sp_edge, g.sp_edge, g.sp_edge));
  int xd = 0, yd = 0, zd = 0;
  if (minus.x < b.x && minus.x > (T)0.0) {
    st.insert3(g, ix - 1, iy, iz);
    xd = -1;
  } else if (plus.x > add_rn(b.x, g.sp_edge) && plus.x < part_len) {
    st.insert3(g, ix + 1, iy, iz);
    xd = 1;
  }
  if (minus.y < b.y && minus.y > (T)0.0) {
    st.insert3(g, ix, iy - 1, iz);
    yd = -1;
  } else if (plus.y > add_rn(b.y, g.sp_edge) && plus.y < part_len) {
    st.insert3(g, ix, iy + 1, iz);
    yd = 1;
  }
  if (minus.z < b.z && minus.z > (T)0.0) {
    st.insert3(g, ix, iy, iz - 1);
    zd = -1;
  } else if (plus.z > add_rn(b.z, g.sp_edge) && plus.z < part_len) {
    st.insert3(g, ix, iy, iz + 1);
    zd = 1;
  }
  if (xd && yd) st.insert3(g, ix + xd, iy + yd, iz);
  if (xd && zd) st.insert3(g, ix + xd, iy, iz + zd);
  if (yd && zd) st.insert3(g, ix, iy + yd, iz + zd);
  if (xd && yd && zd) st.insert3(g, ix + xd, iy + yd, iz + zd);
}
template <typename T, class Set>
__device__ __noinline__ void collect_neighbors(const Geo<T>& g, V3<T> pos, int ix, int iy, int iz, T r, Set& st) {
  collect_neighbors_body<T, Set>(g, pos, ix, iy, iz, r, st);
}

// collect_neighbors for the mask, returning what it adds: the caller's mask is not
// passed by reference to the out-of-line call, so it can stay in registers
struct MaskAdd {
  uint64_t bits;
  bool bad;
};
template <typename T>
__device__ __noinline__ MaskAdd neighbors_mask(const Geo<T>& g, V3<T> pos, int ix, int iy, int iz, T r, int x0, int y0,
                                               int z0, uint32_t n3) {
  SubMask m;
  m.bits = 0;
  m.x0 = x0;
  m.y0 = y0;
  m.z0 = z0;
  m.n3 = n3;
  m.bad = false;
  collect_neighbors_body<T, SubMask>(g, pos, ix, iy, iz, r, m);
  return MaskAdd{m.bits, m.bad};
}

// subpartitions whose occupants can collide with the segment: crossed ones and
// their neighbours within R*sqrt(2) (the molecule half of collect_crossed_subparts)
// (in three parts: the start subpartition, each crossing of the walk, the end point;
// trace_molecule runs them along its wall walk, which visits the same crossings)
template <typename T>
__device__ __forceinline__ T collect_radius(const Geo<T>& g) {
  return g.R * (T)1.41421356238;  // POS_SQRT2
}
template <typename T, class Set>
__device__ __forceinline__ void collect_start(const Geo<T>& g, V3<T> pos, int sx, int sy, int sz, Set& st) {
  st.insert3(g, sx, sy, sz);
  collect_neighbors(g, pos, sx, sy, sz, collect_radius(g), st);
}
template <typename T>
__device__ __forceinline__ void add_neighbors(const Geo<T>& g, V3<T> pos, int ix, int iy, int iz, SubMask& st) {
  const MaskAdd a = neighbors_mask(g, pos, ix, iy, iz, collect_radius(g), st.x0, st.y0, st.z0, st.n3);
  st.bits |= a.bits;
  st.bad = st.bad || a.bad;
}
template <typename T>
__device__ __forceinline__ void collect_start(const Geo<T>& g, V3<T> pos, int sx, int sy, int sz, SubMask& st) {
  st.insert3(g, sx, sy, sz);
  add_neighbors(g, pos, sx, sy, sz, st);
}
template <typename T, class Set>
__device__ __forceinline__ void collect_crossing(const Geo<T>& g, const Walk<T>& w, Set& st) {
  st.insert3(g, w.cx, w.cy, w.cz);
  collect_neighbors(g, w.cp, w.cx, w.cy, w.cz, collect_radius(g), st);
}
template <typename T>
__device__ __forceinline__ void collect_crossing(const Geo<T>& g, const Walk<T>& w, SubMask& st) {
  st.insert3(g, w.cx, w.cy, w.cz);
  add_neighbors(g, w.cp, w.cx, w.cy, w.cz, st);
}
template <typename T, class Set>
__device__ __forceinline__ void collect_end(const Geo<T>& g, V3<T> pos, V3<T> disp, Set& st) {
  V3<T> dest = pos + disp;
  int ex, ey, ez;
  sub3(g, dest, ex, ey, ez);
  collect_neighbors(g, dest, ex, ey, ez, collect_radius(g), st);
}
template <typename T>
__device__ __forceinline__ void collect_end(const Geo<T>& g, V3<T> pos, V3<T> disp, SubMask& st) {
  V3<T> dest = pos + disp;
  int ex, ey, ez;
  sub3(g, dest, ex, ey, ez);
  add_neighbors(g, dest, ex, ey, ez, st);
}
template <typename T, class Set>
__device__ void collect_for_molecules(const Geo<T>& g, V3<T> pos, uint32_t sp, V3<T> disp, Set& st) {
  int sx, sy, sz;
  decode_sp(g, sp, sx, sy, sz);
  collect_start(g, pos, sx, sy, sz, st);
  Walk<T> w;
  w.start(g, pos, sp, disp);
  while (w.next(g)) collect_crossing(g, w, st);
  collect_end(g, pos, disp, st);
}

// ------------------------------------------------------------------ walls

enum : int { CT_MISS = 0, CT_REDO = 1, CT_FRONT = 2, CT_BACK = 3 };

// jump_away_line (collision_utils.inl:568-603)
// `u`: its one 32-bit draw (the sign of the jump); returns the new move
template <typename T>
__device__ __noinline__ V3<T> jump_away_line(V3<T> p, T k, V3<T> A, V3<T> B, V3<T> n, uint32_t u, V3<T> v) {
  V3<T> e = B - A;
  T elen2 = dot(e, e);
  T le_1 = (T)1.0 / sqrt(elen2);
  e = cmul(e, v3<T>(le_1, le_1, le_1));
  V3<T> f;
  f.x = n.y * e.z - n.z * e.y;
  f.y = n.z * e.x - n.x * e.z;
  f.z = n.x * e.y - n.y * e.x;
  T tiny;
  if (sizeof(T) == 8) {
    tiny = Eps<T>::pos * (abs_max_2vec(p, v) + (T)1.0) / (k * tmax(tmax(tabs(f.x), tabs(f.y)), tabs(f.z)));
  } else {
    tiny = Eps<T>::pos_sqrt;  // fp32 branch of the reference
  }
  if ((u & 1) == 0) tiny = -tiny;
  v.x -= tiny * f.x;
  v.y -= tiny * f.y;
  v.z -= tiny * f.z;
  return v;
}

enum : int { PT_MISS = 0, PT_PARALLEL = 1, PT_HIT = 2 };

// plane part of collide_wall (collision_utils.inl:659-716): start and end on the same
// side (with the POS_EPS band) is a miss, a move inside the plane is re-tried,
// otherwise a = time of the crossing
template <typename S>
__device__ __forceinline__ int plane_test(S dd, S dv, S eps, S& a) {
  S d_eps;
  if (dd > 0) {
    d_eps = eps;
    if (dd < d_eps) d_eps = (S)0.5 * dd;
    if (dd + dv > d_eps) return PT_MISS;
  } else {
    d_eps = -eps;
    if (dd > d_eps) d_eps = (S)0.5 * dd;
    if (dd < 0 && dd + dv < d_eps) return PT_MISS;
  }
  if (dd == 0) return dv != 0 ? PT_MISS : PT_PARALLEL;
  a = (S)1.0 / dv;
  a *= -dd;
  return PT_HIT;
}

// in-triangle part of collide_wall (collision_utils.inl:718-810) at a plane crossing
// with coordinates b (along unit_u) and c (along unit_v) from vertex 0: outside,
// inside, or within eps of the edge v1-v2 / v2-v0 / v0-v1 (a re-try)
enum : int { TRI_OUT = 0, TRI_IN = 1, TRI_E12 = 2, TRI_E20 = 3, TRI_E01 = 4 };
template <typename S>
__device__ __forceinline__ int tri_test(S b, S c, S uv1u, S uv2u, S uv2v, S eps) {
  S f;
  if (uv2v < 0) {
    c = -c;
    f = -uv2v;
  } else {
    f = uv2v;
  }
  if (c > 0) {
    S gg = b * f;
    S h = c * uv2u;
    if (gg > h) {
      if (c * uv1u + gg < h + uv1u * uv2v) return TRI_IN;
      if (!distinguishable<S>(c * uv1u + gg, h + uv1u * uv2v, eps)) return TRI_E12;
      return TRI_OUT;
    }
    if (!distinguishable<S>(gg, h, eps)) return TRI_E20;
    return TRI_OUT;
  }
  if (!distinguishable<S>(c, (S)0.0, eps)) return TRI_E01;
  return TRI_OUT;
}

// fp32 tie-break of the plane test, in fp64 with the fp64 plane (the float
// position and move are exact in fp64): near the plane the fp32 side test can
// have the wrong sign (its error grows with the coordinates), letting a molecule
// moving outwards pass a reflective wall. Out of line: rarely taken.
// (results returned by value: nothing of the caller is passed by reference to these
// out-of-line calls, so its variables can stay in registers)
template <typename T>
struct PlaneFp64 {
  int pt;
  T a, dv;
};
template <typename T>
__device__ __noinline__ PlaneFp64<T> plane_test_fp64(const double* w64, V3<T> pos, V3<T> move) {
  const double ddd = (w64[0] * (double)pos.x + w64[1] * (double)pos.y + w64[2] * (double)pos.z) - w64[3];
  const double dvd = w64[0] * (double)move.x + w64[1] * (double)move.y + w64[2] * (double)move.z;
  double ad = 0;
  const int pt = plane_test<double>(ddd, dvd, (double)Eps<T>::pos, ad);
  return PlaneFp64<T>{pt, (T)ad, (T)dvd};
}

// fp32 tie-break near an edge or vertex: the float in-triangle test is within its
// own rounding there, and the float constants of two triangles sharing an edge do
// not meet exactly (a ray can pass between them, or re-try at a face diagonal
// until the watchdog). The crossing and the in-triangle test are redone in fp64
// with the fp64 wall constants and band; only a crossing within that band of the
// edge is re-tried. Returns a TRI_* code (crossing time and point updated), or
// -1 when the fp64 plane test misses. Out of line: rarely taken.
template <typename T>
struct EdgeFp64 {
  int tr;
  T ct, dv;
  V3<T> cpos;
};
template <typename T>
__device__ __noinline__ EdgeFp64<T> edge_test_fp64(const double* w64, V3<T> pos, V3<T> move, int tr, T ct,
                                                   V3<T> cpos, T dv) {
  const double px = pos.x, py = pos.y, pz = pos.z, mx = move.x, my = move.y, mz = move.z;
  const double ddd = (w64[0] * px + w64[1] * py + w64[2] * pz) - w64[3];
  const double dvd = w64[0] * mx + w64[1] * my + w64[2] * mz;
  double ad = 0;
  const int ptd = plane_test<double>(ddd, dvd, Eps<double>::pos, ad);
  if (ptd == PT_MISS) return EdgeFp64<T>{-1, ct, dv, cpos};
  if (ptd != PT_HIT) return EdgeFp64<T>{tr, ct, dv, cpos};
  const double cx = px + mx * ad, cy = py + my * ad, cz = pz + mz * ad;
  const double lx = cx - w64[10], ly = cy - w64[11], lz = cz - w64[12];
  const double bd = lx * w64[4] + ly * w64[5] + lz * w64[6];
  const double cd = lx * w64[7] + ly * w64[8] + lz * w64[9];
  const int t2 = tri_test<double>(bd, cd, w64[13], w64[14], w64[15], Eps<double>::pos);
  return EdgeFp64<T>{t2, (T)ad, (T)dvd, v3<T>((T)cx, (T)cy, (T)cz)};
}

// collide_wall (collision_utils.inl:629-812)
template <typename T, class D>
__device__ int collide_wall(const Geo<T>& g, V3<T> pos, uint32_t wi, D& draws, V3<T>& move, T& ct, V3<T>& cpos) {
  const P4<T> rj = g.wrej[wi];
  V3<T> normal = v3<T>(rj.x, rj.y, rj.z);
  T dp = dot(normal, pos);
  T dv = dot(normal, move);
  T dd = dp - rj.w;
  T a;
  int pt;
  if (sizeof(T) == 4 && tabs(dd) < (T)1e-2) {
    const PlaneFp64<T> q = plane_test_fp64<T>(g.w64 + 16 * (size_t)wi, pos, move);
    pt = q.pt;
    a = q.a;
    dv = q.dv;
  } else {
    pt = plane_test<T>(dd, dv, Eps<T>::pos, a);
  }
  if (pt == PT_MISS) return CT_MISS;
  if (pt == PT_PARALLEL) {
    a = (abs_max_2vec(pos, move) + (T)1.0) * Eps<T>::pos;
    if ((draws.u32() & 1) == 0) a = -a;
    move = move - cmul(v3<T>(a, a, a), normal);
    return CT_REDO;
  }
  ct = a;
  cpos = pos + scale(move, a);
  const WallFace<T>& w = g.wface[wi];
  V3<T> local = cpos - w.v0;
  // fp32: a crossing within the rounding of this computation of an edge (16 ulp of
  // the coordinates: cpos and v0 each carry about one) is decided in fp64 by
  // edge_test_fp64. POS_EPS alone is far narrower than fp32's rounding away from the
  // origin, where the fp32 test would otherwise pick the neighbour across the edge.
  T teps = Eps<T>::pos;
  if (sizeof(T) == 4) {
    const T mag = tmax(tmax(tabs(cpos.x), tabs(cpos.y)), tmax(tabs(cpos.z), (T)1));
    teps = tmax(teps, mag * (T)(16.0 * 1.1920928955078125e-07));
  }
  int tr = tri_test<T>(dot(local, w.u), dot(local, w.v), w.uv1u, w.uv2u, w.uv2v, teps);
  if (sizeof(T) == 4 && tr >= TRI_E12) {
    const EdgeFp64<T> q = edge_test_fp64<T>(g.w64 + 16 * (size_t)wi, pos, move, tr, ct, cpos, dv);
    tr = q.tr;
    ct = q.ct;
    cpos = q.cpos;
    dv = q.dv;
    if (tr < 0) return CT_MISS;
  }
  if (tr == TRI_IN) return dv > 0 ? CT_BACK : CT_FRONT;
  if (tr == TRI_OUT) return CT_MISS;
  if (tr == TRI_E12)
    move = jump_away_line(pos, ct, w.v1, w.v2, normal, draws.u32(), move);
  else if (tr == TRI_E20)
    move = jump_away_line(pos, ct, w.v2, w.v0, normal, draws.u32(), move);
  else
    move = jump_away_line(pos, ct, w.v0, w.v1, normal, draws.u32(), move);
  return CT_REDO;
}

// fp32 tie-break in fp64: puts `pos` on the given side (+1 front, -1 back) of the
// wall plane by a margin of a few ulps of its coordinates (~1 pm at 1 um) when
// rounding left it on the plane or on the other side. Returns true if it moved.
// With near_only, only a position within the margin of the plane is moved.
template <typename T>
__device__ bool keep_side(const P4<T>& rj, double side, V3<T>& pos, bool near_only = false) {
  const double ddn = ((double)pos.x * (double)rj.x + (double)pos.y * (double)rj.y + (double)pos.z * (double)rj.z) -
                     (double)rj.w;
  const double margin =
      8.0 * 1.1920928955078125e-07 * (double)tmax(tmax(tabs(pos.x), tabs(pos.y)), tmax(tabs(pos.z), (T)1));
  if (ddn * side >= margin) return false;
  if (near_only && (ddn >= margin || ddn <= -margin)) return false;
  const T push = (T)(side * (margin - ddn * side));
  pos = pos + scale(v3<T>(rj.x, rj.y, rj.z), push);
  return true;
}

// The entries of subpartition sp whose wall reaches a cell of `om`, in ascending order
// (the order the reference tests its wall list in). For a subpartition of at most 64
// walls the candidates come from the per-cell entry masks (one load per touched cell);
// otherwise every entry's cell mask is tested.
template <typename T>
struct WallEntries {
  uint32_t b, e, k;
  uint64_t cand, om;
  bool masked;
  __device__ __forceinline__ void start(const Geo<T>& g, uint32_t sp, uint64_t cells) {
    b = g.wsp_off[sp];
    e = g.wsp_off[sp + 1];
    om = cells;
    const uint32_t cm = g.wsp_cm[sp];
    masked = cm != NONE;
    k = b;
    cand = 0;
    if (masked) {
      if (cells == ~0ull) {
        cand = (e - b) >= 64 ? ~0ull : ((1ull << (e - b)) - 1);
      } else {
        const uint64_t* ce = g.wsp_cellent + (size_t)cm * 64;
        for (uint64_t m = cells; m; m &= m - 1) cand |= __ldg(ce + (__ffsll((long long)m) - 1));
      }
    }
  }
  // the next entry index, false when there is none
  __device__ __forceinline__ bool next(const Geo<T>& g, uint32_t& entry) {
    if (masked) {
      if (!cand) return false;
      entry = b + (uint32_t)(__ffsll((long long)cand) - 1);
      cand &= cand - 1;
      return true;
    }
    while (k < e) {
      const uint32_t q = k++;
      if (g.wsp_cells[q] & om) {
        entry = q;
        return true;
      }
    }
    return false;
  }
};

// fp32: moves `pos` off any wall plane of subpartition sp that it lies on (within
// keep_side's margin) to the side `ref` is on; `skip` is left alone. The point
// reached a rounded position on a segment from `ref` that crossed none of these
// walls (except `skip`).
template <typename T>
__device__ MCG_GUARD_INLINE void guard_sides(const Geo<T>& g, uint32_t sp, V3<T>& pos, V3<T> ref, uint32_t skip) {
  if (g.wsp_off[sp] == g.wsp_off[sp + 1]) return;  // no wall listed here
  V3<T> glo, ghi;
  seg_box(pos, v3<T>(0, 0, 0), (T)2e-2, glo, ghi);
  const uint64_t gm = cells_touched(g, sp, glo, ghi);
  WallEntries<T> it;
  it.start(g, sp, gm);
  uint32_t k;
  while (it.next(g, k)) {
    const uint32_t wi = g.wsp_list[k];
    if (wi == skip) continue;
    const P4<T> rj = g.wrej[wi];
    // cheap fp32 screen first; the fp64 side test only for points near the plane
    const T d1 = dot(v3<T>(rj.x, rj.y, rj.z), pos) - rj.w;
    if (tabs(d1) > (T)1e-2) continue;
    const double d0 = ((double)ref.x * (double)rj.x + (double)ref.y * (double)rj.y + (double)ref.z * (double)rj.z) -
                      (double)rj.w;
    keep_side(rj, d0 >= 0 ? 1.0 : -1.0, pos, true);
  }
}

// the same, out of line, for the rare sites (reflection and crossing points)
template <typename T>
__device__ __noinline__ V3<T> guard_sides_rare(const Geo<T>& g, uint32_t sp, V3<T> pos, V3<T> ref, uint32_t skip) {
  guard_sides(g, sp, pos, ref, skip);
  return pos;
}

template <typename T>
struct WallHit {
  int type;
  T t;
  V3<T> pos;
  uint32_t wall;
};

// get_closest_wall_collision (collision_utils.inl:819-914). In fp32 the reference
// also keeps hits that land in another subpartition as tentative ones (:885-893).
template <typename T, class D>
__device__ bool closest_wall_collision(const Geo<T>& g, V3<T> pos, uint32_t sp, uint32_t last_hit, D& draws,
                                       V3<T>& disp, WallHit<T>& closest, WallHit<T>& tentative,
                                       uint32_t& err) {
  if (g.wsp_off[sp] == g.wsp_off[sp + 1]) return false;  // no wall listed here
  int redo = 0;
restart:
  bool found = false;
  T closest_t = (T)1e20;
  // A wall can only be hit (or re-tried at an edge) where it meets the segment, so walls
  // that reach none of the octants the segment's box touches are skipped. The one
  // exception is collide_wall's re-try of a move lying exactly in a wall's plane
  // (dd == 0 && dv == 0), which happens wherever the triangle is; it needs a move
  // exactly perpendicular to the wall normal.
  // A move with an exactly zero component (e.g. nothing left after a reflection at
  // t = 1, or an axis-aligned injected move) is not filtered, so that re-try stays.
  V3<T> lo, hi;
  seg_box(pos, disp, g.sp_edge * (T)1e-3, lo, hi);
  const uint64_t om =
      (disp.x == 0 || disp.y == 0 || disp.z == 0) ? ~0ull : cells_touched(g, sp, lo, hi);
  WallEntries<T> it;
  it.start(g, sp, om);
  uint32_t k;
  while (it.next(g, k)) {
    const uint32_t wi = g.wsp_list[k];
    if (wi == last_hit) continue;
    T t;
    V3<T> cp;
    int ct = collide_wall(g, pos, wi, draws, disp, t, cp);
    if (ct == CT_REDO) {
      if (++redo > MAX_REDO || draws.overrun()) {
        err |= ST_WATCHDOG;
        return false;
      }
      goto restart;
    } else if (ct != CT_MISS) {
      if (subpart_of(g, cp) != sp) {
        if (sizeof(T) == 4 && t < tentative.t) {
          tentative.type = ct;
          tentative.t = t;
          tentative.pos = cp;
          tentative.wall = wi;
        }
        continue;
      }
      if (t < closest_t) {
        found = true;
        closest_t = t;
        closest.type = ct;
        closest.t = t;
        closest.pos = cp;
        closest.wall = wi;
      }
    }
  }
  return found;
}

// ------------------------------------------------------------------ inside a closed object

// wall constants in fp64 (the fp64 engine's own, the fp32 engine's tie-break copy)
template <typename T>
__device__ __forceinline__ void wall_fp64(const Geo<T>& g, uint32_t wi, double* c) {
  if (sizeof(T) == 4) {
    for (int k = 0; k < 16; k++) c[k] = g.w64[16 * (size_t)wi + k];
  } else {
    const P4<T> r = g.wrej[wi];
    const WallFace<T> f = g.wface[wi];
    const double q[16] = {(double)r.x,    (double)r.y,    (double)r.z,    (double)r.w,    (double)f.u.x, (double)f.u.y,
                          (double)f.u.z,  (double)f.v.x,  (double)f.v.y,  (double)f.v.z,  (double)f.v0.x, (double)f.v0.y,
                          (double)f.v0.z, (double)f.uv1u, (double)f.uv2u, (double)f.uv2v};
    for (int k = 0; k < 16; k++) c[k] = q[k];
  }
}

// The inside tests (counted-volume membership at upload and release, releases into a
// closed object) count a ray's wall crossings as the reference does, in fp64 from the
// walls' fp64 constants. The fp32 engine's translation unit allows fused multiply-adds,
// so the arithmetic here is written with round-to-nearest intrinsics: both engines
// reproduce the reference's fp64 decisions bit for bit.
__device__ __forceinline__ double rn_dot3(double ax, double ay, double az, double bx, double by, double bz) {
  return __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
}
__device__ __forceinline__ bool rn_distinguishable(double a, double b, double eps) {
  const double c = fabs(__dsub_rn(a, b));
  a = fabs(a);
  if (a < 1) a = 1;
  b = fabs(b);
  eps = b < a ? __dmul_rn(eps, a) : __dmul_rn(eps, b);
  return c > eps;
}

// collide_wall (collision_utils.inl:629-812) for the inside tests, with a wall's fp64
// constants c[16] (wall_fp64): CT_MISS, CT_FRONT, CT_BACK, or CT_REDO where the
// reference re-tries (a ray in the wall's plane or through an edge, which makes its
// inside tests give up: must_redo_test)
static __device__ __noinline__ int collide_wall_rn(const double* c, V3<double> pos, V3<double> move) {
  const double dp = rn_dot3(c[0], c[1], c[2], pos.x, pos.y, pos.z);
  const double dv = rn_dot3(c[0], c[1], c[2], move.x, move.y, move.z);
  const double dd = __dsub_rn(dp, c[3]);
  double a = 0;
  const int pt = plane_test<double>(dd, dv, Eps<double>::pos, a);
  if (pt == PT_MISS) return CT_MISS;
  if (pt == PT_PARALLEL) return CT_REDO;
  const double lx = __dsub_rn(__dadd_rn(pos.x, __dmul_rn(a, move.x)), c[10]);
  const double ly = __dsub_rn(__dadd_rn(pos.y, __dmul_rn(a, move.y)), c[11]);
  const double lz = __dsub_rn(__dadd_rn(pos.z, __dmul_rn(a, move.z)), c[12]);
  const double b = rn_dot3(lx, ly, lz, c[4], c[5], c[6]);
  double cc = rn_dot3(lx, ly, lz, c[7], c[8], c[9]);
  const double uv1u = c[13], uv2u = c[14], uv2v = c[15];
  double f;
  if (uv2v < 0) {
    cc = -cc;
    f = -uv2v;
  } else {
    f = uv2v;
  }
  if (cc > 0) {
    const double gg = __dmul_rn(b, f), h = __dmul_rn(cc, uv2u);
    if (gg > h) {
      const double lhs = __dadd_rn(__dmul_rn(cc, uv1u), gg), rhs = __dadd_rn(h, __dmul_rn(uv1u, uv2v));
      if (lhs < rhs) return dv > 0 ? CT_BACK : CT_FRONT;
      return rn_distinguishable(lhs, rhs, Eps<double>::pos) ? CT_MISS : CT_REDO;
    }
    return rn_distinguishable(gg, h, Eps<double>::pos) ? CT_MISS : CT_REDO;
  }
  return rn_distinguishable(cc, 0.0, Eps<double>::pos) ? CT_MISS : CT_REDO;
}

// raycast_with_endpoints with compute_inputs_for_raycast_with_endpoints
// (collision_utils.inl:138-244): the subpartitions a ray from p1 to p2 visits, in
// order. Like the reference's, it ends as soon as the axis it would step along has
// reached p2's subpartition, which can be before p2's subpartition on the others.
struct RayCells {
  int ix, iy, iz, ex, ey, ez, dx, dy, dz, n, n2;
  double tx, ty, tz, gx, gy, gz;
  uint32_t sp;
  template <typename T>
  __device__ void start(const Geo<T>& g, V3<double> p1, V3<double> p2, V3<double> d) {
    n = g.nsub;
    n2 = g.nsub2;
    dx = d.x > 0 ? 1 : (d.x < 0 ? -1 : 0);
    dy = d.y > 0 ? 1 : (d.y < 0 ? -1 : 0);
    dz = d.z > 0 ? 1 : (d.z < 0 ? -1 : 0);
    const double ax = d.x == 0 ? Eps<double>::pos : fabs(d.x), ay = d.y == 0 ? Eps<double>::pos : fabs(d.y),
                 az = d.z == 0 ? Eps<double>::pos : fabs(d.z);
    const double rx = 1.0 / ax, ry = 1.0 / ay, rz = 1.0 / az;
    const double side = g.sp_edge64, rcp = g.sp_rcp64;
    gx = __dmul_rn(side, rx);
    gy = __dmul_rn(side, ry);
    gz = __dmul_rn(side, rz);
    ix = (int)__dmul_rn(__dsub_rn(p1.x, g.origin64[0]), rcp);
    iy = (int)__dmul_rn(__dsub_rn(p1.y, g.origin64[1]), rcp);
    iz = (int)__dmul_rn(__dsub_rn(p1.z, g.origin64[2]), rcp);
    ex = (int)__dmul_rn(__dsub_rn(p2.x, g.origin64[0]), rcp);
    ey = (int)__dmul_rn(__dsub_rn(p2.y, g.origin64[1]), rcp);
    ez = (int)__dmul_rn(__dsub_rn(p2.z, g.origin64[2]), rcp);
    sp = (uint32_t)(ix + iy * n + iz * n2);
    // the cell boundaries are multiples of the cell side from 0 (the partition's corner is one)
    const double mx = __dmul_rn(floor(__dmul_rn(p1.x, rcp)), side), my = __dmul_rn(floor(__dmul_rn(p1.y, rcp)), side),
                 mz = __dmul_rn(floor(__dmul_rn(p1.z, rcp)), side);
    tx = __dmul_rn(dx == -1 ? __dsub_rn(p1.x, mx) : __dsub_rn(__dadd_rn(mx, side), p1.x), rx);
    ty = __dmul_rn(dy == -1 ? __dsub_rn(p1.y, my) : __dsub_rn(__dadd_rn(my, side), p1.y), ry);
    tz = __dmul_rn(dz == -1 ? __dsub_rn(p1.z, mz) : __dsub_rn(__dadd_rn(mz, side), p1.z), rz);
  }
  // after visiting sp: to the next subpartition, false when the ray is done
  __device__ bool next() {
    if (tx <= ty && tx <= tz) {
      if (ix == ex) return false;
      tx = __dadd_rn(tx, gx);
      ix += dx;
      sp += (uint32_t)dx;
    } else if (ty <= tz) {
      if (iy == ey) return false;
      ty = __dadd_rn(ty, gy);
      iy += dy;
      sp += (uint32_t)(dy * n);
    } else {
      if (iz == ez) return false;
      tz = __dadd_rn(tz, gz);
      iz += dz;
      sp += (uint32_t)(dz * n2);
    }
    return true;
  }
};

template <typename T>
__device__ __forceinline__ bool listed_in(const Geo<T>& g, uint32_t sp, uint32_t wi) {
  if (sp >= g.n3) return false;
  uint32_t lo = g.wsp_off[sp], hi = g.wsp_off[sp + 1];  // ascending wall indices
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    const uint32_t v = g.wsp_list[mid];
    if (v == wi) return true;
    if (v < wi)
      lo = mid + 1;
    else
      hi = mid;
  }
  return false;
}

// Crossings of a ray from p to dst (moved by -POS_EPS on every axis, as the reference
// moves its displacement) with the walls of the objects `want` selects (a bit per
// counted-object slot, or the object itself): each wall counts once, at the first
// subpartition of the ray that lists it (get_num_crossed_walls_per_object /
// get_num_crossed_region_walls, collision_utils.inl:1328-1465). Returns the crossings
// per slot as parity bits, or NONE when the ray met an edge or lay in a wall's plane.
// `region` >= 0: count the walls of that object into bit 0 instead of the slots.
template <typename T>
__device__ uint32_t ray_parity(const Geo<T>& g, V3<double> p, V3<double> dst, int region) {
  const V3<double> d = v3<double>(__dsub_rn(__dsub_rn(dst.x, p.x), Eps<double>::pos),
                                  __dsub_rn(__dsub_rn(dst.y, p.y), Eps<double>::pos),
                                  __dsub_rn(__dsub_rn(dst.z, p.z), Eps<double>::pos));
  RayCells rc;
  rc.start(g, p, dst, d);
  uint32_t parity = 0;
  int k = 0;
  for (int guard = 0; guard < 3 * g.nsub + 3; guard++, k++) {
    const uint32_t sp = rc.sp;
    if (sp < g.n3) {
      for (uint32_t e = g.wsp_off[sp]; e < g.wsp_off[sp + 1]; e++) {
        const uint32_t wi = g.wsp_list[e];
        const uint32_t o = g.wall_obj[wi];
        uint32_t bits;
        if (region >= 0) {
          bits = o == (uint32_t)region ? 1u : 0u;
        } else {
          bits = 0;
          for (uint32_t q = 0; q < g.n_cv; q++)
            if (g.cv_obj[q] == o) bits |= 1u << q;
        }
        if (!bits) continue;
        double c[16];
        wall_fp64(g, wi, c);
        const int ct = collide_wall_rn(c, p, d);
        if (ct == CT_REDO) return NONE;
        if (ct == CT_MISS) continue;
        // counted once: skip when an earlier subpartition of the ray lists the wall
        bool seen = false;
        RayCells r2;
        r2.start(g, p, dst, d);
        for (int j = 0; j < k && !seen; j++) {
          seen = listed_in(g, r2.sp, wi);
          if (!r2.next()) break;
        }
        if (!seen) parity ^= bits;
      }
    }
    if (!rc.next()) break;
  }
  return parity;
}

// compute_counted_volume_for_pos (collision_utils.inl:1515-1545): the counted objects
// (bit q for slot q of cv_obj) whose walls a ray from p to the partition's corner,
// moved by (edge/11, edge/21, 0) subpartition edges, crosses an odd number of times;
// NONE when the ray met an edge (the reference stops there)
template <typename T>
__device__ uint32_t counted_volume_bits(const Geo<T>& g, V3<double> p) {
  const double e = g.sp_edge64;
  const V3<double> dst = v3<double>(__dadd_rn(g.origin64[0], e / 11.0), __dadd_rn(g.origin64[1], e / 21.0),
                                    g.origin64[2]);
  return ray_parity(g, p, dst, -1);
}

// is_point_inside_region_no_waypoints (collision_utils.inl:1484-1510) for the closed
// region made of object obj's walls, whose bounding box's low corner is llf: 1 inside,
// 0 outside, NONE when the ray met an edge
template <typename T>
__device__ uint32_t inside_region(const Geo<T>& g, V3<double> p, uint32_t obj, const double* llf) {
  const double e = g.sp_edge64;
  V3<double> dst = v3<double>(__dsub_rn(llf[0], Eps<double>::pos), __dsub_rn(llf[1], Eps<double>::pos),
                              __dsub_rn(llf[2], Eps<double>::pos));
  dst.x = __dadd_rn(dst.x, e / 11.0);
  dst.y = __dadd_rn(dst.y, e / 22.0);
  return ray_parity(g, p, dst, (int)obj);
}

// ------------------------------------------------------------------ collisions with molecules

// one vol-vol collision candidate: relative time and index of the partner; the
// collision point (pos + t * disp), the partner id and the reaction are looked up
// again when the candidate is processed
template <typename T>
struct VV {
  T t;
  uint32_t idx;
};

template <typename T>
struct Colls {
  VV<T> c[MAXC];
  int n;
  bool overflow;
  // sort_collisions_by_time order: time ascending, equal times by id descending
  __device__ __forceinline__ static bool before(const VV<T>& a, const VV<T>& b, const uint64_t* uid) {
    if (a.t < b.t) return true;
    if (a.t > b.t) return false;
    return uid[a.idx] > uid[b.idx];
  }
  // cap: the page's capacity (MAXC; tests lower it)
  __device__ void insert(const VV<T>& x, const uint64_t* uid, int cap) {
    int i = n;
    if (n == cap) {
      overflow = true;
      if (!before(x, c[cap - 1], uid)) return;
      i = cap - 1;
    } else {
      n++;
    }
    while (i > 0 && before(x, c[i - 1], uid)) {
      c[i] = c[i - 1];
      i--;
    }
    c[i] = x;
  }
};

// The collector of the exact fallbacks (out of line, rare): a later page of
// candidates takes only those after the last one of the previous page in
// sort_collisions_by_time order (the cursor); a partner scan along the walk visits
// subpartitions more than once and drops repeated candidates. A candidate evicted
// from a full page is always later than the page's last one, so it is refused again
// when it comes back: the pages together hold every candidate exactly once, in order.
template <typename T>
struct CollsX {
  Colls<T>& c;
  bool cursor, dedupe;
  T ct;
  uint64_t cuid;
  __device__ void insert(const VV<T>& x, const uint64_t* uid, int cap) {
    if (cursor && (x.t < ct || (x.t == ct && !(cuid > uid[x.idx])))) return;
    if (dedupe)
      for (int i = 0; i < c.n; i++)
        if (c.c[i].idx == x.idx) return;
    c.insert(x, uid, cap);
  }
};

// What a refill of a full candidate page needs to collect the segment's candidates
// again: kept in the stack frame (written only when a page overflows, through an
// out-of-line call), so that the common path holds none of it in registers.
template <typename T>
struct RefillState {
  SubMask sm;
  V3<T> mdisp;
  uint32_t sp;
  int mode;
};

// Occupants of a subpartition are binned by octant (key = ((subpart * 8 + octant) *
// n_species + species)). A partner can only satisfy collide_mol if it lies within R
// of the segment, i.e. inside the segment's bounding box grown by R, so octants
// outside that box are skipped: an exact filter (with a rounding margin) that does
// not change which partners are found.
template <typename T>
__device__ __forceinline__ uint32_t octant_of(const Geo<T>& g, V3<T> p, int ix, int iy, int iz) {
  V3<T> r = p - g.origin;
  const T half = (T)0.5;
  uint32_t o = 0;
  if (r.x * g.sp_rcp - (T)ix >= half) o |= 1;
  if (r.y * g.sp_rcp - (T)iy >= half) o |= 2;
  if (r.z * g.sp_rcp - (T)iz >= half) o |= 4;
  return o;
}

// collide_mol (collision_utils.inl:464-515) against every reacting occupant of the
// collected subpartitions
// occupants of one subpartition (the partner species' octant ranges the segment box touches)
template <typename T, class C>
__device__ __forceinline__ void occupants_of(const Geo<T>& g, const Cells<T>& cells, uint32_t self, V3<T> pos,
                                             V3<T> disp, uint32_t pmask, T movelen2, T sigma2, V3<T> lo, V3<T> hi,
                                             uint32_t sp, C& out) {
  const uint32_t om = g.oct_shift ? octants_touched(g, sp, lo, hi) : 1u;
  uint32_t m = pmask;
  while (m) {
    const int b = __ffs(m) - 1;
    m &= m - 1;
    // the octants of (subpartition, species) are consecutive keys, so a run of
    // consecutive octants is one range of occupants
    const uint32_t base = g.kbase + (((uint32_t)b * g.n3 + sp) << g.oct_shift);
    for (uint32_t oo = om; oo;) {
      const uint32_t o = (uint32_t)(__ffs(oo) - 1);
      const uint32_t run = (uint32_t)(__ffs(~(oo >> o)) - 1);
      oo &= ~(((1u << run) - 1u) << o);
      const uint32_t j0 = __ldg(cells.start + base + o), j1 = __ldg(cells.start + base + o + run);
      // MCG_OCC_BATCH occupants per round: their loads are issued together (latency overlap)
      for (uint32_t j4 = j0; j4 < j1; j4 += MCG_OCC_BATCH) {
        P4<T> q4[MCG_OCC_BATCH];
#pragma unroll
        for (int u = 0; u < MCG_OCC_BATCH; u++)
          if (j4 + u < j1) q4[u] = cells.pos[j4 + u];
#pragma unroll
        for (int u = 0; u < MCG_OCC_BATCH; u++) {
          const uint32_t j = j4 + u;
          if (j >= j1) break;
          const V3<T> dir = v3<T>(q4[u].x, q4[u].y, q4[u].z) - pos;
          const T d = dot_rn(dir, disp);
          if (d < 0) continue;
          if (d > movelen2) continue;
          const T dirlen2 = dot_rn(dir, dir);
          if (misses_disk(movelen2, dirlen2, d, sigma2)) continue;
          if (j == self) continue;
          if (cells.dead && cells.dead[j] == 2) continue;
          VV<T> c;
          c.t = d / movelen2;
          c.idx = j;
          out.insert(c, cells.uid, cells.maxc);
        }
      }
    }
  }
}

template <typename T, class C>
__device__ void collide_with_occupants(const Geo<T>& g, const Cells<T>& cells, uint32_t self, V3<T> pos, int species,
                                       V3<T> disp, const SubSet& st, C& out) {
  const Chem& ch = *g.chem;
  const uint32_t pmask = ch.partners[species];
  const T movelen2 = dot_rn(disp, disp);
  const T sigma2 = mul_rn(g.R, g.R);
  // segment box grown by R plus a margin that covers rounding in the octant test
  const V3<T> e = pos + disp;
  const T mg = add_rn(mul_rn(g.R, (T)1.01), mul_rn(g.sp_edge, (T)1e-3));
  const V3<T> lo = v3<T>(min(pos.x, e.x) - mg, min(pos.y, e.y) - mg, min(pos.z, e.z) - mg);
  const V3<T> hi = v3<T>(max(pos.x, e.x) + mg, max(pos.y, e.y) + mg, max(pos.z, e.z) + mg);
  for (int i = 0; i < st.n; i++) occupants_of(g, cells, self, pos, disp, pmask, movelen2, sigma2, lo, hi, st.s[i], out);
}

// the same over a mask (set bits in index order; the candidate list keeps the
// earliest collisions by time and id, so the visiting order does not matter)
template <typename T, class C>
__device__ void collide_with_occupants(const Geo<T>& g, const Cells<T>& cells, uint32_t self, V3<T> pos, int species,
                                       V3<T> disp, const SubMask& sm, C& out) {
  const Chem& ch = *g.chem;
  const uint32_t pmask = ch.partners[species];
  const T movelen2 = dot_rn(disp, disp);
  const T sigma2 = mul_rn(g.R, g.R);
  // segment box grown by R plus a margin that covers rounding in the octant test
  const V3<T> e = pos + disp;
  const T mg = add_rn(mul_rn(g.R, (T)1.01), mul_rn(g.sp_edge, (T)1e-3));
  const V3<T> lo = v3<T>(min(pos.x, e.x) - mg, min(pos.y, e.y) - mg, min(pos.z, e.z) - mg);
  const V3<T> hi = v3<T>(max(pos.x, e.x) + mg, max(pos.y, e.y) + mg, max(pos.z, e.z) + mg);
  for (uint64_t mb = sm.bits; mb; mb &= mb - 1) {
    const int bit = __ffsll((long long)mb) - 1;
    const uint32_t sp = sub_of3(g, sm.x0 + (bit & 3), sm.y0 + ((bit >> 2) & 3), sm.z0 + (bit >> 4));
    occupants_of(g, cells, self, pos, disp, pmask, movelen2, sigma2, lo, hi, sp, out);
  }
}

// The 4x4x4 window of the partner set (SubMask) of a segment: its box grown by
// R*sqrt(2) (with a rounding margin), anchored at the low corner. sm.bad when the box
// spans more than 4 subpartitions on an axis; the list takes over then.
template <typename T>
__device__ __forceinline__ void mask_box(const Geo<T>& g, V3<T> pos, V3<T> mdisp, SubMask& sm) {
  const T rn = g.R * (T)1.41421356238 * (T)1.01;
  const V3<T> me = pos + mdisp;
  sm.bits = 0;
  sm.n3 = (uint32_t)g.nsub2 * (uint32_t)g.nsub;
  sm.bad = false;
  sm.x0 = (int)floor((min(pos.x, me.x) - rn - g.origin.x) * g.sp_rcp);
  sm.y0 = (int)floor((min(pos.y, me.y) - rn - g.origin.y) * g.sp_rcp);
  sm.z0 = (int)floor((min(pos.z, me.z) - rn - g.origin.z) * g.sp_rcp);
  if ((int)floor((max(pos.x, me.x) + rn - g.origin.x) * g.sp_rcp) - sm.x0 > 3 ||
      (int)floor((max(pos.y, me.y) + rn - g.origin.y) * g.sp_rcp) - sm.y0 > 3 ||
      (int)floor((max(pos.z, me.z) + rn - g.origin.z) * g.sp_rcp) - sm.z0 > 3)
    sm.bad = true;
}

// the partner set of a segment cut short by a wall hit; out of line: rarely taken
template <typename T>
__device__ __noinline__ SubMask recollect_mask(const Geo<T>& g, V3<T> pos, uint32_t sp, V3<T> mdisp) {
  SubMask sm;
  mask_box(g, pos, mdisp, sm);
  if (!sm.bad) collect_for_molecules(g, pos, sp, mdisp, sm);
  return sm;
}

// The partner set visited without storing it: every subpartition the collection
// generates (crossed ones and their neighbours, with repeats) has its occupants
// scanned at once; the collector drops repeated candidates.
template <typename T>
struct StreamSet {
  const Cells<T>* cells;
  CollsX<T>* out;
  uint32_t self, pmask, n3;
  V3<T> pos, disp, lo, hi;
  T movelen2, sigma2;
  template <typename G>
  __device__ void insert3(const G& g, int x, int y, int z) {
    const uint32_t sp = sub_of3(g, x, y, z);
    if (sp >= n3) return;
    occupants_of(g, *cells, self, pos, disp, pmask, movelen2, sigma2, lo, hi, sp, *out);
  }
};

// partner modes of a segment: how its candidates were collected (a refill repeats it)
enum : int { PM_MASK = 0, PM_LIST = 1, PM_STREAM = 2 };

// candidates of a segment over its partner list (PM_LIST), or, when the list
// overflows its capacity, along the walk (PM_STREAM); out: cursor and dedupe as the
// caller sets them
template <typename T>
__device__ int partners_listed(const Geo<T>& g, const Cells<T>& cells, uint32_t self, V3<T> pos, uint32_t sp,
                               V3<T> mdisp, int species, V3<T> remaining, int mode, CollsX<T>& out, uint32_t& err) {
  if (mode == PM_LIST) {
    SubSet st;
    st.n = 0;
    st.cap = cells.maxset;
    st.n3 = (uint32_t)g.nsub2 * (uint32_t)g.nsub;
    st.overflow = false;
    collect_for_molecules(g, pos, sp, mdisp, st);
    if (!st.overflow) {
      collide_with_occupants(g, cells, self, pos, species, remaining, st, out);
      return PM_LIST;
    }
    err |= ST_SET_OVERFLOW;
  }
  StreamSet<T> ss;
  ss.cells = &cells;
  ss.out = &out;
  ss.self = self;
  ss.pmask = g.chem->partners[species];
  ss.n3 = (uint32_t)g.nsub2 * (uint32_t)g.nsub;
  ss.pos = pos;
  ss.disp = remaining;
  ss.movelen2 = dot_rn(remaining, remaining);
  ss.sigma2 = mul_rn(g.R, g.R);
  const V3<T> e = pos + remaining;
  const T mg = add_rn(mul_rn(g.R, (T)1.01), mul_rn(g.sp_edge, (T)1e-3));
  ss.lo = v3<T>(min(pos.x, e.x) - mg, min(pos.y, e.y) - mg, min(pos.z, e.z) - mg);
  ss.hi = v3<T>(max(pos.x, e.x) + mg, max(pos.y, e.y) + mg, max(pos.z, e.z) + mg);
  out.dedupe = true;
  collect_for_molecules(g, pos, sp, mdisp, ss);
  return PM_STREAM;
}

// the partner scan over a list of subpartitions, for segments whose set does not fit
// the 4x4x4 mask (long moves, fine grids); out of line: rarely taken. Returns the
// partner mode used (PM_LIST or PM_STREAM).
template <typename T>
__device__ __noinline__ int partners_by_list(const Geo<T>& g, const Cells<T> cells, uint32_t self, V3<T> pos,
                                             uint32_t sp, V3<T> mdisp, int species, V3<T> remaining,
                                             Colls<T>& colls) {
  CollsX<T> x{colls, false, false, (T)0, 0};
  uint32_t err = 0;
  const int mode = partners_listed(g, cells, self, pos, sp, mdisp, species, remaining, PM_LIST, x, err);
  return mode | (int)(err << 8);  // the mode, and ST_SET_OVERFLOW shifted into bits 8+
}

template <typename T>
__device__ __noinline__ void save_refill(RefillState<T>* rs, SubMask sm, V3<T> mdisp, uint32_t sp, int mode) {
  rs->sm = sm;
  rs->mdisp = mdisp;
  rs->sp = sp;
  rs->mode = mode;
}

// The next page of candidates after a page that overflowed: those after its last
// one in time order, collected the way the first page was. Out of line: rare.
template <typename T>
__device__ __noinline__ uint32_t refill_colls(const Geo<T>& g, const Cells<T> cells, uint32_t self, V3<T> pos,
                                              int species, V3<T> remaining, const RefillState<T>* rs,
                                              Colls<T>& colls) {
  const VV<T> last = colls.c[colls.n - 1];
  CollsX<T> x{colls, true, false, last.t, cells.uid[last.idx]};
  colls.n = 0;
  colls.overflow = false;
  uint32_t err = 0;
  if (rs->mode == PM_MASK)
    collide_with_occupants(g, cells, self, pos, species, remaining, rs->sm, x);
  else
    partners_listed(g, cells, self, pos, rs->sp, rs->mdisp, species, remaining, rs->mode, x, err);
  return err;
}

// ------------------------------------------------------------------ exact disk

// exd_zetize (exact_disk_utils.inl:54-80)
template <typename T>
__device__ T zetize(T y, T x) {
  if (y >= 0) {
    if (x >= 0) {
      if (x < y) return 1 - (T)0.5 * x / y;
      return (T)0.5 * y / x;
    }
    if (-x < y) return 1 - (T)0.5 * x / y;
    return 2 + (T)0.5 * y / x;
  }
  if (x <= 0) {
    if (y < x) return 3 - (T)0.5 * x / y;
    return 2 + (T)0.5 * y / x;
  }
  if (x < -y) return 3 - (T)0.5 * x / y;
  return 4 + (T)0.5 * y / x;
}

template <typename T>
struct ExV {
  T u, v, r2, zeta;
};

constexpr int MAX_DISK_EDGES = 8;

// visible part of the disk when several wall chords occlude it: integrate
// r(theta)^2 / 2 between consecutive critical angles (chord ends and crossings)
template <typename T>
__device__ __noinline__ T sweep_area(const ExV<T>* pa, const ExV<T>* pb, int n, T R2) {
  T ang[2 * MAX_DISK_EDGES + MAX_DISK_EDGES * (MAX_DISK_EDGES - 1) / 2];
  int na = 0;
  for (int i = 0; i < n; i++) {
    ang[na++] = atan2(pa[i].v, pa[i].u);
    ang[na++] = atan2(pb[i].v, pb[i].u);
  }
  for (int i = 0; i < n; i++) {
    for (int j = i + 1; j < n; j++) {
      T d1u = pb[i].u - pa[i].u, d1v = pb[i].v - pa[i].v;
      T d2u = pb[j].u - pa[j].u, d2v = pb[j].v - pa[j].v;
      T den = d1u * d2v - d1v * d2u;
      if (den == 0) continue;
      T wu = pa[j].u - pa[i].u, wv = pa[j].v - pa[i].v;
      T t = (wu * d2v - wv * d2u) / den;
      T s = (wu * d1v - wv * d1u) / den;
      if (t > 0 && t < 1 && s > 0 && s < 1) ang[na++] = atan2(pa[i].v + t * d1v, pa[i].u + t * d1u);
    }
  }
  for (int i = 1; i < na; i++) {
    T x = ang[i];
    int j = i - 1;
    while (j >= 0 && ang[j] > x) {
      ang[j + 1] = ang[j];
      j--;
    }
    ang[j + 1] = x;
  }
  T area = 0;
  const T R = sqrt(R2);
  for (int k = 0; k < na; k++) {
    T a0 = ang[k];
    T a1 = (k + 1 < na) ? ang[k + 1] : ang[0] + (T)(2 * MY_PI);
    if (a1 - a0 <= 0) continue;
    T am = (T)0.5 * (a0 + a1);
    T cu = cos(am), cv = sin(am);
    int best = -1;
    T best_r = R;
    for (int i = 0; i < n; i++) {
      T du = pb[i].u - pa[i].u, dv = pb[i].v - pa[i].v;
      T den = cu * dv - cv * du;
      if (den == 0) continue;
      T r = (pa[i].u * dv - pa[i].v * du) / den;
      T s = (pa[i].u * cv - pa[i].v * cu) / den;
      if (r > 0 && s >= 0 && s <= 1 && r < best_r) {
        best_r = r;
        best = i;
      }
    }
    if (best < 0) {
      area += (T)0.5 * R2 * (a1 - a0);
    } else {
      T du = pb[best].u - pa[best].u, dv = pb[best].v - pa[best].v;
      T num = pa[best].u * dv - pa[best].v * du;
      T r0 = num / (cos(a0) * dv - sin(a0) * du);
      T r1 = num / (cos(a1) * dv - sin(a1) * du);
      area += (T)0.5 * r0 * r1 * sin(a1 - a0);
    }
  }
  return area;
}

// exact_disk (exact_disk_utils.inl:840-1145, use_expanded_list): fraction of the
// interaction disk around the collision point not occluded by walls, < 0 if a wall
// separates the molecules
// (kept out of line: it runs for a small fraction of collisions and would bloat the
// hot loop's code)
template <typename T>
__device__ __noinline__ T exact_disk(const Geo<T>& g, V3<T> loc, V3<T> mv, int moving_species, V3<T> target) {
  const T R = g.R;
  const T R2 = R * R;
  const T m2_i = 1 / dot(mv, mv);
  V3<T> m, u, v;
  {
    // exd_coordize (:94-145)
    T a = 1 / sqrt(dot(mv, mv));
    m = cmul(v3<T>(a, a, a), mv);
    T mx2 = m.x * m.x, my2 = m.y * m.y, mz2 = m.z * m.z;
    if (mx2 > my2) {
      if (mx2 > mz2) {
        if (my2 > mz2) {
          u = v3<T>(m.y, -m.x, 0); a = 1 - mz2; v = v3<T>(m.z * m.x, m.z * m.y, -a);
        } else {
          u = v3<T>(m.z, 0, -m.x); a = 1 - my2; v = v3<T>(-m.y * m.x, a, -m.y * m.z);
        }
      } else {
        u = v3<T>(-m.z, 0, m.x); a = 1 - my2; v = v3<T>(m.y * m.x, -a, m.y * m.z);
      }
    } else {
      if (my2 > mz2) {
        if (mx2 > mz2) {
          u = v3<T>(-m.y, m.x, 0); a = 1 - mz2; v = v3<T>(-m.z * m.x, -m.z * m.y, a);
        } else {
          u = v3<T>(0, m.z, -m.y); a = 1 - mx2; v = v3<T>(-a, m.x * m.y, m.x * m.z);
        }
      } else {
        u = v3<T>(0, -m.z, m.y); a = 1 - mx2; v = v3<T>(a, -m.x * m.y, -m.x * m.z);
      }
    }
    a = 1 / sqrt(a);
    u = scale(u, a);
    v = scale(v, a);
  }
  V3<T> L = v3<T>(dot(loc, m), dot(loc, u), dot(loc, v));
  ExV<T> sm;
  {
    // distinguishable_vec3 (src4/defines.h:766)
    T c = tabs(loc.x), cc, d;
    d = tabs(loc.y); if (d > c) c = d;
    d = tabs(loc.z); if (d > c) c = d;
    d = tabs(target.x); if (d > c) c = d;
    d = tabs(target.y); if (d > c) c = d;
    d = tabs(target.z); if (d > c) c = d;
    cc = tabs(loc.x - target.x);
    d = tabs(loc.y - target.y); if (d > cc) cc = d;
    d = tabs(loc.z - target.z); if (d > cc) cc = d;
    if (c < Eps<T>::pos) c = Eps<T>::pos;
    if (!(c * Eps<T>::pos < cc)) {
      sm.u = sm.v = sm.r2 = sm.zeta = 0;
    } else {
      V3<T> td = target - loc;
      sm.u = dot(td, u);
      sm.v = dot(td, v);
      sm.r2 = sm.u * sm.u + sm.v * sm.v;
      sm.zeta = zetize(sm.v, sm.u);
    }
  }
  ExV<T> ea[MAX_DISK_EDGES], eb[MAX_DISK_EDGES];
  int n_edges = 0;
  const uint32_t sp = subpart_of(g, loc);
  const Chem& ch = *g.chem;
  // only walls reaching the cells within R of the collision point can occlude the disk
  V3<T> blo, bhi;
  seg_box(loc, v3<T>(0, 0, 0), R * (T)1.01 + g.sp_edge * (T)1e-3, blo, bhi);
  const uint64_t om = cells_touched(g, sp, blo, bhi);
  WallEntries<T> it;
  it.start(g, sp, om);
  uint32_t k;
  while (it.next(g, k)) {
    const uint32_t wi = g.wsp_list[k];
    const P4<T> rj = g.wrej[wi];
    V3<T> wn = v3<T>(rj.x, rj.y, rj.z);
    T l_n = dot(loc, wn);
    T d = rj.w - l_n;
    T m_n = dot(mv, wn);
    if (d * d >= R2 * (1 - m2_i * m_n * m_n)) continue;
    const WallFace<T>& wf = g.wface[wi];
    V3<T> wv[3] = {wf.v0, wf.v1, wf.v2};
    V3<T> llf, urb;
    llf.x = urb.x = wv[0].x;
    llf.y = urb.y = wv[0].y;
    llf.z = urb.z = wv[0].z;
    if (wv[1].x < llf.x) llf.x = wv[1].x; else if (wv[1].x > urb.x) urb.x = wv[1].x;
    if (wv[2].x < llf.x) llf.x = wv[2].x; else if (wv[2].x > urb.x) urb.x = wv[2].x;
    if (wv[1].y < llf.y) llf.y = wv[1].y; else if (wv[1].y > urb.y) urb.y = wv[1].y;
    if (wv[2].y < llf.y) llf.y = wv[2].y; else if (wv[2].y > urb.y) urb.y = wv[2].y;
    if (wv[1].z < llf.z) llf.z = wv[1].z; else if (wv[1].z > urb.z) urb.z = wv[1].z;
    if (wv[2].z < llf.z) llf.z = wv[2].z; else if (wv[2].z > urb.z) urb.z = wv[2].z;
    T a, b;
    b = R2 * (1 - mv.x * mv.x * m2_i);
    a = llf.x - loc.x; if (a > 0 && a * a >= b) continue;
    a = loc.x - urb.x; if (a > 0 && a * a >= b) continue;
    b = R2 * (1 - mv.y * mv.y * m2_i);
    a = llf.y - loc.y; if (a > 0 && a * a >= b) continue;
    a = loc.y - urb.y; if (a > 0 && a * a >= b) continue;
    b = R2 * (1 - mv.z * mv.z * m2_i);
    a = llf.z - loc.z; if (a > 0 && a * a >= b) continue;
    a = loc.z - urb.z; if (a > 0 && a * a >= b) continue;
    if (ch.can_volwall[moving_species] && g.wall_class[(size_t)wi * g.nsp + moving_species] == 1) continue;
    V3<T> p0 = v3<T>(dot(wv[0], m), dot(wv[0], u), dot(wv[0], v)) - L;
    V3<T> p1 = v3<T>(dot(wv[1], m), dot(wv[1], u), dot(wv[1], v)) - L;
    V3<T> p2 = v3<T>(dot(wv[2], m), dot(wv[2], u), dot(wv[2], v)) - L;
    ExV<T> pa, pb;
    auto isect = [](V3<T> P, V3<T> Q, ExV<T>& o) {
      T t = P.x / (P.x - Q.x);
      o.u = P.y + t * (Q.y - P.y);
      o.v = P.z + t * (Q.z - P.z);
    };
    if ((p0.x < 0) == (p1.x < 0)) {
      if ((p2.x < 0) == (p1.x < 0)) continue;
      isect(p0, p2, pa);
      isect(p1, p2, pb);
    } else if ((p0.x < 0) == (p2.x < 0)) {
      isect(p0, p1, pa);
      isect(p2, p1, pb);
    } else {
      isect(p1, p0, pa);
      isect(p2, p0, pb);
    }
    pa.r2 = pa.u * pa.u + pa.v * pa.v;
    pb.r2 = pb.u * pb.u + pb.v * pb.v;
    if (pa.r2 < Eps<T>::pos * R2 || pb.r2 < Eps<T>::pos * R2) return -1;
    if (!distinguishable<T>(pa.u * pb.v, pb.u * pa.v, Eps<T>::pos) && (pa.u * pb.u + pa.v * pb.v) < 0) return -1;
    T ti = 0, si = 1;
    if (pa.r2 > R2 || pb.r2 > R2) {
      T pa_pb = pa.u * pb.u + pa.v * pb.v;
      if (!distinguishable<T>(pa.r2 + pb.r2, 2 * pa_pb, Eps<T>::pos)) {
        if (sm.r2 < pa.r2 && sm.r2 < pb.r2 && distinguishable<T>(sm.r2, pa.r2, Eps<T>::pos) &&
            distinguishable<T>(sm.r2, pa.r2, Eps<T>::pos))
          continue;
        if (!distinguishable<T>(sm.u * pa.v, sm.v * pa.u, Eps<T>::pos_sqrt) ||
            !distinguishable<T>(sm.u * pb.v, sm.v * pb.u, Eps<T>::pos_sqrt))
          return -1;
        continue;
      }
      T ia = 1 / (pa.r2 + pb.r2 - 2 * pa_pb);
      T ib = (pa_pb - pa.r2) * ia;
      T ic = (R2 - pa.r2) * ia;
      T id = ib * ib + ic;
      if (id <= 0) continue;
      id = sqrt(id);
      ti = -ib - id;
      if (ti >= 1) continue;
      if (ti < 0) ti = 0;
      si = -ib + id;
      if (si <= 0) continue;
      if (si > 1) si = 1;
    }
    ExV<T> qa, qb;
    if (ti > 0) {
      qa.u = pa.u + ti * (pb.u - pa.u);
      qa.v = pa.v + ti * (pb.v - pa.v);
      qa.r2 = qa.u * qa.u + qa.v * qa.v;
      qa.zeta = zetize(qa.v, qa.u);
    } else {
      qa = pa;
      qa.zeta = zetize(pa.v, pa.u);
    }
    if (si < 1) {
      qb.u = pa.u + si * (pb.u - pa.u);
      qb.v = pa.v + si * (pb.v - pa.v);
      qb.r2 = qb.u * qb.u + qb.v * qb.v;
      qb.zeta = zetize(qb.v, qb.u);
    } else {
      qb = pb;
      qb.zeta = zetize(pb.v, pb.u);
    }
    a = qb.zeta - qa.zeta;
    if (a < 0) a += 4;
    if (a >= 2) {
      ExV<T> t = qa;
      qa = qb;
      qb = t;
      a = 4 - a;
    }
    b = sm.zeta - qa.zeta;
    if (b < 0) b += 4;
    if (b < a) {
      T au = qa.u - sm.u, av = qa.v - sm.v, bu = qb.u - sm.u, bv = qb.v - sm.v;
      T c = au * bv - av * bu;
      if (c < 0 || !distinguishable<T>(au * bv, av * bu, Eps<T>::pos)) return -1;
    }
    if (n_edges < MAX_DISK_EDGES) {
      ea[n_edges] = qa;
      eb[n_edges] = qb;
      n_edges++;
    }
  }
  if (n_edges == 0) return 1;
  if (n_edges == 1) {
    T ares = ea[0].u * eb[0].u + ea[0].v * eb[0].v;
    T bres = ea[0].u * eb[0].v - ea[0].v * eb[0].u;
    T sres;
    if (ares <= 0)
      sres = atan(-ares / bres) + (T)(0.5 * MY_PI);
    else
      sres = atan(bres / ares);
    return ((T)0.5 * bres + R2 * ((T)MY_PI - (T)0.5 * sres)) / ((T)MY_PI * R2);
  }
  return sweep_area(ea, eb, n_edges, R2) / ((T)MY_PI * R2);
}

// ------------------------------------------------------------------ reaction tests

// binary_search_double (rxn_utils.inl:301-321) with mult = 1 over a class's cumulative
// pathway probabilities: the pathway a probability below the class's maximum selects
// (RxnClass::get_pathway_index_for_probability; MCell3 src/react_cond.c:80-104)
__device__ __forceinline__ int pathway_for(const double* cum, int npw, double match) {
  int lo = 0, hi = npw - 1;
  while (hi - lo > 1) {
    const int mid = (hi + lo) / 2;
    if (match > cum[mid])
      lo = mid;
    else
      hi = mid;
  }
  return match > cum[lo] ? hi : lo;
}

// test_bimolecular (rxn_utils.inl:336-414): the pathway that fires, or -1. Out of
// line (fp64 arithmetic, run for few candidates): a smaller diffuse kernel.
// `u`: the one 32-bit draw it takes (rng_dbl), drawn by the caller so that the
// generator's state is not passed by reference to this out-of-line call
static __device__ __noinline__ int test_bimolecular(const double* cum, int npw, double scaling, uint32_t u) {
  const double max_fixed_p = cum[npw - 1];
  const double r = (double)u * (1.0 / 4294967296.0);
  double prob;
  if (max_fixed_p < scaling) {
    prob = r * scaling;
    if (prob >= max_fixed_p) return -1;
  } else {
    const float max_p = (float)max_fixed_p;
    if (max_p >= scaling) {
      // cannot scale enough: keep the proportions of the pathways
      prob = r * max_p;
    } else {
      prob = r * scaling;
      if (prob >= max_p) return -1;
    }
  }
  return npw == 1 ? 0 : pathway_for(cum, npw, prob);
}

// which_unimolecular (rxn_utils.inl:774-783): the pathway of a unimolecular reaction
// that happens; a draw only when the class has several
template <class D>
__device__ __forceinline__ int which_unimolecular(const double* cum, int npw, D& draws) {
  if (npw <= 1) return 0;
  const double match = draw_dbl(draws) * cum[npw - 1];
  return pathway_for(cum, npw, match);
}

// test_intersect (rxn_utils.inl:593-626) for an absorptive surface class (rate DBL_GIGANTIC)
template <class D>
__device__ __forceinline__ bool test_intersect_absorb(double scaling, D& draws) {
  const double max_prob = GIGANTIC;
  double p;
  if (max_prob > scaling) {
    p = draw_dbl(draws) * max_prob;
  } else {
    p = draw_dbl(draws) * scaling;
    if (p > max_prob) return false;
  }
  if (p > max_prob) return false;
  (void)draw_dbl(draws);
  return true;
}

// time_of_unimol (rxn_utils.inl:721-735)
template <class D>
__device__ __forceinline__ double time_of_unimol(double k_tot, D& draws) {
  double p = draw_dbl(draws);
  if (k_tot <= 0 || !distinguishable<double>(p, 0.0, EPS)) return TIME_FOREVER;
  return -log(p) / k_tot;
}

// ------------------------------------------------------------------ one molecule, one step

// diffuse_vol_molecule from the known displacement on (diffuse_react_event.cpp:450-618):
// ray trace, sort, collisions in time order, wall interactions; loops while walls are hit.
template <typename T, class D, class E>
__device__ TraceOut<T> trace_molecule(const Geo<T>& g, const Cells<T>& cells, uint32_t self, V3<T> pos, int species,
                                      V3<T> disp, T r_rate_factor, T t_steps, T start_time, D& draws, E& ev,
                                      bool allow_vv = true) {
  TraceOut<T> res;
  res.status = 0;
  res.err = 0;
  res.cv_mask = 0;
  res.cv_val = 0;
  res.partner = NONE;
  res.t_abs = 0;
  res.pathway = 0;
  res.rxn_pos = pos;
  const Chem& ch = *g.chem;
  const bool can_vol_react = allow_vv && ch.partners[species] != 0;
  uint32_t sp = subpart_of(g, pos);
  uint32_t last_hit = NONE;
  T elapsed = start_time;
  V3<T> remaining = disp;
  int bounces = 0;
  bool was_defunct = false;
  bool hit_wall;
  RefillState<T> rs;  // written only when a candidate page overflows
  do {
    // ---- ray_trace_vol (diffuse_react_event.cpp:627-780)
    hit_wall = false;
    V3<T> pdisp = remaining;
    if (!in_partition(g, pos + remaining)) pdisp = disp_up_to_partition_boundary(g, pos, remaining);
    WallHit<T> hit, tentative;
    tentative.t = (T)1e20;
    tentative.type = CT_MISS;
    bool hit_in_last = false, used_tentative = false;
    const V3<T> up_to_init = remaining;  // displacement_up_to_wall_collision before the search
    // The partner set of the whole segment (collect_for_molecules over pdisp) is
    // collected along the wall walk: the same walk, the same crossing points. It is
    // kept unless a wall is hit before the last subpartition (then re-collected below).
    SubMask sm;
    sm.bad = true;
    // collide_mol divides by the squared length of the move: a move of zero length
    // (what a wall met exactly at the end of the move, t = 1, leaves for the next
    // segment), or one whose square underflows in fp32, meets no molecule. The
    // reference asserts a non-zero length there; its release build would take every
    // occupant scanned as a collision at t = 0/0.
    const bool scan = can_vol_react && dot_rn(remaining, remaining) > (T)0;
    {
      Walk<T> w;
      w.start(g, pos, sp, pdisp);
      if (scan) {
        mask_box(g, pos, pdisp, sm);
        if (!sm.bad) collect_start(g, pos, w.cx, w.cy, w.cz, sm);
      }
      uint32_t cur = sp;
      for (;;) {
        if (closest_wall_collision(g, pos, cur, last_hit, draws, remaining, hit, tentative, res.err)) {
          hit_wall = true;
          hit_in_last = (cur == w.dest);
          break;
        }
        if (res.err & ST_ERRORS) break;
        if (!w.next(g)) break;
        cur = w.cur;
        if (!sm.bad) collect_crossing(g, w, sm);
      }
      if (!hit_wall && sizeof(T) == 4 && tentative.type != CT_MISS) {
        hit = tentative;
        hit_wall = true;
        used_tentative = true;
      }
    }
    if (res.err & ST_ERRORS) {
      res.status = 3;
      break;
    }
    Colls<T> colls;
    colls.n = 0;
    colls.overflow = false;
    if (scan) {
      // ray_trace_vol keeps the set of the first collection unless a wall was hit
      // before the last crossed subpartition, then re-collects up to the hit
      V3<T> mdisp = pdisp;
      // the set lies within the segment's box grown by R*sqrt(2): a 4x4x4 mask when
      // that box spans at most 4 subpartitions per axis, else (or if an insertion
      // falls outside) the list
      if (hit_wall && !hit_in_last) {
        mdisp = used_tentative ? up_to_init : hit.pos - pos;
        sm = recollect_mask(g, pos, sp, mdisp);
      } else if (!sm.bad) {
        collect_end(g, pos, pdisp, sm);
      }
      int pmode = PM_MASK;
      if (!sm.bad) {
        collide_with_occupants(g, cells, self, pos, species, remaining, sm, colls);
      } else {
        const int pm = partners_by_list(g, cells, self, pos, sp, mdisp, species, remaining, colls);
        pmode = pm & 0xFF;
        res.err |= (uint32_t)pm >> 8;
      }
      // a full page: how to collect the next one (rare)
      if (colls.overflow) save_refill(&rs, sm, mdisp, sp, pmode);
    }
    const V3<T> pos_at_start = pos;  // collision points are measured from here
    if (!hit_wall) {
      const V3<T> seg_start = pos;
      pos = pos + remaining;
      sp = subpart_of(g, pos);
      if (sizeof(T) == 4) {
        // fp32: a segment that crossed no wall may still end on a wall plane after
        // rounding; a later step starting exactly on the plane would then pass the wall
        // (collide_wall treats "starts on the plane" as a miss). Keep it on the side it
        // came from.
        guard_sides(g, sp, pos, seg_start, NONE);
        sp = subpart_of(g, pos);
      }
    }
    // ---- collisions in time order (diffuse_react_event.cpp:450-572)
    bool wall_done = false;
    for (int i = 0; i <= colls.n; i++) {
      if (i == colls.n && colls.overflow) {
        // the page held only the earliest candidates: the next ones, in time order
        res.err |= ST_COLL_OVERFLOW;
        res.err |= refill_colls(g, cells, self, pos_at_start, species, remaining, &rs, colls);
        i = -1;
        continue;
      }
      bool take_wall;
      if (i == colls.n) {
        take_wall = hit_wall;
      } else {
        // the wall sorts before a later molecule; equal times keep the molecule first
        take_wall = hit_wall && hit.t < colls.c[i].t;
      }
      if (take_wall) {
        const int side = hit.type == CT_FRONT ? 1 : 2;
        const int kind = ch.can_volwall[species] ? g.wall_class[(size_t)hit.wall * g.nsp + species] : 0;
        const T t_abs = elapsed + t_steps * hit.t;
        if (kind == 1) {
          if (g.n_cv) {
            const uint32_t f = cv_bits_of_wall(g, hit.wall);
            res.cv_mask |= f;
            res.cv_val = hit.type == CT_FRONT ? (res.cv_val | f) : (res.cv_val & ~f);
          }
          pos = hit.pos;
          sp = subpart_of(g, pos);
          const T t_smash = hit.t;
          const T f = (T)1 - t_smash;
          remaining = cmul(remaining, v3<T>(f, f, f));
          elapsed += t_steps * t_smash;
          t_steps *= f;
          if (t_steps < (T)EPS) t_steps = (T)EPS;
          last_hit = hit.wall;
          // fp32: make sure the crossing point lies on the far side, else the neighbouring
          // triangle of the crossed edge is hit again at t ~ 0 and re-tried without end
          if (sizeof(T) == 4) {
            keep_side(g.wrej[hit.wall], hit.type == CT_FRONT ? -1.0 : 1.0, pos);
            pos = guard_sides_rare(g, sp, pos, pos_at_start, hit.wall);  // every other plane: the side it came from
            sp = subpart_of(g, pos);
          }
          ev.put(2, hit.wall, side, (double)hit.t, (double)t_abs, (double)hit.pos.x, (double)hit.pos.y,
                 (double)hit.pos.z);
        } else if (kind == 2 && test_intersect_absorb((double)r_rate_factor, draws)) {
          ev.put(3, hit.wall, side, (double)hit.t, (double)t_abs, (double)hit.pos.x, (double)hit.pos.y,
                 (double)hit.pos.z);
          was_defunct = true;
          res.status = 2;
          res.t_abs = t_abs;
          res.rxn_pos = hit.pos;
        } else {
          // reflect_from_wall (collision_utils.inl:1711-1747)
          elapsed += t_steps * hit.t;
          const P4<T> rj = g.wrej[hit.wall];
          V3<T> n = v3<T>(rj.x, rj.y, rj.z);
          T t_reflect = hit.t;
          pos = hit.pos;
          sp = subpart_of(g, pos);
          t_steps *= (T)1 - t_reflect;
          last_hit = hit.wall;
          T rf = (T)-2.0 * dot(remaining, n);
          if (sizeof(T) == 4 && (T)1 - t_reflect < Eps<T>::pos_sqrt) t_reflect -= Eps<T>::pos_sqrt;
          const T f = (T)1 - t_reflect;
          remaining = cmul(remaining + cmul(v3<T>(rf, rf, rf), n), v3<T>(f, f, f));
          // fp32: the rounded reflection point must stay on the side the molecule came
          // from, else a coplanar neighbour triangle can reflect it outwards
          // (and on the side it came from of every other plane it lies on: a hit on the
          // edge of two faces rounds onto both planes)
          if (sizeof(T) == 4) {
            keep_side(rj, hit.type == CT_FRONT ? 1.0 : -1.0, pos);
            pos = guard_sides_rare(g, sp, pos, pos_at_start, hit.wall);
            sp = subpart_of(g, pos);
          }
          ev.put(1, hit.wall, side, (double)hit.t, (double)t_abs, (double)hit.pos.x, (double)hit.pos.y,
                 (double)hit.pos.z);
        }
        wall_done = true;
        break;
      }
      if (i == colls.n) break;
      const VV<T> c = colls.c[i];
      if (c.t < Eps<T>::stime) continue;  // is_immediate_collision
      const T t_abs = elapsed + t_steps * c.t;
      const P4<T> q = cells.pos[c.idx];
      const uint64_t cuid = cells.uid[c.idx];
      const V3<T> cpos = pos_at_start + scale(remaining, c.t);  // collide_mol's rel_collision_pos
      // exact_disk returns exactly 1 when the collision point's subpartition lists no
      // wall (its wall loop finds no edge); the call is skipped then
      const uint32_t csp = subpart_of(g, cpos);
      const T factor = g.wsp_off[csp] == g.wsp_off[csp + 1]
                           ? (T)1
                           : exact_disk(g, cpos, remaining, species, v3<T>(q.x, q.y, q.z));
      if (factor < 0) {
        ev.put(6, cuid, 0, (double)c.t, (double)t_abs, (double)cpos.x, (double)cpos.y, (double)cpos.z);
        continue;
      }
      const double scaling = (double)factor * (double)r_rate_factor;
      const uint32_t ps = meta_of(q) & META_SPECIES_MASK;
      const int pw = test_bimolecular(ch.bimol_cum[species][ps], ch.bimol_npw[species][ps], scaling, draws.u32());
      if (pw < 0) {
        ev.put(4, cuid, 0, (double)c.t, (double)t_abs, (double)cpos.x, (double)cpos.y, (double)cpos.z);
        continue;
      }
      ev.put(5, cuid, pw, (double)c.t, (double)t_abs, (double)cpos.x, (double)cpos.y, (double)cpos.z);
      was_defunct = true;
      res.status = 1;
      res.pathway = pw;
      res.partner = c.idx;
      res.t_abs = t_abs;
      res.rxn_pos = cpos;
      break;
    }
    if (draws.overrun() || ++bounces > MAX_BOUNCES) {
      res.err |= ST_WATCHDOG;
      res.status = 3;
      break;
    }
  } while (hit_wall && !was_defunct);
  res.pos = pos;
  res.subpart = sp;
  res.elapsed = elapsed;
  res.t_steps = t_steps;
  return res;
}

}  // namespace mcg
