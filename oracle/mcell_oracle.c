/*
 * mcell_oracle.c: CPU restatement (plain C, fp64) of MCell4's volume-molecule
 * diffuse-react step. TEST INFRASTRUCTURE ONLY (checker and timed CPU baseline);
 * the product never links or calls this file.
 *
 * Reference files restated (paths within mcellteam/mcell):
 *   src4/simulation_config.cpp:45-70     subpartition edge and reciprocal
 *   src4/partition.h:248-298             partition / subpartition indexing
 *   src4/wall.cpp:281-342                wall constants
 *   src4/geometry_utils.inl:66-200       wall bounding box, wall -> subpartition binning
 *   src4/wall_utils.inl:326-516          wall_in_box
 *   src4/collision_utils_subparts.inl    collect_neighboring_subparts, collect_crossed_subparts
 *   src4/collision_utils.inl:48-114      get_displacement_up_to_partition_boundary
 *   src4/collision_utils.inl:464-552     collide_mol, collide_mol_loop_body
 *   src4/collision_utils.inl:568-914     jump_away_line, collide_wall, get_closest_wall_collision
 *   src4/collision_utils.inl:1711-1747   reflect_from_wall
 *   src4/diffuse_react_event.cpp:341-364 sort_collisions_by_time
 *   src4/diffuse_react_event.cpp:367-780 diffuse_vol_molecule, ray_trace_vol
 *   src4/diffuse_react_event.cpp:786-829 collide_and_react_with_vol_mol
 *   src4/diffuse_react_event.cpp:991-1067, :3007-3099  wall reactions, transparent crossing
 *   src4/exact_disk_utils.inl:54-1145    exact_disk (0 and 1 occluding edge restated; the
 *                                        area with 2+ edges is computed by an angular sweep)
 *   src4/rxn_utils.inl:336-414, :593-626, :721-735  test_bimolecular, test_intersect, time_of_unimol
 *   src4/diffusion_utils.inl:113-119, :366-432      displacement
 *   src4/diffuse_react_event.cpp:67-337, :1731-1826, :2446-2933, :2939  scheduling and outcomes
 * All arithmetic keeps the reference's operation order (no FMA contraction:
 * build with -ffp-contract=off) so fp64 results are bit-identical.
 */
#include "mcell_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* libbng / MCell3 constants (src/mcell_structs.h:238-240, src/mcell_structs_shared.h:18) */
#define EPS 1e-12
#define SQRT_EPS 1e-6
#define POS_EPS EPS
#define POS_SQRT_EPS SQRT_EPS
#define STIME_EPS EPS
#define GIGANTIC 1e140
#define MY_PI 3.14159265358979323846
#define POS_SQRT2 1.41421356238
#define TIME_INVALID (-256.0)
#define TIME_FOREVER 1e20
#define IDX_INVALID 0xFFFFFFFFu

typedef struct { double x, y, z; } v3;

static inline v3 V(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, v3 b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vdiv(v3 a, v3 b) { return V(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline v3 vscale(v3 a, double s) { return V(a.x * s, a.y * s, a.z * s); }
/* glm::dot for vec3: tmp = a*b; tmp.x + tmp.y + tmp.z */
static inline double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* glm::cross */
static inline v3 vcross(v3 a, v3 b) {
  return V(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double max3abs(v3 a) { return dmax(dmax(fabs(a.x), fabs(a.y)), fabs(a.z)); }
/* abs_max_2vec (src4/defines.h:644) */
static inline double abs_max_2vec(v3 a, v3 b) {
  return dmax(dmax(dmax(fabs(a.x), fabs(b.x)), dmax(fabs(a.y), fabs(b.y))), dmax(fabs(a.z), fabs(b.z)));
}
/* guard_zero_div (src4/defines.h:811) */
static inline v3 guard_zero(v3 a) {
  if (a.x == 0) a.x = FLT_MIN;
  if (a.y == 0) a.y = FLT_MIN;
  if (a.z == 0) a.z = FLT_MIN;
  return a;
}
/* distinguishable (src/util.c:449) */
static inline int distinguishable(double a, double b, double eps) {
  double c = fabs(a - b);
  a = fabs(a);
  if (a < 1) a = 1;
  b = fabs(b);
  if (b < a) eps *= a; else eps *= b;
  return c > eps;
}
/* distinguishable_vec3 (src4/defines.h:766) */
static int distinguishable_vec3(v3 a, v3 b, double eps) {
  double c = fabs(a.x), cc, d;
  d = fabs(a.y); if (d > c) c = d;
  d = fabs(a.z); if (d > c) c = d;
  d = fabs(b.x); if (d > c) c = d;
  d = fabs(b.y); if (d > c) c = d;
  d = fabs(b.z); if (d > c) c = d;
  cc = fabs(a.x - b.x);
  d = fabs(a.y - b.y); if (d > cc) cc = d;
  d = fabs(a.z - b.z); if (d > cc) cc = d;
  if (c < eps) c = eps;
  return c * eps < cc;
}

/* ------------------------------------------------------------------ scene */

typedef struct {
  v3 normal;
  double d;
  v3 unit_u, unit_v;
  double uv1u, uv2u, uv2v;
  unsigned vi[3];
} owall;

typedef struct {
  unsigned* ids;
  unsigned n, cap;
} idvec;

static void idvec_push(idvec* v, unsigned id) {
  if (v->n == v->cap) {
    v->cap = v->cap ? v->cap * 2 : 8;
    v->ids = (unsigned*)realloc(v->ids, sizeof(unsigned) * v->cap);
  }
  v->ids[v->n++] = id;
}
static void idvec_remove(idvec* v, unsigned id) {
  for (unsigned i = 0; i < v->n; i++) {
    if (v->ids[i] == id) {
      v->ids[i] = v->ids[--v->n];
      return;
    }
  }
}

typedef struct {
  v3 pos;
  unsigned species;
  unsigned subpart;
  int defunct;
  double diffusion_time;
  double unimol_time;
  int schedule_unimol;
} omol;

typedef struct {
  v3 origin, opposite;
  double part_edge, sp_edge, sp_rcp, R;
  unsigned nsub, nsub2, nsub3;
  unsigned nv, nw, nspecies;
  v3* verts;
  owall* walls;
  unsigned* wsp_off; /* CSR of walls per subpartition, ascending wall index */
  unsigned* wsp_list;
  double* space_step;
  unsigned char* wall_class; /* [nw * nspecies] */
  int* can_volwall;          /* species has a non-reflective wall class */
  double* bimol_p;           /* [nspecies * nspecies] max_fixed_p, < 0 = no reaction */
  /* reaction class per reactant pair (BNG::RxnClass): its pathways' cumulative
     probabilities and the reaction index of each pathway, in the order added */
  double* bimol_cum;         /* [nspecies * nspecies * ORC_MAX_PATHWAYS] */
  int* bimol_npw;            /* [nspecies * nspecies] */
  int* bimol_rxn;            /* [nspecies * nspecies * ORC_MAX_PATHWAYS] reaction index */
  int* can_vol_react;
  /* molecules and per-subpartition occupant lists (set semantics) */
  omol* mols;
  unsigned nmol, capmol;
  idvec* occ; /* [nsub3] ids of live molecules in the subpartition */
} oscene;

/* SimulationConfig::init_subpartition_edge_length (simulation_config.cpp:45, fp64 branch) */
static void scene_init_grid(oscene* s, const double* origin, double partition_edge, unsigned nsub) {
  s->nsub = nsub;
  s->sp_edge = partition_edge / (double)nsub;
  s->sp_rcp = 1.0 / s->sp_edge;
  s->part_edge = s->sp_edge * nsub;
  s->nsub2 = nsub * nsub;
  s->nsub3 = nsub * nsub * nsub;
  s->origin = V(origin[0], origin[1], origin[2]);
  /* Partition ctor (partition.cpp:56): opposite = origin + edge */
  s->opposite = vadd(s->origin, V(s->part_edge, s->part_edge, s->part_edge));
}

/* Partition::in_this_partition / get_subpart_* (partition.h:248-298) */
static inline int in_partition(const oscene* s, v3 p) {
  return p.x >= s->origin.x && p.y >= s->origin.y && p.z >= s->origin.z &&
         p.x < s->opposite.x && p.y < s->opposite.y && p.z < s->opposite.z;
}
static inline void subpart_3d(const oscene* s, v3 p, int* ix, int* iy, int* iz) {
  v3 rel = vsub(p, s->origin);
  *ix = (int)(rel.x * s->sp_rcp);
  *iy = (int)(rel.y * s->sp_rcp);
  *iz = (int)(rel.z * s->sp_rcp);
}
static inline unsigned subpart_of_3d(const oscene* s, int x, int y, int z) {
  return (unsigned)(x + y * (int)s->nsub + z * (int)s->nsub2);
}
static inline unsigned subpart_index(const oscene* s, v3 p) {
  int x, y, z;
  subpart_3d(s, p, &x, &y, &z);
  return subpart_of_3d(s, x, y, z);
}
static inline void subpart_3d_from_index(const oscene* s, unsigned i, int* x, int* y, int* z) {
  *x = (int)(i % s->nsub);
  *y = (int)((i / s->nsub) % s->nsub);
  *z = (int)((i / s->nsub2) % s->nsub);
}

/* Wall::initialize_wall_constants (wall.cpp:281-342) */
static void wall_constants(const oscene* s, owall* w) {
  v3 v0 = s->verts[w->vi[0]], v1 = s->verts[w->vi[1]], v2 = s->verts[w->vi[2]];
  v3 vA = vsub(v1, v0), vB = vsub(v2, v0), vX = vcross(vA, vB);
  double area = 0.5 * sqrt(vX.x * vX.x + vX.y * vX.y + vX.z * vX.z);
  if (!distinguishable(area, 0, EPS)) {
    memset(&w->normal, 0, sizeof(v3));
    memset(&w->unit_u, 0, sizeof(v3));
    memset(&w->unit_v, 0, sizeof(v3));
    w->uv1u = w->uv2u = w->uv2v = w->d = 0;
    return;
  }
  v3 f1 = vsub(v1, v0);
  double f1_len_squared = f1.x * f1.x + f1.y * f1.y + f1.z * f1.z;
  double inv_f1_len = 1 / sqrt(f1_len_squared);
  w->unit_u = vmul(f1, V(inv_f1_len, inv_f1_len, inv_f1_len));
  v3 f2 = vsub(v2, v0);
  v3 n = vcross(w->unit_u, f2);
  double nl2 = n.x * n.x + n.y * n.y + n.z * n.z;
  double inv_nl = 1 / sqrt(nl2);
  w->normal = vmul(n, V(inv_nl, inv_nl, inv_nl));
  w->unit_v = vcross(w->normal, w->unit_u);
  w->d = vdot(v0, w->normal);
  w->uv1u = vdot(f1, w->unit_u);
  w->uv2u = vdot(f2, w->unit_u);
  w->uv2v = vdot(f2, w->unit_v);
}

/* get_wall_bounding_box (geometry_utils.inl:66-100) */
static void wall_bbox(const v3* wv, v3* llf, v3* urb) {
  llf->x = urb->x = wv[0].x;
  llf->y = urb->y = wv[0].y;
  llf->z = urb->z = wv[0].z;
  if (wv[1].x < llf->x) llf->x = wv[1].x; else if (wv[1].x > urb->x) urb->x = wv[1].x;
  if (wv[2].x < llf->x) llf->x = wv[2].x; else if (wv[2].x > urb->x) urb->x = wv[2].x;
  if (wv[1].y < llf->y) llf->y = wv[1].y; else if (wv[1].y > urb->y) urb->y = wv[1].y;
  if (wv[2].y < llf->y) llf->y = wv[2].y; else if (wv[2].y > urb->y) urb->y = wv[2].y;
  if (wv[1].z < llf->z) llf->z = wv[1].z; else if (wv[1].z > urb->z) urb->z = wv[1].z;
  if (wv[2].z < llf->z) llf->z = wv[2].z; else if (wv[2].z > urb->z) urb->z = wv[2].z;
}

static inline int point_in_box(v3 p, v3 llf, v3 urb) {
  return p.x >= llf.x && p.x <= urb.x && p.y >= llf.y && p.y <= urb.y && p.z >= llf.z && p.z <= urb.z;
}

/* one face test of wall_in_box: edge v1->v2 crossing the plane (axis a) = c, then the
   other two coordinates (b, d) inside the face rectangle */
static int edge_hits_face(double v1a, double v2a, double c, double v1b, double v2b, double v1d, double v2d,
                          double lob, double hib, double lod, double hid) {
  if ((v1a <= c && c < v2a) || (v1a > c && c >= v2a)) {
    double r = (c - v1a) / (v2a - v1a);
    double a3 = v1b + r * (v2b - v1b);
    double a4 = v1d + r * (v2d - v1d);
    if (lob <= a3 && a3 <= hib && lod <= a4 && a4 <= hid) return 1;
  }
  return 0;
}

/* wall_in_box (wall_utils.inl:326-516) */
static int wall_in_box(const oscene* s, const owall* w, v3 llf, v3 urb) {
  const v3* vert[3] = {&s->verts[w->vi[0]], &s->verts[w->vi[1]], &s->verts[w->vi[2]]};
  for (int i = 0; i < 3; i++) {
    if (point_in_box(*vert[i], llf, urb)) return 1;
  }
  for (int i = 0; i < 3; i++) {
    const v3* v2 = vert[i];
    const v3* v1 = (i == 0) ? vert[2] : vert[i - 1];
    /* x faces: (y, z) in the face */
    if (edge_hits_face(v1->x, v2->x, llf.x, v1->y, v2->y, v1->z, v2->z, llf.y, urb.y, llf.z, urb.z)) return 2;
    if (edge_hits_face(v1->x, v2->x, urb.x, v1->y, v2->y, v1->z, v2->z, llf.y, urb.y, llf.z, urb.z)) return 3;
    /* y faces: (x, z) */
    if (edge_hits_face(v1->y, v2->y, llf.y, v1->x, v2->x, v1->z, v2->z, llf.x, urb.x, llf.z, urb.z)) return 4;
    if (edge_hits_face(v1->y, v2->y, urb.y, v1->x, v2->x, v1->z, v2->z, llf.x, urb.x, llf.z, urb.z)) return 5;
    /* z faces: (y, x) */
    if (edge_hits_face(v1->z, v2->z, llf.z, v1->y, v2->y, v1->x, v2->x, llf.y, urb.y, llf.x, urb.x)) return 6;
    if (edge_hits_face(v1->z, v2->z, urb.z, v1->y, v2->y, v1->x, v2->x, llf.y, urb.y, llf.x, urb.x)) return 7;
  }
  /* box edges against the triangle: the 12 cube edges are visited as a path over
     the 8 corners (first 7 edges) and then the 5 remaining edges; corner k has
     bits (x,y,z) given by the tables below */
  static const int wx1[12] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 1};
  static const int wy1[12] = {0, 0, 1, 1, 1, 1, 0, 0, 0, 0, 1, 0};
  static const int wz1[12] = {0, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1, 0};
  static const int wx2[12] = {0, 0, 0, 1, 1, 1, 1, 0, 0, 1, 1, 0};
  static const int wy2[12] = {0, 1, 1, 1, 1, 0, 0, 0, 1, 0, 1, 1};
  static const int wz2[12] = {1, 1, 0, 0, 1, 1, 0, 0, 0, 1, 1, 0};
  static const int e1[12] = {0, 1, 3, 2, 6, 7, 5, 4, 0, 1, 3, 4};
  static const int e2[12] = {1, 3, 2, 6, 7, 5, 4, 0, 2, 5, 7, 2};
  v3 n = w->normal;
  double d = w->d;
  double vu[3], vv[3];
  v3 u = vsub(*vert[1], *vert[0]);
  double lus = u.x * u.x + u.y * u.y + u.z * u.z;
  double r_u = 1 / sqrt(lus);
  u = vmul(u, V(r_u, r_u, r_u));
  v3 v = vcross(n, u);
  for (int j = 0; j < 3; j++) {
    vu[j] = vdot(*vert[j], u);
    vv[j] = vdot(*vert[j], v);
  }
  v3 bb = llf, ba = llf;
  double d_box[8];
  d_box[0] = vdot(bb, n);
  for (int i = 0; i < 12; i++) {
    double a1, a2;
    if (i < 7) {
      ba = bb;
      bb.x = wx2[i] ? urb.x : llf.x;
      bb.y = wy2[i] ? urb.y : llf.y;
      bb.z = wz2[i] ? urb.z : llf.z;
      a2 = d_box[e2[i]] = vdot(bb, n);
      a1 = d_box[e1[i]];
      if ((a1 - d < 0 && a2 - d < 0) || (a1 - d > 0 && a2 - d > 0)) continue;
    }
    else {
      a1 = d_box[e1[i]];
      a2 = d_box[e2[i]];
      if ((a1 - d < 0 && a2 - d < 0) || (a1 - d > 0 && a2 - d > 0)) continue;
      ba.x = wx1[i] ? urb.x : llf.x;
      ba.y = wy1[i] ? urb.y : llf.y;
      ba.z = wz1[i] ? urb.z : llf.z;
      bb.x = wx2[i] ? urb.x : llf.x;
      bb.y = wy2[i] ? urb.y : llf.y;
      bb.z = wz2[i] ? urb.z : llf.z;
    }
    double r = (d - a1) / (a2 - a1);
    v3 c = vadd(ba, vmul(V(r, r, r), vsub(bb, ba)));
    double cu = vdot(c, u), cv = vdot(c, v);
    int crossings = 0;
    for (int j = 0; j < 3; j++) {
      int k = (j == 0) ? 2 : j - 1;
      if ((vu[k] < cu && cu <= vu[j]) || (vu[k] >= cu && cu > vu[j])) {
        r = (cu - vu[k]) / (vu[j] - vu[k]);
        if ((vv[k] + r * (vv[j] - vv[k])) > cv) crossings++;
      }
    }
    if (crossings & 1) return 8 + i;
  }
  return 0;
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* wall_subparts_collision_test (geometry_utils.inl:110-200) + Partition::finalize_walls (partition.cpp:91) */
static void bin_walls(oscene* s) {
  unsigned* counts = (unsigned*)calloc(s->nsub3 + 1, sizeof(unsigned));
  unsigned cap = 1024, n = 0;
  unsigned* pairs = (unsigned*)malloc(sizeof(unsigned) * 2 * cap);
  for (unsigned wi = 0; wi < s->nw; wi++) {
    const owall* w = &s->walls[wi];
    v3 wv[3] = {s->verts[w->vi[0]], s->verts[w->vi[1]], s->verts[w->vi[2]]};
    v3 llf, urb;
    wall_bbox(wv, &llf, &urb);
    double leeway = 1;
    if (llf.x < -leeway) leeway = -llf.x;
    if (llf.y < -leeway) leeway = -llf.y;
    if (llf.z < -leeway) leeway = -llf.z;
    if (urb.x > leeway) leeway = urb.x;
    if (urb.y > leeway) leeway = urb.y;
    if (urb.z > leeway) leeway = urb.z;
    leeway = POS_EPS + leeway * POS_EPS;
    leeway += s->R; /* use_expanded_list */
    v3 l3 = V(leeway, leeway, leeway);
    llf = vsub(llf, l3);
    urb = vadd(urb, l3);
    int x0, y0, z0, x1, y1, z1;
    subpart_3d(s, llf, &x0, &y0, &z0);
    subpart_3d(s, urb, &x1, &y1, &z1);
    int hi = (int)s->nsub - 1;
    x0 = clampi(x0, 0, hi); y0 = clampi(y0, 0, hi); z0 = clampi(z0, 0, hi);
    x1 = clampi(x1, 0, hi); y1 = clampi(y1, 0, hi); z1 = clampi(z1, 0, hi);
    for (int x = x0; x <= x1; x++) {
      for (int y = y0; y <= y1; y++) {
        for (int z = z0; z <= z1; z++) {
          unsigned sp = subpart_of_3d(s, x, y, z);
          v3 sl = vadd(s->origin, vmul(V(x, y, z), V(s->sp_edge, s->sp_edge, s->sp_edge)));
          v3 su = vadd(sl, V(s->sp_edge, s->sp_edge, s->sp_edge));
          sl = vsub(sl, l3);
          su = vadd(su, l3);
          if (wall_in_box(s, w, sl, su) != 0) {
            if (n == cap) {
              cap *= 2;
              pairs = (unsigned*)realloc(pairs, sizeof(unsigned) * 2 * cap);
            }
            pairs[2 * n] = sp;
            pairs[2 * n + 1] = wi;
            n++;
            counts[sp]++;
          }
        }
      }
    }
  }
  s->wsp_off = (unsigned*)calloc(s->nsub3 + 1, sizeof(unsigned));
  for (unsigned i = 0; i < s->nsub3; i++) s->wsp_off[i + 1] = s->wsp_off[i] + counts[i];
  s->wsp_list = (unsigned*)malloc(sizeof(unsigned) * (n ? n : 1));
  memset(counts, 0, sizeof(unsigned) * s->nsub3);
  /* walls were visited in ascending index, so each list is ascending */
  for (unsigned k = 0; k < n; k++) {
    unsigned sp = pairs[2 * k];
    s->wsp_list[s->wsp_off[sp] + counts[sp]++] = pairs[2 * k + 1];
  }
  free(pairs);
  free(counts);
}

static void occ_add(oscene* s, unsigned id) { idvec_push(&s->occ[s->mols[id].subpart], id); }
static void occ_remove(oscene* s, unsigned id) { idvec_remove(&s->occ[s->mols[id].subpart], id); }

static unsigned scene_add_mol(oscene* s, v3 pos, unsigned species) {
  if (s->nmol == s->capmol) {
    s->capmol = s->capmol ? s->capmol * 2 : 1024;
    s->mols = (omol*)realloc(s->mols, sizeof(omol) * s->capmol);
  }
  unsigned id = s->nmol++;
  omol* m = &s->mols[id];
  memset(m, 0, sizeof(*m));
  m->pos = pos;
  m->species = species;
  m->subpart = subpart_index(s, pos);
  m->unimol_time = TIME_INVALID;
  occ_add(s, id);
  return id;
}

static oscene* scene_build(const double* origin, double partition_edge, unsigned nsub, double rxn_radius,
                           unsigned nv, const double* verts, unsigned nw, const unsigned* tris,
                           unsigned nspecies, const double* space_steps, const unsigned char* wall_class) {
  oscene* s = (oscene*)calloc(1, sizeof(oscene));
  scene_init_grid(s, origin, partition_edge, nsub);
  s->R = rxn_radius;
  s->nv = nv;
  s->nw = nw;
  s->nspecies = nspecies;
  s->verts = (v3*)malloc(sizeof(v3) * (nv ? nv : 1));
  for (unsigned i = 0; i < nv; i++) s->verts[i] = V(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  s->walls = (owall*)calloc(nw ? nw : 1, sizeof(owall));
  for (unsigned i = 0; i < nw; i++) {
    for (int k = 0; k < 3; k++) s->walls[i].vi[k] = tris[3 * i + k];
    wall_constants(s, &s->walls[i]);
  }
  bin_walls(s);
  s->space_step = (double*)malloc(sizeof(double) * nspecies);
  memcpy(s->space_step, space_steps, sizeof(double) * nspecies);
  s->wall_class = (unsigned char*)calloc((size_t)(nw ? nw : 1) * nspecies, 1);
  if (wall_class) memcpy(s->wall_class, wall_class, (size_t)nw * nspecies);
  s->can_volwall = (int*)calloc(nspecies, sizeof(int));
  for (unsigned w = 0; w < nw; w++)
    for (unsigned i = 0; i < nspecies; i++)
      if (s->wall_class[(size_t)w * nspecies + i]) s->can_volwall[i] = 1;
  s->bimol_p = (double*)malloc(sizeof(double) * nspecies * nspecies);
  s->bimol_cum = (double*)calloc((size_t)nspecies * nspecies * ORC_MAX_PATHWAYS, sizeof(double));
  s->bimol_npw = (int*)calloc((size_t)nspecies * nspecies, sizeof(int));
  s->bimol_rxn = (int*)malloc(sizeof(int) * nspecies * nspecies * ORC_MAX_PATHWAYS);
  for (unsigned i = 0; i < nspecies * nspecies; i++) s->bimol_p[i] = -1;
  for (unsigned i = 0; i < nspecies * nspecies * ORC_MAX_PATHWAYS; i++) s->bimol_rxn[i] = -1;
  s->can_vol_react = (int*)calloc(nspecies, sizeof(int));
  s->occ = (idvec*)calloc(s->nsub3, sizeof(idvec));
  return s;
}

/* reaction r (probability p) of the pair (a, b): a further pathway of the pair's class;
   returns 0, or -1 when the class is full */
static int scene_set_bimol(oscene* s, unsigned r, unsigned a, unsigned b, double p) {
  const unsigned ab = a * s->nspecies + b, ba = b * s->nspecies + a;
  const int k = s->bimol_npw[ab];
  if (k >= ORC_MAX_PATHWAYS) return -1;
  const double c = (k ? s->bimol_cum[ab * ORC_MAX_PATHWAYS + k - 1] : 0.0) + p;
  for (int pass = 0; pass < (ab == ba ? 1 : 2); pass++) {
    const unsigned q = pass ? ba : ab;
    s->bimol_cum[q * ORC_MAX_PATHWAYS + k] = c;
    s->bimol_rxn[q * ORC_MAX_PATHWAYS + k] = (int)r;
    s->bimol_npw[q] = k + 1;
    s->bimol_p[q] = c;
  }
  s->can_vol_react[a] = 1;
  s->can_vol_react[b] = 1;
  return 0;
}

static void scene_free(oscene* s) {
  if (!s) return;
  for (unsigned i = 0; i < s->nsub3; i++) free(s->occ[i].ids);
  free(s->occ);
  free(s->mols);
  free(s->verts);
  free(s->walls);
  free(s->wsp_off);
  free(s->wsp_list);
  free(s->space_step);
  free(s->wall_class);
  free(s->can_volwall);
  free(s->bimol_p);
  free(s->bimol_cum);
  free(s->bimol_npw);
  free(s->bimol_rxn);
  free(s->can_vol_react);
  free(s);
}

/* ------------------------------------------------------------------ RNG */

typedef struct {
  int injected;
  const unsigned* draws;
  unsigned n, used;
  int overrun;
  uint64_t s[4]; /* xoshiro256** state for the engine */
  int have_spare;
  double spare;
} orng;

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t xoshiro_next(orng* r) {
  uint64_t res = rotl(r->s[1] * 5, 7) * 9;
  uint64_t t = r->s[1] << 17;
  r->s[2] ^= r->s[0];
  r->s[3] ^= r->s[1];
  r->s[1] ^= r->s[2];
  r->s[0] ^= r->s[3];
  r->s[2] ^= t;
  r->s[3] = rotl(r->s[3], 45);
  return res;
}
static void rng_seed(orng* r, uint64_t seed) {
  memset(r, 0, sizeof(*r));
  uint64_t z = seed;
  for (int i = 0; i < 4; i++) { /* splitmix64 */
    z += 0x9e3779b97f4a7c15ull;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    r->s[i] = x ^ (x >> 31);
  }
}
static inline unsigned rng_uint(orng* r) {
  if (r->injected) {
    if (r->used >= r->n) {
      r->overrun = 1;
      return 0;
    }
    return r->draws[r->used++];
  }
  return (unsigned)(xoshiro_next(r) >> 32);
}
/* rng_dbl: 32-bit draw * 2^-32 (src/isaac64.h isaac64_dbl32) */
static inline double rng_dbl(orng* r) { return (double)rng_uint(r) * (1.0 / 4294967296.0); }
/* standard normal for the engine (Marsaglia polar method on 53-bit uniforms) */
static double rng_gauss(orng* r) {
  if (r->have_spare) {
    r->have_spare = 0;
    return r->spare;
  }
  double u, v, q;
  do {
    u = (double)(xoshiro_next(r) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    v = (double)(xoshiro_next(r) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    q = u * u + v * v;
  } while (q >= 1.0 || q == 0.0);
  double f = sqrt(-2.0 * log(q) / q);
  r->spare = v * f;
  r->have_spare = 1;
  return u * f;
}

/* ------------------------------------------------------------------ collisions */

enum { CT_MISS = 0, CT_REDO, CT_FRONT, CT_BACK, CT_VV };

typedef struct {
  int type;
  double time;
  v3 pos;
  unsigned partner; /* molecule id (vol-vol) */
  unsigned wall;
  unsigned cls;     /* reaction class of the pair (vol-vol): index a * nspecies + b */
} ocoll;

#define MAX_COLL 256
typedef struct {
  ocoll c[MAX_COLL];
  int n;
} ocolls;

/* get_displacement_up_to_partition_boundary (collision_utils.inl:48-114) */
static v3 disp_up_to_partition_boundary(const oscene* s, v3 pos, v3 disp) {
  v3 nz = guard_zero(disp);
  v3 dir = V(nz.x > 0 ? 1 : 0, nz.y > 0 ? 1 : 0, nz.z > 0 ? 1 : 0);
  v3 edges = vadd(s->origin, vscale(dir, s->part_edge));
  v3 diff = vsub(edges, pos);
  double hit_time = 1;
  if (fabs(diff.x) < POS_EPS || fabs(diff.y) < POS_EPS || fabs(diff.z) < POS_EPS) {
    return V(0, 0, 0);
  }
  v3 t = vdiv(diff, nz);
  if (t.x >= 0 && t.x < t.y && t.x <= t.z) hit_time = t.x;
  else if (t.y >= 0 && t.y <= t.z) hit_time = t.y;
  else if (t.z >= 0) hit_time = t.z;
  return vscale(disp, hit_time - STIME_EPS);
}

typedef struct {
  unsigned w[512];
  int nw;
  unsigned m[512];
  int nm;
} ospset;

static void set_insert(ospset* st, unsigned sp) {
  for (int i = 0; i < st->nm; i++) if (st->m[i] == sp) return;
  if (st->nm < 512) st->m[st->nm++] = sp;
}

/* collect_neighboring_subparts (collision_utils_subparts.inl:38-122) */
static void collect_neighbors(const oscene* s, v3 pos, int ix, int iy, int iz, double r, ospset* st) {
  double part_len = s->part_edge;
  v3 rel = vsub(pos, s->origin);
  v3 plus = vadd(rel, V(r, r, r));
  v3 minus = vsub(rel, V(r, r, r));
  v3 boundary = vmul(V(ix, iy, iz), V(s->sp_edge, s->sp_edge, s->sp_edge));
  int xd = 0, yd = 0, zd = 0;
  if (minus.x < boundary.x && minus.x > 0.0) { set_insert(st, subpart_of_3d(s, ix - 1, iy, iz)); xd = -1; }
  else if (plus.x > boundary.x + s->sp_edge && plus.x < part_len) { set_insert(st, subpart_of_3d(s, ix + 1, iy, iz)); xd = 1; }
  if (minus.y < boundary.y && minus.y > 0.0) { set_insert(st, subpart_of_3d(s, ix, iy - 1, iz)); yd = -1; }
  else if (plus.y > boundary.y + s->sp_edge && plus.y < part_len) { set_insert(st, subpart_of_3d(s, ix, iy + 1, iz)); yd = 1; }
  if (minus.z < boundary.z && minus.z > 0.0) { set_insert(st, subpart_of_3d(s, ix, iy, iz - 1)); zd = -1; }
  else if (plus.z > boundary.z + s->sp_edge && plus.z < part_len) { set_insert(st, subpart_of_3d(s, ix, iy, iz + 1)); zd = 1; }
  if (xd && yd) set_insert(st, subpart_of_3d(s, ix + xd, iy + yd, iz));
  if (xd && zd) set_insert(st, subpart_of_3d(s, ix + xd, iy, iz + zd));
  if (yd && zd) set_insert(st, subpart_of_3d(s, ix, iy + yd, iz + zd));
  if (xd && yd && zd) set_insert(st, subpart_of_3d(s, ix + xd, iy + yd, iz + zd));
}

/* collect_crossed_subparts (collision_utils_subparts.inl:127-300) */
static unsigned collect_crossed(const oscene* s, v3 pos, unsigned cur_sp, v3 disp, double R,
                                int for_mols, int for_walls, ospset* st) {
  if (for_walls) st->w[st->nw++] = cur_sp;
  if (for_mols) set_insert(st, cur_sp);
  v3 dest = vadd(pos, disp);
  v3 nz = guard_zero(disp);
  int dx = nz.x > 0, dy = nz.y > 0, dz = nz.z > 0;
  int sx, sy, sz, ex, ey, ez;
  subpart_3d_from_index(s, cur_sp, &sx, &sy, &sz);
  subpart_3d(s, dest, &ex, &ey, &ez);
  double rn = R * POS_SQRT2;
  if (for_mols) collect_neighbors(s, pos, sx, sy, sz, rn, st);
  unsigned dest_sp = subpart_of_3d(s, ex, ey, ez);
  if (cur_sp != dest_sp) {
    int ax = dx ? 1 : -1, ay = dy ? 1 : -1, az = dz ? 1 : -1;
    v3 cp = pos;
    int cx = sx, cy = sy, cz = sz;
    unsigned csp;
    v3 rcp = vdiv(V(1.0, 1.0, 1.0), nz);
    do {
      v3 len = V(s->sp_edge, s->sp_edge, s->sp_edge);
      v3 edges = vadd(vadd(s->origin, vmul(V(cx, cy, cz), len)), vmul(V(dx, dy, dz), len));
      v3 diff = vsub(edges, cp);
      v3 t = vmul(diff, rcp);
      if (t.x < t.y && t.x <= t.z) {
        cp = vadd(cp, vscale(disp, t.x));
        cx += ax;
        if (cx < 0 || cx >= (int)s->nsub) break;
      }
      else if (t.y <= t.z) {
        cp = vadd(cp, vscale(disp, t.y));
        cy += ay;
        if (cy < 0 || cy >= (int)s->nsub) break;
      }
      else {
        cp = vadd(cp, vscale(disp, t.z));
        cz += az;
        if (cz < 0 || cz >= (int)s->nsub) break;
      }
      csp = subpart_of_3d(s, cx, cy, cz);
      if (for_walls && st->nw < 512) st->w[st->nw++] = csp;
      if (for_mols) set_insert(st, csp);
      if (for_mols) collect_neighbors(s, cp, cx, cy, cz, rn, st);
    } while (csp != dest_sp);
  }
  if (for_mols) collect_neighbors(s, dest, ex, ey, ez, rn, st);
  return dest_sp;
}

/* jump_away_line (collision_utils.inl:568-603, fp64 branch) */
static void jump_away_line(v3 p, double k, v3 A, v3 B, v3 n, orng* rng, v3* v) {
  v3 e = vsub(B, A);
  double elen2 = vdot(e, e);
  double le_1 = 1.0 / sqrt(elen2);
  e = vmul(e, V(le_1, le_1, le_1));
  v3 f;
  f.x = n.y * e.z - n.z * e.y;
  f.y = n.z * e.x - n.x * e.z;
  f.z = n.x * e.y - n.y * e.x;
  double tiny = POS_EPS * (abs_max_2vec(p, *v) + 1.0) / (k * max3abs(f));
  if ((rng_uint(rng) & 1) == 0) tiny = -tiny;
  v->x -= tiny * f.x;
  v->y -= tiny * f.y;
  v->z -= tiny * f.z;
}

/* collide_wall (collision_utils.inl:629-812) */
static int collide_wall(const oscene* s, v3 pos, unsigned wi, orng* rng, int update_move, v3* move,
                        double* ct, v3* cpos) {
  const owall* w = &s->walls[wi];
  v3 normal = w->normal;
  double dp = vdot(normal, pos);
  double dv = vdot(normal, *move);
  double dd = dp - w->d;
  double d_eps;
  if (dd > 0) {
    d_eps = POS_EPS;
    if (dd < d_eps) d_eps = 0.5 * dd;
    if (dd + dv > d_eps) return CT_MISS;
  }
  else {
    d_eps = -POS_EPS;
    if (dd > d_eps) d_eps = 0.5 * dd;
    if (dd < 0 && dd + dv < d_eps) return CT_MISS;
  }
  double a;
  if (dd == 0) {
    if (dv != 0) return CT_MISS;
    if (update_move) {
      a = (abs_max_2vec(pos, *move) + 1.0) * POS_EPS;
      if ((rng_uint(rng) & 1) == 0) a = -a;
      *move = vsub(*move, vmul(V(a, a, a), normal));
      return CT_REDO;
    }
    return CT_MISS;
  }
  a = 1.0 / dv;
  a *= -dd;
  *ct = a;
  *cpos = vadd(pos, vscale(*move, a));
  v3 v0 = s->verts[w->vi[0]];
  v3 local = vsub(*cpos, v0);
  double b = vdot(local, w->unit_u);
  double c = vdot(local, w->unit_v);
  double f;
  if (w->uv2v < 0) {
    c = -c;
    f = -w->uv2v;
  }
  else {
    f = w->uv2v;
  }
  if (c > 0) {
    double g = b * f;
    double h = c * w->uv2u;
    if (g > h) {
      if (c * w->uv1u + g < h + w->uv1u * w->uv2v) {
        return dv > 0 ? CT_BACK : CT_FRONT;
      }
      else if (!distinguishable(c * w->uv1u + g, h + w->uv1u * w->uv2v, POS_EPS)) {
        if (update_move) {
          jump_away_line(pos, a, s->verts[w->vi[1]], s->verts[w->vi[2]], w->normal, rng, move);
          return CT_REDO;
        }
        return CT_MISS;
      }
      return CT_MISS;
    }
    else if (!distinguishable(g, h, POS_EPS)) {
      if (update_move) {
        jump_away_line(pos, a, s->verts[w->vi[2]], v0, w->normal, rng, move);
        return CT_REDO;
      }
      return CT_MISS;
    }
    return CT_MISS;
  }
  else if (!distinguishable(c, 0.0, POS_EPS)) {
    if (update_move) {
      jump_away_line(pos, a, v0, s->verts[w->vi[1]], w->normal, rng, move);
      return CT_REDO;
    }
    return CT_MISS;
  }
  return CT_MISS;
}

/* get_closest_wall_collision (collision_utils.inl:819-914, fp64 branch) */
static int closest_wall_collision(const oscene* s, v3 pos, unsigned sp, unsigned last_hit, orng* rng,
                                  v3* disp, v3* disp_up_to_wall, ocoll* closest) {
restart:;
  int found = 0;
  double closest_t = TIME_FOREVER;
  for (unsigned k = s->wsp_off[sp]; k < s->wsp_off[sp + 1]; k++) {
    unsigned wi = s->wsp_list[k];
    if (wi == last_hit) continue;
    double t;
    v3 cp;
    int ct = collide_wall(s, pos, wi, rng, 1, disp, &t, &cp);
    if (ct == CT_REDO) {
      if (rng->overrun) return 0;
      goto restart;
    }
    else if (ct != CT_MISS) {
      if (subpart_index(s, cp) != sp) continue;
      if (t < closest_t) {
        found = 1;
        closest_t = t;
        closest->type = ct;
        closest->time = t;
        closest->pos = cp;
        closest->wall = wi;
        closest->partner = IDX_INVALID;
      }
    }
  }
  if (found) *disp_up_to_wall = vsub(closest->pos, pos);
  return found;
}

/* collide_mol (collision_utils.inl:464-515) */
static int collide_mol(const oscene* s, v3 pos, unsigned self, v3 disp, unsigned target, double* t, v3* cpos) {
  const omol* tm = &s->mols[target];
  v3 dir = vsub(tm->pos, pos);
  double d = vdot(dir, disp);
  if (d < 0) return 0;
  double movelen2 = vdot(disp, disp);
  if (d > movelen2) return 0;
  double dirlen2 = vdot(dir, dir);
  double sigma2 = s->R * s->R;
  if (movelen2 * dirlen2 - d * d > movelen2 * sigma2) return 0;
  if (self == target) return 0;
  if (tm->defunct) return 0;
  *t = d / movelen2;
  *cpos = vadd(pos, vscale(disp, *t));
  return 1;
}

/* sort_collisions_by_time (diffuse_react_event.cpp:341-364): time ascending, vol-vol ties by id descending */
static int coll_before(const ocoll* a, const ocoll* b) {
  if (a->time < b->time) return 1;
  if (a->time > b->time) return 0;
  if (a->type == CT_VV && b->type == CT_VV) return a->partner > b->partner;
  return 0;
}
static void sort_collisions(ocolls* c) {
  for (int i = 1; i < c->n; i++) {
    ocoll x = c->c[i];
    int j = i - 1;
    while (j >= 0 && coll_before(&x, &c->c[j])) {
      c->c[j + 1] = c->c[j];
      j--;
    }
    c->c[j + 1] = x;
  }
}

enum { RT_FINISHED = 0, RT_HIT_WALL = 1 };

/* ray_trace_vol (diffuse_react_event.cpp:627-780, fp64 branch) */
static int ray_trace_vol(const oscene* s, unsigned id, v3* pos, unsigned* sp, unsigned species, orng* rng,
                         int can_vol_react, unsigned last_hit, v3* remaining, ocolls* colls) {
  int res = RT_FINISHED;
  colls->n = 0;
  double R = s->R;
  v3 pdisp;
  if (!in_partition(s, vadd(*pos, *remaining))) pdisp = disp_up_to_partition_boundary(s, *pos, *remaining);
  else pdisp = *remaining;
  ospset st;
  st.nw = st.nm = 0;
  unsigned last_sp = collect_crossed(s, *pos, *sp, pdisp, R, can_vol_react, 1, &st);
  v3 up_to_wall = *remaining;
  int hit_in_last = 0;
  for (int i = 0; i < st.nw; i++) {
    ocoll cc;
    if (closest_wall_collision(s, *pos, st.w[i], last_hit, rng, remaining, &up_to_wall, &cc)) {
      colls->c[colls->n++] = cc;
      res = RT_HIT_WALL;
      hit_in_last = last_sp == st.w[i];
      break;
    }
  }
  if (can_vol_react) {
    if (res == RT_HIT_WALL && !hit_in_last) {
      st.nw = st.nm = 0;
      collect_crossed(s, *pos, *sp, up_to_wall, R, 1, 0, &st);
    }
    for (int i = 0; i < st.nm; i++) {
      const idvec* occ = &s->occ[st.m[i]];
      for (unsigned k = 0; k < occ->n; k++) {
        unsigned pid = occ->ids[k];
        double p = s->bimol_p[species * s->nspecies + s->mols[pid].species];
        if (p < 0) continue;
        double t;
        v3 cp;
        if (collide_mol(s, *pos, id, *remaining, pid, &t, &cp) && colls->n < MAX_COLL) {
          ocoll* c = &colls->c[colls->n++];
          c->type = CT_VV;
          c->time = t;
          c->pos = cp;
          c->partner = pid;
          c->wall = IDX_INVALID;
          c->cls = species * s->nspecies + s->mols[pid].species;
        }
      }
    }
  }
  if (res == RT_FINISHED) {
    *pos = vadd(*pos, *remaining);
    *sp = subpart_index(s, *pos);
  }
  return res;
}

/* binary_search_double (rxn_utils.inl:301-321) with mult = 1: the pathway a probability
   selects from a class's cumulative probabilities (get_pathway_index_for_probability) */
static int pathway_for(const double* cum, int npw, double match) {
  int lo = 0, hi = npw - 1;
  while (hi - lo > 1) {
    int mid = (hi + lo) / 2;
    if (match > cum[mid]) lo = mid;
    else hi = mid;
  }
  return match > cum[lo] ? hi : lo;
}

/* test_bimolecular (rxn_utils.inl:336-414): the pathway that fires, or -2 */
static int test_bimolecular(const double* cum, int npw, double scaling, orng* rng) {
  double max_fixed_p = cum[npw - 1];
  double prob;
  if (max_fixed_p < scaling) {
    prob = rng_dbl(rng) * scaling;
    if (prob >= max_fixed_p) return -2;
  }
  else {
    float max_p = (float)max_fixed_p;
    if (max_p >= scaling) {
      prob = rng_dbl(rng) * max_p;
    }
    else {
      prob = rng_dbl(rng) * scaling;
      if (prob >= max_p) return -2;
    }
  }
  return pathway_for(cum, npw, prob);
}

/* which_unimolecular (rxn_utils.inl:774-783): a draw only for several pathways */
static int which_unimolecular(const double* cum, int npw, orng* rng) {
  if (npw <= 1) return 0;
  double match = rng_dbl(rng) * cum[npw - 1];
  return pathway_for(cum, npw, match);
}

/* test_intersect (rxn_utils.inl:593-626) for an absorptive class (rate DBL_GIGANTIC) */
static int test_intersect_absorb(double scaling, orng* rng) {
  double max_prob = GIGANTIC;
  double p;
  if (max_prob > scaling) {
    p = rng_dbl(rng) * max_prob;
  }
  else {
    p = rng_dbl(rng) * scaling;
    if (p > max_prob) return -2;
  }
  if (p > max_prob) return -2;
  (void)rng_dbl(rng); /* pathway draw */
  return 0;
}

/* time_of_unimol (rxn_utils.inl:721-735) */
static double time_of_unimol(double k_tot, orng* rng) {
  double p = rng_dbl(rng);
  if (k_tot <= 0 || !distinguishable(p, 0, EPS)) return TIME_FOREVER;
  return -log(p) / k_tot;
}

/* ------------------------------------------------------------------ exact disk */

/* exd_zetize (exact_disk_utils.inl:54-80) */
static double zetize(double y, double x) {
  if (y >= 0) {
    if (x >= 0) {
      if (x < y) return 1 - 0.5 * x / y;
      return 0.5 * y / x;
    }
    if (-x < y) return 1 - 0.5 * x / y;
    return 2 + 0.5 * y / x;
  }
  if (x <= 0) {
    if (y < x) return 3 - 0.5 * x / y;
    return 2 + 0.5 * y / x;
  }
  if (x < -y) return 3 - 0.5 * x / y;
  return 4 + 0.5 * y / x;
}

/* exd_coordize (exact_disk_utils.inl:94-145) */
static void coordize(v3 mv, v3* m, v3* u, v3* v) {
  double a = 1 / sqrt(vdot(mv, mv));
  *m = vmul(V(a, a, a), mv);
  double mx2 = m->x * m->x, my2 = m->y * m->y, mz2 = m->z * m->z;
  if (mx2 > my2) {
    if (mx2 > mz2) {
      if (my2 > mz2) { *u = V(m->y, -m->x, 0); a = 1 - mz2; *v = V(m->z * m->x, m->z * m->y, -a); }
      else { *u = V(m->z, 0, -m->x); a = 1 - my2; *v = V(-m->y * m->x, a, -m->y * m->z); }
    }
    else { *u = V(-m->z, 0, m->x); a = 1 - my2; *v = V(m->y * m->x, -a, m->y * m->z); }
  }
  else {
    if (my2 > mz2) {
      if (mx2 > mz2) { *u = V(-m->y, m->x, 0); a = 1 - mz2; *v = V(-m->z * m->x, -m->z * m->y, a); }
      else { *u = V(0, m->z, -m->y); a = 1 - mx2; *v = V(-a, m->x * m->y, m->x * m->z); }
    }
    else { *u = V(0, -m->z, m->y); a = 1 - mx2; *v = V(a, -m->x * m->y, -m->x * m->z); }
  }
  a = 1 / sqrt(a);
  *u = vscale(*u, a);
  *v = vscale(*v, a);
}

typedef struct { double u, v, r2, zeta; } exv;

/* visible fraction of the disk of radius R around the origin when straight wall
   segments (pa[i], pb[i]) occlude it: integrate r(theta)^2 / 2 over the angular
   intervals between segment endpoints and pairwise segment crossings */
static double sweep_area(const exv* pa, const exv* pb, int n, double R2) {
  double ang[4 * 16 + 2 * 16 * 16];
  int na = 0;
  for (int i = 0; i < n; i++) {
    ang[na++] = atan2(pa[i].v, pa[i].u);
    ang[na++] = atan2(pb[i].v, pb[i].u);
  }
  for (int i = 0; i < n; i++) {
    for (int j = i + 1; j < n; j++) {
      double d1u = pb[i].u - pa[i].u, d1v = pb[i].v - pa[i].v;
      double d2u = pb[j].u - pa[j].u, d2v = pb[j].v - pa[j].v;
      double den = d1u * d2v - d1v * d2u;
      if (den == 0) continue;
      double wu = pa[j].u - pa[i].u, wv = pa[j].v - pa[i].v;
      double t = (wu * d2v - wv * d2u) / den;
      double s = (wu * d1v - wv * d1u) / den;
      if (t > 0 && t < 1 && s > 0 && s < 1) {
        ang[na++] = atan2(pa[i].v + t * d1v, pa[i].u + t * d1u);
      }
    }
  }
  /* sort */
  for (int i = 1; i < na; i++) {
    double x = ang[i];
    int j = i - 1;
    while (j >= 0 && ang[j] > x) { ang[j + 1] = ang[j]; j--; }
    ang[j + 1] = x;
  }
  double area = 0;
  for (int k = 0; k < na; k++) {
    double a0 = ang[k];
    double a1 = (k + 1 < na) ? ang[k + 1] : ang[0] + 2 * MY_PI;
    if (a1 - a0 <= 0) continue;
    double am = 0.5 * (a0 + a1);
    double cu = cos(am), cv = sin(am);
    /* nearest segment along the mid ray */
    int best = -1;
    double best_r = sqrt(R2);
    for (int i = 0; i < n; i++) {
      double du = pb[i].u - pa[i].u, dv = pb[i].v - pa[i].v;
      double den = cu * dv - cv * du;
      if (den == 0) continue;
      double r = (pa[i].u * dv - pa[i].v * du) / den;
      double s = (pa[i].u * cv - pa[i].v * cu) / den;
      if (r > 0 && s >= 0 && s <= 1 && r < best_r) {
        best_r = r;
        best = i;
      }
    }
    if (best < 0) {
      area += 0.5 * R2 * (a1 - a0);
    }
    else {
      double du = pb[best].u - pa[best].u, dv = pb[best].v - pa[best].v;
      double c0u = cos(a0), c0v = sin(a0), c1u = cos(a1), c1v = sin(a1);
      double r0 = (pa[best].u * dv - pa[best].v * du) / (c0u * dv - c0v * du);
      double r1 = (pa[best].u * dv - pa[best].v * du) / (c1u * dv - c1v * du);
      area += 0.5 * r0 * r1 * sin(a1 - a0);
    }
  }
  return area;
}

/* exact_disk (exact_disk_utils.inl:840-1145) with use_expanded_list = true */
static double exact_disk(const oscene* s, v3 loc, v3 mv, double R, unsigned moving_species, v3 target_pos) {
  double R2 = R * R;
  double m2_i = 1 / vdot(mv, mv);
  v3 m, u, v;
  coordize(mv, &m, &u, &v);
  v3 Lmuv = V(vdot(loc, m), vdot(loc, u), vdot(loc, v));
  exv sm;
  if (!distinguishable_vec3(loc, target_pos, POS_EPS)) {
    sm.u = sm.v = sm.r2 = sm.zeta = 0;
  }
  else {
    v3 td = vsub(target_pos, loc);
    sm.u = vdot(td, u);
    sm.v = vdot(td, v);
    sm.r2 = sm.u * sm.u + sm.v * sm.v;
    sm.zeta = zetize(sm.v, sm.u);
  }
  exv ea[16], eb[16];
  int n_edges = 0;
  unsigned sp = subpart_index(s, loc);
  for (unsigned k = s->wsp_off[sp]; k < s->wsp_off[sp + 1]; k++) {
    unsigned wi = s->wsp_list[k];
    const owall* w = &s->walls[wi];
    v3 wv[3] = {s->verts[w->vi[0]], s->verts[w->vi[1]], s->verts[w->vi[2]]};
    double l_n = vdot(loc, w->normal);
    double d = w->d - l_n;
    double m_n = vdot(mv, w->normal);
    if (d * d >= R2 * (1 - m2_i * m_n * m_n)) continue;
    v3 llf, urb;
    wall_bbox(wv, &llf, &urb);
    double a, b;
    b = R2 * (1 - mv.x * mv.x * m2_i);
    a = llf.x - loc.x; if (a > 0 && a * a >= b) continue;
    a = loc.x - urb.x; if (a > 0 && a * a >= b) continue;
    b = R2 * (1 - mv.y * mv.y * m2_i);
    a = llf.y - loc.y; if (a > 0 && a * a >= b) continue;
    a = loc.y - urb.y; if (a > 0 && a * a >= b) continue;
    b = R2 * (1 - mv.z * mv.z * m2_i);
    a = llf.z - loc.z; if (a > 0 && a * a >= b) continue;
    a = loc.z - urb.z; if (a > 0 && a * a >= b) continue;
    if (s->can_volwall[moving_species] && s->wall_class[(size_t)wi * s->nspecies + moving_species] == 1) {
      continue; /* transparent for the moving species */
    }
    v3 p0 = vsub(V(vdot(wv[0], m), vdot(wv[0], u), vdot(wv[0], v)), Lmuv);
    v3 p1 = vsub(V(vdot(wv[1], m), vdot(wv[1], u), vdot(wv[1], v)), Lmuv);
    v3 p2 = vsub(V(vdot(wv[2], m), vdot(wv[2], u), vdot(wv[2], v)), Lmuv);
    exv pa, pb;
    /* compute_intersect_w_m0 (:213-223) on the two edges that cross m = 0 */
#define ISECT(P, Q, OUT) do { double t_ = (P).x / ((P).x - (Q).x); \
      (OUT).u = (P).y + t_ * ((Q).y - (P).y); (OUT).v = (P).z + t_ * ((Q).z - (P).z); } while (0)
    if ((p0.x < 0) == (p1.x < 0)) {
      if ((p2.x < 0) == (p1.x < 0)) continue;
      ISECT(p0, p2, pa);
      ISECT(p1, p2, pb);
    }
    else if ((p0.x < 0) == (p2.x < 0)) {
      ISECT(p0, p1, pa);
      ISECT(p2, p1, pb);
    }
    else {
      ISECT(p1, p0, pa);
      ISECT(p2, p0, pb);
    }
#undef ISECT
    pa.r2 = pa.u * pa.u + pa.v * pa.v;
    pb.r2 = pb.u * pb.u + pb.v * pb.v;
    if (pa.r2 < POS_EPS * R2 || pb.r2 < POS_EPS * R2) return -1;
    if (!distinguishable(pa.u * pb.v, pb.u * pa.v, POS_EPS) && (pa.u * pb.u + pa.v * pb.v) < 0) return -1;
    /* test_intersect_line_with_circle (:226-272) */
    double ti = 0, si = 1;
    if (pa.r2 > R2 || pb.r2 > R2) {
      double pa_pb = pa.u * pb.u + pa.v * pb.v;
      if (!distinguishable(pa.r2 + pb.r2, 2 * pa_pb, POS_EPS)) {
        if (sm.r2 < pa.r2 && sm.r2 < pb.r2 && distinguishable(sm.r2, pa.r2, POS_EPS) &&
            distinguishable(sm.r2, pa.r2, POS_EPS)) {
          continue;
        }
        if (!distinguishable(sm.u * pa.v, sm.v * pa.u, POS_SQRT_EPS) ||
            !distinguishable(sm.u * pb.v, sm.v * pb.u, POS_SQRT_EPS)) {
          return -1;
        }
        continue;
      }
      double ia = 1 / (pa.r2 + pb.r2 - 2 * pa_pb);
      double ib = (pa_pb - pa.r2) * ia;
      double ic = (R2 - pa.r2) * ia;
      double id = ib * ib + ic;
      if (id <= 0) continue;
      id = sqrt(id);
      ti = -ib - id;
      if (ti >= 1) continue;
      if (ti < 0) ti = 0;
      si = -ib + id;
      if (si <= 0) continue;
      if (si > 1) si = 1;
    }
    /* construct_final_endpoints (:275-307) */
    exv qa, qb;
    if (ti > 0) {
      qa.u = pa.u + ti * (pb.u - pa.u);
      qa.v = pa.v + ti * (pb.v - pa.v);
      qa.r2 = qa.u * qa.u + qa.v * qa.v;
      qa.zeta = zetize(qa.v, qa.u);
    }
    else {
      qa = pa;
      qa.zeta = zetize(pa.v, pa.u);
    }
    if (si < 1) {
      qb.u = pa.u + si * (pb.u - pa.u);
      qb.v = pa.v + si * (pb.v - pa.v);
      qb.r2 = qb.u * qb.u + qb.v * qb.v;
      qb.zeta = zetize(qb.v, qb.u);
    }
    else {
      qb = pb;
      qb.zeta = zetize(pb.v, pb.u);
    }
    a = qb.zeta - qa.zeta;
    if (a < 0) a += 4;
    if (a >= 2) {
      exv t = qa;
      qa = qb;
      qb = t;
      a = 4 - a;
    }
    b = sm.zeta - qa.zeta;
    if (b < 0) b += 4;
    if (b < a) {
      double au = qa.u - sm.u, av = qa.v - sm.v, bu = qb.u - sm.u, bv = qb.v - sm.v;
      double c = au * bv - av * bu;
      if (c < 0 || !distinguishable(au * bv, av * bu, POS_EPS)) return -1;
    }
    if (n_edges < 16) {
      ea[n_edges] = qa;
      eb[n_edges] = qb;
      n_edges++;
    }
  }
  if (n_edges == 0) return 1;
  if (n_edges == 1) {
    double ares = ea[0].u * eb[0].u + ea[0].v * eb[0].v;
    double bres = ea[0].u * eb[0].v - ea[0].v * eb[0].u;
    double sres;
    if (ares <= 0) sres = atan(-ares / bres) + 0.5 * MY_PI;
    else sres = atan(bres / ares);
    return (0.5 * bres + R2 * (MY_PI - 0.5 * sres)) / (MY_PI * R2);
  }
  return sweep_area(ea, eb, n_edges, R2) / (MY_PI * R2);
}

/* ------------------------------------------------------------------ one molecule step */

typedef struct {
  int status;       /* 0 finished, 1 reacted, 2 absorbed, 3 error */
  unsigned partner; /* reaction partner */
  int pathway;      /* pathway of the pair's reaction class that fired */
  double rxn_time;  /* absolute time of the reaction / absorption */
  v3 rxn_pos;
  double elapsed, t_steps;
} ostep;

static void put_event(double* out, int kind, int index, int side, double t_rel, double t_abs, v3 pos) {
  if (!out) return;
  int n = (int)out[6];
  if (n < ORC_EV_MAX) {
    double* e = out + ORC_RES_HDR + n * ORC_EV_SIZE;
    e[0] = kind; e[1] = index; e[2] = side; e[3] = t_rel; e[4] = t_abs;
    e[5] = pos.x; e[6] = pos.y; e[7] = pos.z;
  }
  out[6] = n + 1;
}

/* DiffuseReactEvent::diffuse_vol_molecule (diffuse_react_event.cpp:367-618), volume branch,
   from the point where the displacement is known */
static ostep diffuse_vol(oscene* s, unsigned id, v3 disp, orng* rng, double r_rate_factor, double t_steps,
                         double start_time, double* out) {
  omol* vm = &s->mols[id];
  unsigned species = vm->species;
  int can_vol_react = s->can_vol_react[species];
  v3 remaining = disp;
  unsigned last_hit = IDX_INVALID;
  double elapsed = start_time;
  ostep res;
  memset(&res, 0, sizeof(res));
  ocolls colls;
  int state, was_defunct = 0, guard = 0;
  v3 pos = vm->pos;
  unsigned sp = vm->subpart;
  do {
    state = ray_trace_vol(s, id, &pos, &sp, species, rng, can_vol_react, last_hit, &remaining, &colls);
    if (colls.n > 1) sort_collisions(&colls);
    for (int i = 0; i < colls.n; i++) {
      ocoll* c = &colls.c[i];
      if (c->type == CT_VV) {
        if (c->time < STIME_EPS) continue; /* is_immediate_collision */
        double t_abs = elapsed + t_steps * c->time;
        double factor = exact_disk(s, c->pos, remaining, s->R, species, s->mols[c->partner].pos);
        if (factor < 0) {
          put_event(out, 6, (int)c->partner, 0, c->time, t_abs, c->pos);
          continue;
        }
        double scaling = factor * r_rate_factor;
        int pw = test_bimolecular(&s->bimol_cum[c->cls * ORC_MAX_PATHWAYS], s->bimol_npw[c->cls], scaling, rng);
        if (pw < 0) {
          put_event(out, 4, (int)c->partner, 0, c->time, t_abs, c->pos);
          continue;
        }
        put_event(out, 5, (int)c->partner, pw, c->time, t_abs, c->pos);
        was_defunct = 1;
        res.status = 1;
        res.pathway = pw;
        res.partner = c->partner;
        res.rxn_time = t_abs;
        res.rxn_pos = c->pos;
        break;
      }
      else {
        int side = c->type == CT_FRONT ? 1 : 2;
        int kind = s->wall_class[(size_t)c->wall * s->nspecies + species];
        double t_abs = elapsed + t_steps * c->time;
        if (kind == 1) {
          /* cross_transparent_wall (diffuse_react_event.cpp:3062-3094) */
          pos = c->pos;
          sp = subpart_index(s, pos);
          double t_smash = c->time;
          remaining = vmul(remaining, V(1.0 - t_smash, 1.0 - t_smash, 1.0 - t_smash));
          elapsed += t_steps * t_smash;
          t_steps *= (1.0 - t_smash);
          if (t_steps < EPS) t_steps = EPS;
          last_hit = c->wall;
          put_event(out, 2, (int)c->wall, side, c->time, t_abs, c->pos);
          break;
        }
        if (kind == 2 && test_intersect_absorb(r_rate_factor, rng) >= 0) {
          put_event(out, 3, (int)c->wall, side, c->time, t_abs, c->pos);
          was_defunct = 1;
          res.status = 2;
          res.rxn_time = t_abs;
          res.rxn_pos = c->pos;
          break;
        }
        /* reflect_from_wall (collision_utils.inl:1711-1747) */
        elapsed += t_steps * c->time;
        const owall* w = &s->walls[c->wall];
        double t_reflect = c->time;
        pos = c->pos;
        sp = subpart_index(s, pos);
        t_steps *= (1.0 - t_reflect);
        last_hit = c->wall;
        double rf = -2.0 * vdot(remaining, w->normal);
        remaining = vmul(vadd(remaining, vmul(V(rf, rf, rf), w->normal)),
                         V(1.0 - t_reflect, 1.0 - t_reflect, 1.0 - t_reflect));
        put_event(out, 1, (int)c->wall, side, c->time, t_abs, c->pos);
        break;
      }
    }
    if (rng->overrun || ++guard > 100000) {
      res.status = 3;
      break;
    }
  } while (state != RT_FINISHED && !was_defunct);
  if (rng->overrun) res.status = 3;
  /* the diffusing molecule's live position (ray_trace_vol moves it in place) */
  vm->pos = pos;
  vm->subpart = sp;
  res.elapsed = elapsed;
  res.t_steps = t_steps;
  return res;
}

/* ------------------------------------------------------------------ case API */

typedef struct {
  oscene* s;
} ocase_scene;

void* orc_scene_new(
    const double* origin, double partition_edge, unsigned nsub, double rxn_radius,
    unsigned nv, const double* verts, unsigned nw, const unsigned* tris,
    unsigned nspecies, const double* space_steps, const unsigned char* wall_class,
    unsigned nrxn, const unsigned* rxn_ab, const double* rxn_p,
    unsigned nmol, const double* mol_pos, const unsigned* mol_species) {
  oscene* s = scene_build(origin, partition_edge, nsub, rxn_radius, nv, verts, nw, tris, nspecies,
                          space_steps, wall_class);
  for (unsigned r = 0; r < nrxn; r++) scene_set_bimol(s, r, rxn_ab[2 * r], rxn_ab[2 * r + 1], rxn_p[r]);
  for (unsigned m = 0; m < nmol; m++) {
    scene_add_mol(s, V(mol_pos[3 * m], mol_pos[3 * m + 1], mol_pos[3 * m + 2]), mol_species[m]);
  }
  return s;
}

void orc_scene_free(void* s) { scene_free((oscene*)s); }

void orc_scene_info(void* sp, double* out) {
  oscene* s = (oscene*)sp;
  out[0] = s->sp_edge;
  out[1] = s->sp_rcp;
  out[2] = s->part_edge;
  out[3] = s->origin.x; out[4] = s->origin.y; out[5] = s->origin.z;
  out[6] = s->nsub;
}

void orc_scene_wall_consts(void* sp, double* out) {
  oscene* s = (oscene*)sp;
  for (unsigned i = 0; i < s->nw; i++) {
    const owall* w = &s->walls[i];
    double* o = out + 14 * i;
    o[0] = w->normal.x; o[1] = w->normal.y; o[2] = w->normal.z; o[3] = w->d;
    o[4] = w->unit_u.x; o[5] = w->unit_u.y; o[6] = w->unit_u.z;
    o[7] = w->unit_v.x; o[8] = w->unit_v.y; o[9] = w->unit_v.z;
    o[10] = w->uv1u; o[11] = w->uv2u; o[12] = w->uv2v; o[13] = 0;
  }
}

unsigned orc_scene_walls_in_subparts(void* sp, unsigned* counts, unsigned* list, unsigned cap) {
  oscene* s = (oscene*)sp;
  unsigned total = 0;
  for (unsigned i = 0; i < s->nsub3; i++) {
    counts[i] = s->wsp_off[i + 1] - s->wsp_off[i];
    for (unsigned k = s->wsp_off[i]; k < s->wsp_off[i + 1]; k++) {
      if (total < cap) list[total] = s->wsp_list[k];
      total++;
    }
  }
  return total;
}

unsigned orc_subpart_index(void* sp, const double* pos) {
  return subpart_index((oscene*)sp, V(pos[0], pos[1], pos[2]));
}

void orc_diffuse_case(void* sp, unsigned mol, const double* disp, const unsigned* draws, unsigned ndraws,
                      double r_rate_factor, double t_steps, double* out) {
  oscene* s = (oscene*)sp;
  omol saved = s->mols[mol];
  memset(out, 0, sizeof(double) * ORC_RES_SIZE);
  orng rng;
  memset(&rng, 0, sizeof(rng));
  rng.injected = 1;
  rng.draws = draws;
  rng.n = ndraws;
  ostep r = diffuse_vol(s, mol, V(disp[0], disp[1], disp[2]), &rng, r_rate_factor, t_steps, 0.0, out);
  out[0] = r.status;
  out[1] = s->mols[mol].pos.x; out[2] = s->mols[mol].pos.y; out[3] = s->mols[mol].pos.z;
  out[4] = s->mols[mol].subpart;
  out[5] = rng.used;
  out[7] = r.elapsed;
  out[8] = r.t_steps;
  s->mols[mol] = saved;
}

double orc_exact_disk(void* sp, const double* loc, const double* mv, unsigned moving, unsigned target) {
  oscene* s = (oscene*)sp;
  return exact_disk(s, V(loc[0], loc[1], loc[2]), V(mv[0], mv[1], mv[2]), s->R, s->mols[moving].species,
                    s->mols[target].pos);
}

int orc_test_bimolecular(double max_fixed_p, double scaling, unsigned draw) {
  return orc_test_bimolecular_pw(&max_fixed_p, 1, scaling, draw);
}

int orc_test_bimolecular_pw(const double* cum, unsigned n, double scaling, unsigned draw) {
  orng rng;
  memset(&rng, 0, sizeof(rng));
  rng.injected = 1;
  rng.draws = &draw;
  rng.n = 1;
  return test_bimolecular(cum, (int)n, scaling, &rng);
}

int orc_which_unimolecular(const double* cum, unsigned n, unsigned draw) {
  orng rng;
  memset(&rng, 0, sizeof(rng));
  rng.injected = 1;
  rng.draws = &draw;
  rng.n = 1;
  return which_unimolecular(cum, (int)n, &rng);
}

double orc_time_of_unimol(double k_tot, unsigned draw) {
  orng rng;
  memset(&rng, 0, sizeof(rng));
  rng.injected = 1;
  rng.draws = &draw;
  rng.n = 1;
  return time_of_unimol(k_tot, &rng);
}

/* ------------------------------------------------------------------ serial engine */

typedef struct {
  oscene* s;
  orng rng;
  unsigned nbimol, nunimol;
  int* bimol_prod;     /* [nbimol * 2] */
  /* unimolecular class of each species: cumulative rates and reaction index per pathway */
  int* uni_npw;        /* [nspecies] */
  double* uni_cum;     /* [nspecies * ORC_MAX_PATHWAYS] */
  int* uni_rxn;        /* [nspecies * ORC_MAX_PATHWAYS] */
  int* unimol_prod;    /* [nunimol * 2] */
  unsigned* queue;     /* new diffuse actions (ids), FIFO within an iteration */
  unsigned nqueue, capqueue;
  uint64_t iteration;
  uint64_t mol_steps;
  int error;
} oengine;

static void queue_push(oengine* e, unsigned id) {
  if (e->nqueue == e->capqueue) {
    e->capqueue = e->capqueue ? e->capqueue * 2 : 1024;
    e->queue = (unsigned*)realloc(e->queue, sizeof(unsigned) * e->capqueue);
  }
  e->queue[e->nqueue++] = id;
}

void* orc_engine_new(const orc_engine_desc* d) {
  oengine* e = (oengine*)calloc(1, sizeof(oengine));
  e->s = scene_build(d->origin, d->partition_edge, d->nsub, d->rxn_radius, d->nv, d->verts, d->nw, d->tris,
                     d->nspecies, d->space_steps, d->wall_class);
  e->nbimol = d->nbimol;
  e->bimol_prod = (int*)malloc(sizeof(int) * 2 * (d->nbimol ? d->nbimol : 1));
  for (unsigned r = 0; r < d->nbimol; r++) {
    scene_set_bimol(e->s, r, d->bimol_reactants[2 * r], d->bimol_reactants[2 * r + 1], d->bimol_p[r]);
    e->bimol_prod[2 * r] = d->bimol_products[2 * r];
    e->bimol_prod[2 * r + 1] = d->bimol_products[2 * r + 1];
  }
  e->nunimol = d->nunimol;
  e->uni_npw = (int*)calloc(d->nspecies, sizeof(int));
  e->uni_cum = (double*)calloc((size_t)d->nspecies * ORC_MAX_PATHWAYS, sizeof(double));
  e->uni_rxn = (int*)calloc((size_t)d->nspecies * ORC_MAX_PATHWAYS, sizeof(int));
  e->unimol_prod = (int*)malloc(sizeof(int) * 2 * (d->nunimol ? d->nunimol : 1));
  for (unsigned r = 0; r < d->nunimol; r++) {
    const unsigned a = d->unimol_reactant[r];
    const int k = e->uni_npw[a];
    if (k < ORC_MAX_PATHWAYS) {
      e->uni_cum[a * ORC_MAX_PATHWAYS + k] = (k ? e->uni_cum[a * ORC_MAX_PATHWAYS + k - 1] : 0.0) + d->unimol_k[r];
      e->uni_rxn[a * ORC_MAX_PATHWAYS + k] = (int)r;
      e->uni_npw[a] = k + 1;
    }
    e->unimol_prod[2 * r] = d->unimol_products[2 * r];
    e->unimol_prod[2 * r + 1] = d->unimol_products[2 * r + 1];
  }
  for (unsigned m = 0; m < d->nmol; m++) {
    unsigned id = scene_add_mol(e->s, V(d->mol_pos[3 * m], d->mol_pos[3 * m + 1], d->mol_pos[3 * m + 2]),
                                d->mol_species[m]);
    e->s->mols[id].diffusion_time = 0;
    e->s->mols[id].schedule_unimol = 1; /* released molecules get their unimol time on first diffusion */
  }
  rng_seed(&e->rng, d->seed);
  return e;
}

void orc_engine_free(void* ep) {
  oengine* e = (oengine*)ep;
  if (!e) return;
  scene_free(e->s);
  free(e->bimol_prod);
  free(e->uni_npw);
  free(e->uni_cum);
  free(e->uni_rxn);
  free(e->unimol_prod);
  free(e->queue);
  free(e);
}

static void set_defunct(oengine* e, unsigned id) {
  omol* m = &e->s->mols[id];
  if (m->defunct) return;
  occ_remove(e->s, id);
  m->defunct = 1;
}

static int before_iteration_end(const oengine* e, double t) {
  double end = (double)e->iteration + 1.0;
  return t < end && !(fabs(t - end) < EPS);
}

static void create_product(oengine* e, int species, v3 pos, double time) {
  if (species < 0) return;
  unsigned id = scene_add_mol(e->s, pos, (unsigned)species);
  omol* m = &e->s->mols[id];
  m->diffusion_time = time;
  m->schedule_unimol = 1;
  if (before_iteration_end(e, time)) queue_push(e, id);
}

/* pick_unimol_rxn_class_and_set_rxn_time (diffuse_react_event.cpp:1731-1760) */
static void set_unimol_time(oengine* e, omol* m, double now) {
  const int npw = e->uni_npw[m->species];
  if (npw == 0) {
    m->unimol_time = TIME_INVALID;
    return;
  }
  m->unimol_time = now + time_of_unimol(e->uni_cum[m->species * ORC_MAX_PATHWAYS + npw - 1], &e->rng);
}

/* DiffuseReactEvent::diffuse_single_molecule (diffuse_react_event.cpp:201-337) */
static void diffuse_single(oengine* e, unsigned id) {
  oscene* s = e->s;
  omol* m = &s->mols[id];
  if (m->defunct) return;
  double start = m->diffusion_time;
  if (m->unimol_time != TIME_INVALID && m->unimol_time <= start) {
    /* react_unimol_single_molecule / outcome_unimolecular (:1764-1826, :2939) */
    const int npw = e->uni_npw[m->species];
    if (npw > 0) {
      const double* cum = &e->uni_cum[m->species * ORC_MAX_PATHWAYS];
      const int r = e->uni_rxn[m->species * ORC_MAX_PATHWAYS + which_unimolecular(cum, npw, &e->rng)];
      v3 pos = m->pos;
      double t = m->unimol_time;
      set_defunct(e, id);
      create_product(e, e->unimol_prod[2 * r], pos, t);
      create_product(e, e->unimol_prod[2 * r + 1], pos, t);
      return;
    }
  }
  m = &s->mols[id];
  if (m->schedule_unimol) {
    m->schedule_unimol = 0;
    set_unimol_time(e, m, start);
  }
  /* get_max_time (:164-198) with the barrier one iteration ahead */
  double max_time = 1.0 - (m->diffusion_time - (double)e->iteration);
  if (m->unimol_time != TIME_INVALID && m->unimol_time < m->diffusion_time + max_time) {
    max_time = m->unimol_time - m->diffusion_time;
  }
  double space_step = s->space_step[m->species];
  if (space_step != 0) {
    /* compute_vol_displacement (diffusion_utils.inl:366-432) */
    double steps = 1.0, t_steps = 1.0, r_rate_factor = 1.0;
    if (t_steps > max_time) {
      t_steps = max_time;
      steps = max_time / 1.0;
    }
    if (steps < EPS) {
      steps = EPS;
      t_steps = EPS * 1.0;
    }
    double scale = space_step;
    if (steps != 1.0) {
      double rate_factor = sqrt(steps);
      r_rate_factor = 1.0 / rate_factor;
      scale = rate_factor * space_step;
    }
    v3 disp;
    disp.x = scale * rng_gauss(&e->rng) * 0.70710678118654752440;
    disp.y = scale * rng_gauss(&e->rng) * 0.70710678118654752440;
    disp.z = scale * rng_gauss(&e->rng) * 0.70710678118654752440;
    max_time = t_steps;
    e->mol_steps++;
    occ_remove(s, id);
    ostep r = diffuse_vol(s, id, disp, &e->rng, r_rate_factor, t_steps, start, NULL);
    m = &s->mols[id];
    if (!in_partition(s, m->pos)) {
      e->error = -1;
    }
    if (r.status == 1) {
      /* outcome_bimolecular / outcome_products_random (:1833-1895, :2446-2933) */
      m->defunct = 1;
      unsigned partner = r.partner;
      unsigned rx =
          (unsigned)s->bimol_rxn[(m->species * s->nspecies + s->mols[partner].species) * ORC_MAX_PATHWAYS + r.pathway];
      set_defunct(e, partner);
      create_product(e, e->bimol_prod[2 * rx], r.rxn_pos, r.rxn_time);
      create_product(e, e->bimol_prod[2 * rx + 1], r.rxn_pos, r.rxn_time);
      return;
    }
    if (r.status == 2) {
      m->defunct = 1;
      return;
    }
    occ_add(s, id); /* update_molecule_reactants_map (partition.h:406) */
  }
  m = &s->mols[id];
  m->diffusion_time += max_time;
  double end = (double)e->iteration + 1.0;
  if ((m->unimol_time != TIME_INVALID && m->unimol_time < end) || before_iteration_end(e, m->diffusion_time)) {
    queue_push(e, id);
  }
  else {
    double rounded = round(m->diffusion_time);
    if (fabs(m->diffusion_time - rounded) < SQRT_EPS) m->diffusion_time = rounded;
  }
}

int orc_engine_run(void* ep, unsigned n, uint64_t* counts_out) {
  oengine* e = (oengine*)ep;
  oscene* s = e->s;
  for (unsigned it = 0; it < n; it++) {
    /* DiffuseReactEvent::diffuse_molecules (diffuse_react_event.cpp:67-161) */
    unsigned nexisting = s->nmol;
    double end = (double)e->iteration + 1.0;
    for (unsigned id = 0; id < nexisting; id++) {
      omol* m = &s->mols[id];
      if (m->defunct || !(m->diffusion_time < end && !(fabs(m->diffusion_time - end) < EPS))) continue;
      diffuse_single(e, id);
    }
    for (unsigned q = 0; q < e->nqueue; q++) diffuse_single(e, e->queue[q]);
    e->nqueue = 0;
    e->iteration++;
    if (counts_out) {
      uint64_t* c = counts_out + (size_t)it * s->nspecies;
      memset(c, 0, sizeof(uint64_t) * s->nspecies);
      for (unsigned id = 0; id < s->nmol; id++) {
        if (!s->mols[id].defunct) c[s->mols[id].species]++;
      }
    }
    if (e->error) return e->error;
  }
  return 0;
}

uint64_t orc_engine_num_live(void* ep) {
  oengine* e = (oengine*)ep;
  uint64_t n = 0;
  for (unsigned id = 0; id < e->s->nmol; id++) n += !e->s->mols[id].defunct;
  return n;
}

uint64_t orc_engine_mol_steps(void* ep) { return ((oengine*)ep)->mol_steps; }

uint64_t orc_engine_molecules(void* ep, uint64_t cap, double* pos, unsigned* species) {
  oengine* e = (oengine*)ep;
  uint64_t n = 0;
  for (unsigned id = 0; id < e->s->nmol; id++) {
    const omol* m = &e->s->mols[id];
    if (m->defunct) continue;
    if (n < cap) {
      pos[3 * n] = m->pos.x;
      pos[3 * n + 1] = m->pos.y;
      pos[3 * n + 2] = m->pos.z;
      species[n] = m->species;
    }
    n++;
  }
  return n;
}
