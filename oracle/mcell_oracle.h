/*
 * mcell_oracle: CPU restatement (plain C, fp64) of MCell4's volume-molecule
 * diffuse-react step. TEST INFRASTRUCTURE ONLY: it is the checker for the CUDA
 * engine and the timed CPU baseline; the product never links or calls it.
 *
 * Every routine cites the reference file:line it restates. The restatement is
 * pinned against the reference's own routines (compiled into oracle/_ref by
 * oracle/ref/build_ref.py) through the golden fixtures in tests/golden/.
 *
 * Two surfaces:
 *   orc_scene_* / orc_diffuse_case: one molecule, one diffusion step, with the
 *     displacement and the random stream injected (per-routine parity harness);
 *   orc_engine_*: a serial engine with the reference's scheduling semantics
 *     (ensemble parity and CPU baseline).
 */
#ifndef MCELL_ORACLE_H
#define MCELL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* case result layout (doubles), identical to oracle/_ref and the GPU harness */
#define ORC_RES_HDR 9
#define ORC_EV_SIZE 8
#define ORC_EV_MAX 32
#define ORC_RES_SIZE (ORC_RES_HDR + ORC_EV_MAX * ORC_EV_SIZE)
/* pathways of one reaction class (reactions of one reactant pair, or unimolecular
   reactions of one species, in the order given) */
#define ORC_MAX_PATHWAYS 4

void* orc_scene_new(
    const double* origin, double partition_edge, unsigned nsub, double rxn_radius,
    unsigned nv, const double* verts, unsigned nw, const unsigned* tris,
    unsigned nspecies, const double* space_steps, const unsigned char* wall_class,
    unsigned nrxn, const unsigned* rxn_ab, const double* rxn_p,
    unsigned nmol, const double* mol_pos, const unsigned* mol_species);
void orc_scene_free(void* s);
void orc_scene_info(void* s, double* out);
void orc_scene_wall_consts(void* s, double* out);
unsigned orc_scene_walls_in_subparts(void* s, unsigned* counts, unsigned* list, unsigned cap);
unsigned orc_subpart_index(void* s, const double* pos);
void orc_diffuse_case(
    void* s, unsigned mol, const double* disp, const unsigned* draws, unsigned ndraws,
    double r_rate_factor, double t_steps, double* out);
double orc_exact_disk(void* s, const double* loc, const double* mv, unsigned moving, unsigned target);
int orc_test_bimolecular(double max_fixed_p, double scaling, unsigned draw);
/* the same over a class of n pathways (cumulative probabilities); pathway or < 0 */
int orc_test_bimolecular_pw(const double* cum, unsigned n, double scaling, unsigned draw);
/* which_unimolecular over n pathways (cumulative rates); the draw is used for n > 1 */
int orc_which_unimolecular(const double* cum, unsigned n, unsigned draw);
double orc_time_of_unimol(double k_tot, unsigned draw);

/* serial engine */
typedef struct orc_engine_desc {
  double origin[3];
  double partition_edge;
  unsigned nsub;
  double rxn_radius;
  unsigned nv;
  const double* verts;
  unsigned nw;
  const unsigned* tris;
  unsigned nspecies;
  const double* space_steps;          /* internal length units per time step */
  const unsigned char* wall_class;    /* [nw * nspecies]: 0 reflect, 1 transparent, 2 absorptive */
  unsigned nbimol;                    /* reactions of one pair are the pathways of its class */
  const unsigned* bimol_reactants;    /* [nbimol * 2] */
  const double* bimol_p;              /* probability per reaction */
  const int* bimol_products;          /* [nbimol * 2], -1 = none */
  unsigned nunimol;                   /* reactions of one species are the pathways of its class */
  const unsigned* unimol_reactant;    /* [nunimol] */
  const double* unimol_k;             /* rate * time_step (per iteration) */
  const int* unimol_products;         /* [nunimol * 2], -1 = none */
  unsigned nmol;
  const double* mol_pos;
  const unsigned* mol_species;
  uint64_t seed;
} orc_engine_desc;

void* orc_engine_new(const orc_engine_desc* d);
void orc_engine_free(void* e);
/* runs n iterations; counts_out (optional) gets [n * nspecies] live counts after each iteration.
   returns 0, or a negative error (molecule escaped the partition) */
int orc_engine_run(void* e, unsigned n, uint64_t* counts_out);
uint64_t orc_engine_num_live(void* e);
uint64_t orc_engine_mol_steps(void* e);
/* copies live molecules (pos xyz, species) in id order; returns the count */
uint64_t orc_engine_molecules(void* e, uint64_t cap, double* pos, unsigned* species);

#ifdef __cplusplus
}
#endif
#endif
