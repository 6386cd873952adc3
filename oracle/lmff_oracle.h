/* CPU oracle for the Tersoff + ILP force path: a plain-C restatement of the reference
 * algorithm (LAMMPS 3Mar2020 as shipped in the reference snapshot):
 *   MANYBODY/pair_tersoff.cpp          (compute :86-265, read_file :392-532,
 *                                       setup_params :536-580, kernels :584-811)
 *   USER-MISC/pair_ilp_graphene_hbn.cpp (read_file :246-387, init_one :226-240,
 *                                       calc_FvdW :449-541, calc_FRep :547-675,
 *                                       ILP_neigh :681-745, calc_normal :750-1075,
 *                                       Tap/dTap pair_ilp_graphene_hbn.h:80-115)
 *   npair_full_bin_ghost.cpp:36-140    (full list incl. ghosts, rsq <= cutneighsq)
 *   pair.cpp:1554 virial_fdotr_compute, pair.cpp:913/1060 ev_tally(_xyz) per-atom energy
 *
 * TEST INFRASTRUCTURE ONLY.  This code is the oracle for the CUDA engine: the parity
 * tests, the smoke check and the CPU-baseline leg of the benchmark may call it; the
 * engine never does.  Its own correctness is pinned against the reference binary built
 * from the reference sources (oracle/ref.mk) through the fixtures in tests/golden/.
 *
 * Periodic images are materialised as ghost atoms exactly as LAMMPS's brick
 * communication does (every image within cut_force + skin of the box), so the
 * reference's owned+ghost loops carry over unchanged; ghost forces and per-atom
 * energies are folded back onto their owners at the end (LAMMPS reverse_comm).
 */
#ifndef LMFF_ORACLE_H
#define LMFF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAXELEM 8
#define ORC_MAXTYPE 16

typedef struct {           /* pair_tersoff.h:38-53 */
  double lam1, lam2, lam3, c, d, h, gamma, powerm, powern, beta;
  double biga, bigb, bigd, bigr, cut, cutsq, c1, c2, c3, c4;
  int ielement, jelement, kelement, powermint;
} orc_ters_param;

typedef struct {           /* pair_ilp_graphene_hbn.h:53-57; the KC fields: pair_kolmogorov_crespi_full.h */
  double z0, alpha, epsilon, C, delta, d, sR, reff, C6, S;
  double delta2inv, seff, lambda, rcut;
  double C0, C2, C4, A, z06;   /* kolmogorov/crespi/full only */
  int ielement, jelement;
} orc_ilp_param;

typedef struct {
  int ntypes;
  /* Tersoff */
  int t_enabled, t_nelements, t_nparams;
  int t_map[ORC_MAXTYPE + 1];                 /* type -> element, -1 = NULL */
  orc_ters_param t_params[ORC_MAXELEM * ORC_MAXELEM * ORC_MAXELEM];
  int t_e2p[ORC_MAXELEM][ORC_MAXELEM][ORC_MAXELEM];
  double t_cutmax;
  /* interlayer style: ILP (i_model 0) or Kolmogorov-Crespi full (i_model 1) */
  int i_enabled, i_nelements, i_nparams, i_model;
  int i_map[ORC_MAXTYPE + 1];
  orc_ilp_param i_params[ORC_MAXELEM * ORC_MAXELEM];
  int i_e2p[ORC_MAXELEM][ORC_MAXELEM];
  double i_cutILPsq[ORC_MAXELEM][ORC_MAXELEM];
  double cut_global;
  int tap_flag;
  double skin;
  char err[256];
} orc_pot;

typedef struct {
  double e_tersoff, e_ilp, pvector[2];
  double virial[6], virial_tersoff[6], virial_ilp[6];
  int64_t nghost, nlist;
} orc_result;

/* Potential files.  elem_of_type[t-1] names the element of LAMMPS type t, or "NULL". */
int orc_pot_init(orc_pot *p, int ntypes, double cut_global, int tap_flag, double skin);
int orc_read_tersoff(orc_pot *p, const char *path, const char *const *elem_of_type);
int orc_read_ilp(orc_pot *p, const char *path, const char *const *elem_of_type);
/* kolmogorov/crespi/full parameter file (pair_kolmogorov_crespi_full.cpp:247-392) */
int orc_read_kc(orc_pot *p, const char *path, const char *const *elem_of_type);
const char *orc_pot_error(const orc_pot *p);

typedef struct orc_ctx orc_ctx;

orc_ctx *orc_new(const orc_pot *p, int nthreads);
void orc_free(orc_ctx *c);
const char *orc_error(const orc_ctx *c);
/* Set owned atoms and an orthogonal box; builds ghosts and the neighbour list. */
int orc_set_atoms(orc_ctx *c, int n, const double *x, const int *type, const int64_t *mol,
                  const int64_t *tag, const double lo[3], const double hi[3], const int periodic[3]);
/* New owned positions; rebuilds when any atom moved more than skin/2 since the last
 * build (neighbor.cpp:1947-1976 check), else refreshes ghost coordinates only. */
int orc_update_x(orc_ctx *c, const double *x);
/* Forces on owned atoms (overwritten), energies, pvector, fdotr virials, per-atom energy
 * (eatom may be NULL).  which: 1 = Tersoff, 2 = ILP, 3 = both. */
int orc_forces(orc_ctx *c, int which, double *f, double *eatom, orc_result *r);
/* The same with each style's per-atom virial (nlocal*6 each, xx yy zz xy xz yz,
 * overwritten; either may be NULL) as the reference's ev_tally, ev_tally_xyz and
 * v_tally3 calls split it over atoms, ghost shares folded into their owners. */
int orc_forces_va(orc_ctx *c, int which, double *f, double *eatom, double *vatom_ters, double *vatom_ilp,
                  orc_result *r);
/* Velocity-Verlet NVE (fix_nve.cpp:64-111, metal units) for nsteps; x, v, f in/out,
 * f must hold the forces of x on entry.  mass_of_type[t-1]. */
int orc_nve(orc_ctx *c, int nsteps, double dt, const double *mass_of_type, double *x, double *v,
            double *f, orc_result *r);
int64_t orc_nrebuilds(const orc_ctx *c);

/* Lists as (tag_i, tag_j, image) triples, image = sum_c ((s_c+8)&15) << (4c).
 * Full list: all j within cut_force+skin of owned i (npair_full_bin_ghost.cpp:105).
 * ILP intralayer list: ILP_neigh (pair_ilp_graphene_hbn.cpp:732).  Returns counts;
 * the caller passes buffers of capacity cap (triples) or NULL to query. */
int64_t orc_full_list(orc_ctx *c, int64_t *out, int64_t cap);
int64_t orc_ilp_list(orc_ctx *c, int64_t *out, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
