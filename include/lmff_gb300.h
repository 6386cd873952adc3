/*
 * lmff_gb300 -- GB300 (sm_103a) force engine for the layered-materials path of
 * LAMMPS-LMFF: Tersoff intralayer three-body forces + the ILP interlayer potential
 * (per-atom normals and their derivatives) + the neighbour build that feeds both.
 *
 * C ABI: plain pointers and sizes, no C++ or CUDA types.  One engine handle drives one
 * GPU through one CUDA stream; calls on one handle are not reentrant.  Every call returns
 * with its GPU work finished.  Engines on one device share that device's constant
 * memory for the potential tables: the library serialises calls per device and reloads
 * the tables whenever another engine ran in between, so several engines (for example
 * one per LAMMPS sub-style) may be used from one or several host threads.
 *
 * What each entry point replaces in the reference (paths relative to the reference
 * snapshot's source trees):
 *   lmff_create / lmff_create_from_files
 *       PairTersoff::coeff + read_file + setup_params (MANYBODY/pair_tersoff.cpp:293-580)
 *       PairILPGrapheneHBN::settings + coeff + read_file + init_one
 *       (USER-MISC/pair_ilp_graphene_hbn.cpp:132-240, :246-387)
 *   lmff_set_box           Domain box + periodicity consumed by the neighbour build
 *                          (neighbor.cpp:240-317, nbin_standard.cpp:53-192)
 *   lmff_compute           PairHybrid::compute over {tersoff, ilp/graphene/hbn}
 *                          (pair_hybrid.cpp:93-137) = PairTersoff::compute
 *                          (pair_tersoff.cpp:86-265) + PairILPGrapheneHBN::compute
 *                          (pair_ilp_graphene_hbn.cpp:428-443: ILP_neigh, calc_normal,
 *                          calc_FvdW, calc_FRep) + the neighbour build
 *                          (npair_full_bin_ghost.cpp:36-140) + virial_fdotr_compute
 *                          (pair.cpp:1554) + per-atom energy tallies (pair.cpp:913,1060)
 *   lmff_compute_vatom     the per-atom virial tallies of both styles (Pair::vatom:
 *                          pair.cpp ev_tally :913, ev_tally_xyz :1060, v_tally3 :1435)
 *   lmff_upload / lmff_run_nve / lmff_download
 *                          Verlet::run (verlet.cpp:220-339) with FixNVE
 *                          (fix_nve.cpp:64-111) and Neighbor::decide / check_distance
 *                          (neighbor.cpp:1947-1976), device resident
 *   lmff_minimize          Min::setup/run/cleanup with MinCG::iterate and
 *                          MinLineSearch::linemin_quadratic (min.cpp, min_cg.cpp,
 *                          min_linesearch.cpp), device resident
 *   lmff_batch_*           no counterpart: many independent systems per launch
 *   lmff_server_*          no counterpart: a request queue served by continuous batching
 *   lmff_last_error        error->one / error->all messages of both pair styles
 */
#ifndef LMFF_GB300_H
#define LMFF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (0 = success) ------------------------------------------------ */
#define LMFF_OK 0
#define LMFF_EINVAL (-1)              /* bad argument */
#define LMFF_ECUDA (-2)               /* CUDA runtime error (message in lmff_last_error) */
#define LMFF_EOVERFLOW (-3)           /* a neighbour list outgrew its capacity */
#define LMFF_ETOO_MANY_ILP_NEIGH (-4) /* > 3 intralayer neighbours (pair_ilp_graphene_hbn.cpp:739) */
#define LMFF_EZERO_NORMAL (-5)        /* zero normal (pair_ilp_graphene_hbn.cpp:887,1030) */
#define LMFF_EBADPARAM (-6)           /* potential file / parameter error */
#define LMFF_ETIMEDOUT (-7)           /* a bounded device wait gave up */
#define LMFF_EUNSUPPORTED (-8)        /* request outside what the engine implements */
#define LMFF_ENOMEM (-9)              /* device or host allocation failed */
#define LMFF_ENODEV (-10)             /* no usable CUDA device */
#define LMFF_PENDING 1                /* lmff_server_wait: the request has not finished yet */

/* ---- precision modes ------------------------------------------------------------ */
#define LMFF_FP64 0   /* all-FP64 drop-in */
#define LMFF_MIXED 1  /* FP32 pair / three-body arithmetic on FP64 displacements;
                         FP64 integration, per-atom accumulation, reductions and
                         normal-derivative assembly */

/* ---- compute flags (the `which` argument) ----------------------------------------- */
#define LMFF_TERSOFF 1     /* evaluate pair_style tersoff */
#define LMFF_ILP 2         /* evaluate pair_style ilp/graphene/hbn */
#define LMFF_SAME_ATOMS 4  /* caller promises type/mol/tag unchanged since the last call
                              (LAMMPS: no reneighbouring this step); skips their upload */
#define LMFF_OVERWRITE 8   /* store forces / per-atom energies instead of adding to them */

typedef struct lmff_engine lmff_engine;

/* One Tersoff entry; same fields and meaning as PairTersoff::Param
 * (pair_tersoff.h:38-53), derived values (cut, cutsq, c1..c4) filled as setup_params
 * does (pair_tersoff.cpp:565-573). */
typedef struct lmff_tersoff_param {
  double lam1, lam2, lam3, c, d, h, gamma, powerm, powern, beta;
  double biga, bigb, bigd, bigr, cut, cutsq, c1, c2, c3, c4;
  int ielement, jelement, kelement, powermint;
} lmff_tersoff_param;

/* One ILP entry; PairILPGrapheneHBN::Param (pair_ilp_graphene_hbn.h:53-57) after
 * read_file's unit scaling and derived values (pair_ilp_graphene_hbn.cpp:354-364). */
typedef struct lmff_ilp_param {
  double z0, alpha, epsilon, C, delta, d, sR, reff, C6, S;
  double delta2inv, seff, lambda, rcut;
  int ielement, jelement;
} lmff_ilp_param;

/* kolmogorov/crespi/full Param after read_file (pair_kolmogorov_crespi_full.h, :340-365):
 * energies C0 C2 C4 C A already in eV (file meV x 1e-3 x S). */
typedef struct lmff_kc_param {
  double z0, C0, C2, C4, C, delta, lambda, A, S, rcut;
  double delta2inv, z06;
  int ielement, jelement;
} lmff_kc_param;

/* interlayer style held in the ilp_* fields of lmff_params */
#define LMFF_INTERLAYER_ILP 0   /* ilp/graphene/hbn */
#define LMFF_INTERLAYER_KC 1    /* kolmogorov/crespi/full */

/* Everything the two pair styles hold after coeff().  Arrays are copied. */
typedef struct lmff_params {
  int ntypes;                                 /* LAMMPS atom types 1..ntypes (<= 16) */
  /* tersoff; tersoff_nparams == 0 disables the style */
  int tersoff_nelements, tersoff_nparams;
  const lmff_tersoff_param *tersoff_params;
  const int *tersoff_elem2param;              /* [ne*ne*ne], (i*ne+j)*ne+k */
  const int *tersoff_map;                     /* [ntypes+1], entry 0 unused, -1 = NULL */
  double tersoff_cutmax;
  /* ilp/graphene/hbn; ilp_nparams == 0 disables the style */
  int ilp_nelements, ilp_nparams;
  const lmff_ilp_param *ilp_params;
  const int *ilp_elem2param;                  /* [ne*ne] */
  const int *ilp_map;                         /* [ntypes+1] */
  const double *ilp_cutILPsq;                 /* [ne*ne] */
  double ilp_cut_global;                      /* pair_style ... ilp/graphene/hbn <cut> */
  int ilp_tap_flag;                           /* pair_style ... <tap_flag> */
  double skin;                                /* neighbor <skin> bin */
  /* LMFF_INTERLAYER_KC: the interlayer style is kolmogorov/crespi/full; ilp_nparams,
   * ilp_nelements, ilp_elem2param, ilp_map, ilp_cutILPsq (its cutKCsq), cut_global
   * and tap_flag describe it, and kc_params replaces ilp_params */
  int interlayer_model;
  const lmff_kc_param *kc_params;
} lmff_params;

/* Energies and virials of one evaluation.  The virial is the global fdotr virial
 * (xx, yy, zz, xy, xz, yz) of each style; pvector as PairILPGrapheneHBN (vdW, rep). */
typedef struct lmff_result {
  double e_tersoff, e_ilp;
  double pvector[2];
  double virial_tersoff[6], virial_ilp[6];
} lmff_result;

/* Per-step thermo sample of the device-resident NVE loop. */
typedef struct lmff_thermo {
  int64_t step;
  double pe, ke, etotal, temp;
  double virial[6];
} lmff_thermo;

typedef struct lmff_stats {
  int64_t natoms, list_entries, short_entries, list_capacity, rebuilds, steps;
  double list_per_atom, bytes_device;   /* bytes_device: device memory this engine holds */
  double ms_last_build, ms_last_forces;
  int precision, tpa, block;
  /* device time of the last lmff_run_nve (CUDA events on the engine's stream) */
  double ms_last_run;
  /* with option "kernel_timing" = 1: summed device time and launch count per kernel
   * since the last "reset_timing": [0] pair (ILP) kernel, [1] Tersoff, [2] intralayer
   * lists and normals, [3] gather, [4] integrator, [5] neighbour build (one per
   * rebuild), [6] normal-derivative assembly */
  double kernel_ms[7];
  int64_t kernel_launches[7];
  /* interlayer pairs within the ILP cutoff in the current configuration (option
   * "count_pairs" = 1 counts them once, outside any timed region) */
  int64_t pairs_in_cutoff;
  /* steps lmff_run_nve ran through the step graph (see option "graphs"), and chunks
   * redone host-driven after a graph's rebuild outgrew the captured list capacity */
  int64_t graph_steps, graph_redos;
  /* device bytes per atom a batch of the current kind needs (per-atom arrays, the pair
   * list at the current density with headroom, sort workspace): admission estimates */
  double bytes_per_atom_need;
} lmff_stats;

/* ---- lifecycle ------------------------------------------------------------------- */
int lmff_device_count(void);
int lmff_create(lmff_engine **out, const lmff_params *p, int device);
/* Parses the potential files as the reference does (17-word Tersoff entries,
 * 13-word ILP entries, '#' comments, continuation lines, element filtering,
 * duplicate / missing entry errors).  elements[t-1] names the element of type t or
 * "NULL"; either file may be NULL to disable that style. */
int lmff_create_from_files(lmff_engine **out, const char *tersoff_file, const char *ilp_file,
                           int ntypes, const char *const *elements, double cut_global,
                           int tap_flag, double skin, int device);
/* Same with one element list per style, as two pair_coeff lines give them, e.g.
 * `pair_coeff * * tersoff C.opt.tersoff NULL C(O) ...` next to
 * `pair_coeff * * ilp/graphene/hbn BNCH.ILP C C ...`. */
int lmff_create_from_files2(lmff_engine **out, const char *tersoff_file,
                            const char *const *tersoff_elements, const char *ilp_file,
                            const char *const *ilp_elements, int ntypes, double cut_global,
                            int tap_flag, double skin, int device);
/* Tersoff + kolmogorov/crespi/full (12-word entries: elem1 elem2 z0 C0 C2 C4 C delta
 * lambda A S rcut) as the interlayer style, read as the reference's read_file does
 * (pair_kolmogorov_crespi_full.cpp:247-392).  Results report it in the e_ilp,
 * virial_ilp and pvector (vdW, repulsion) fields; without the taper the repulsion
 * energy carries the reference's offset -A (z0/cut)^6 per directed pair (init_one,
 * pair_modify shift yes). */
int lmff_create_kc_from_files(lmff_engine **out, const char *tersoff_file,
                              const char *const *tersoff_elements, const char *kc_file,
                              const char *const *kc_elements, int ntypes, double cut_global,
                              int tap_flag, double skin, int device);
void lmff_destroy(lmff_engine *e);

/* ---- configuration ---------------------------------------------------------------- */
int lmff_set_precision(lmff_engine *e, int mode);
/* Box lo/hi and LAMMPS's tilt factors xy, xz, yz (domain.cpp: the edges (hi-lo)_x,
 * (xy, (hi-lo)_y, 0), (xz, yz, (hi-lo)_z)); periodic[d] != 0 marks periodic dims.
 * A triclinic box (any tilt non-zero) is evaluated by lmff_compute and
 * lmff_compute_vatom only: the engine wraps the atoms into the box by whole lattice
 * vectors, adds the periodic images within the neighbour cutoff of it as ghosts (the
 * atoms a LAMMPS rank would hold, comm_brick.cpp borders) and evaluates them in the
 * subdomain form of lmff_compute_ghost, folding the images' shares into their owners;
 * LMFF_SAME_ATOMS has no effect there.  The resident, batch, device and subdomain
 * calls return LMFF_EUNSUPPORTED / LMFF_EINVAL on a triclinic box. */
int lmff_set_box(lmff_engine *e, const double lo[3], const double hi[3], double xy, double xz,
                 double yz, const int periodic[3]);
/* Tunables: "tpa" threads per atom in the ILP kernel (4,8,16,32), "block" threads per
 * block, "list_full" 1 = keep same-molecule pairs in the pair list (the reference's
 * full list, for set comparisons), "skin" neighbour skin in Angstrom,
 * "kernel_timing" 1 = record per-kernel device time, "reset_timing" clears it,
 * "count_pairs" counts interlayer pairs within the cutoff now (see lmff_stats),
 * "graphs" 1 (default) = lmff_run_nve replays steps between thermo samples as one CUDA
 * graph per step (integrate, displacement test, conditional list rebuild, forces,
 * integrate) with no host synchronisation; 0 = one host-driven step at a time.
 * Per-kernel timing uses the host-driven loop, and so does every engine created while
 * the environment variable LMFF_GB300_GRAPHS is "0" (profilers cannot look inside a
 * graph that has conditional nodes).  "graph_list_cap" > 0 lowers the
 * pair-list capacity a graph's rebuild may fill (testing the overflow redo: a chunk
 * whose rebuild overflows is redone host-driven from its first step, rebuilding the
 * list there, so it equals the uninterrupted run up to summation order).
 * "ters_concurrent" 1 (default) = the Tersoff kernel runs on a second stream beside
 * the interlayer pair kernel (they write disjoint arrays; joined before the gather);
 * 0 = one after the other.  "pair_tile" 2 (default) = the mixed force-only pair kernel
 * takes two list entries per lane and iteration (FP32x2 lanes across the pair), 1 = one
 * entry (the neighbour-tile shape the tuner chooses).  "small_variants" 1 (default) = small
 * systems run the kernel variants made for them (one warp per atom in the list build, 16
 * or 4 lanes per atom in the intralayer lists, 8 in the gather, one lane per bond in
 * Tersoff when it runs alone), 0 = the large-system kernels at every size; the lists and
 * results are the same to the bit either way, except Tersoff run alone, which agrees to
 * rounding.  "pdl" = a mask of the step's dependent kernels launched with programmatic
 * dependent launch up to 65,536 atoms (each scheduled before the previous one ends and
 * waiting for it on the device): 1 the pair kernel, 2 the normal-derivative kernel, 4 the
 * gather, 8 the intralayer lists in step graphs, +16 dependents scheduled as each kernel
 * starts; 0 = ordinary launches; default 14.  The results do not depend on it.  "check_every" = how often
 * lmff_run_nve tests the pair list: 1 = every step, for displacement alone (LAMMPS's
 * neigh_modify every 1 delay 0 check yes); k > 1 = at steps whose index is a multiple
 * of k, rebuilding when an atom may move more than skin/2 before the next test (its
 * displacement plus a look-ahead from its velocity and force); a step between tests
 * that finds an atom past skin/2 rebuilds at once (the step graphs redo their chunk on
 * the host-driven loop).  0 (default) = 1 above 65,536 atoms, else the largest of 8, 4,
 * 2 whose look-ahead from the run's starting motion stays within skin/4.  Forces do
 * not depend on when the list is rebuilt, only the order of some sums does. */
int lmff_set_option(lmff_engine *e, const char *key, double value);

/* ---- one-shot evaluation on host buffers (the pair-style drop-in) ------------------ */
/* x[natoms*3] positions; type[natoms] 1..ntypes; mol[natoms] molecule ids; tag[natoms]
 * atom ids (NULL: 1..natoms).  which = LMFF_TERSOFF | LMFF_ILP.  f[natoms*3] is
 * accumulated (+=); eatom[natoms] accumulated if not NULL.  res may be NULL. */
int lmff_compute(lmff_engine *e, int natoms, const double *x, const int *type, const int64_t *mol,
                 const int64_t *tag, int which, int eflag, int vflag, double *f, double *eatom,
                 lmff_result *res);

/* Subdomain form of lmff_compute for a LAMMPS rank of a domain decomposition: what
 * PairTersoff::compute (pair_tersoff.cpp:86-265) and PairILPGrapheneHBN::compute
 * (pair_ilp_graphene_hbn.cpp:428-675) do on the owned atoms [0, nlocal) and the ghost
 * atoms [nlocal, nall) of the full+ghost list (npair_full_bin_ghost.cpp:36-140), with
 * newton on.  x[nall*3], type, mol, tag[nall] (tags required: a ghost carries its
 * owner's tag).  The engine bins all nall atoms in a non-periodic box of its own (the
 * ghosts carry the periodic images; lmff_set_box is not used).  Evaluated: two-body
 * terms whose end kept by the tag-parity half of the full list is owned (equal tags:
 * the coordinate tie-break of pair_tersoff.cpp:150-158), ILP repulsion terms and
 * Tersoff bond-order terms whose centre is owned.  f[nall*3] and eatom[nall] receive
 * every atom's share, ghosts included, for LAMMPS's reverse communication to fold
 * (verlet.cpp:307-332, Comm::reverse_comm); energies and virials in res are those of
 * the evaluated interactions, equal to the fdotr virial over nall.  which may add
 * LMFF_SAME_ATOMS when the atoms (order, identity, nlocal) are those of the previous
 * call; OVERWRITE as in lmff_compute.  The engine stays in this mode until
 * lmff_set_box; until then the periodic-system calls return LMFF_EINVAL. */
int lmff_compute_ghost(lmff_engine *e, int nlocal, int nall, const double *x, const int *type,
                       const int64_t *mol, const int64_t *tag, int which, int eflag, int vflag,
                       double *f, double *eatom, lmff_result *res);

/* Per-atom virial of the evaluation that the previous call on this engine made
 * (lmff_compute, lmff_compute_ghost, lmff_compute_device or lmff_compute_resident; a
 * second lmff_compute_vatom for the other style may follow; after any other call of
 * the engine that uses the device it returns LMFF_EINVAL): Pair::vatom of
 * PairTersoff::compute (pair_tersoff.cpp:173, :223, :253) and of PairILPGrapheneHBN /
 * PairKolmogorovCrespiFull::compute (pair_ilp_graphene_hbn.cpp:536, :667, :671), split
 * over atoms as their ev_tally, ev_tally_xyz and v_tally3 calls split it (pair.cpp).
 * which = LMFF_TERSOFF and/or LMFF_ILP selects the styles (each sub-style of
 * hybrid/overlay has its own vatom); LMFF_OVERWRITE overwrites instead of accumulating.
 * vatom[natoms*6] in the evaluated call's atom order, rows xx yy zz xy xz yz (LAMMPS
 * order, energy units, not divided by a volume); natoms = that call's natoms (nall in
 * subdomain mode, where ghost rows carry the shares LAMMPS's reverse communication
 * folds into their owners).  A separate pass on the evaluated positions: Tersoff's
 * shares in FP64, the interlayer shares in the evaluation's precision (LMFF_MIXED: FP32
 * pair terms, FP64 sums); not for batches (LMFF_EUNSUPPORTED). */
int lmff_compute_vatom(lmff_engine *e, int which, int natoms, double *vatom);

/* Same on device pointers (d_x[natoms*3] double, d_type int32, d_mol int64, d_tag int64
 * or NULL, d_f double accumulated), ordered on the engine's stream. */
int lmff_compute_device(lmff_engine *e, int natoms, const double *d_x, const int *d_type,
                        const int64_t *d_mol, const int64_t *d_tag, int which, int eflag,
                        int vflag, double *d_f, lmff_result *res);

/* Allocation-free variant of lmff_compute_device for one small system.  No counterpart
 * in the reference: it exists for callers that must not allocate device memory once
 * they run -- an application that hands all GPU memory to its own pool at start-up,
 * or code on a path where cudaMalloc would synchronise the device or is not allowed.
 * The caller passes device inputs (d_x[natoms*3], d_type, d_mol, all required) and the
 * output d_f[natoms*3], which is overwritten; energies and virials go to res.  Nothing
 * is allocated: every buffer the kernels need (sorted atoms, bins, neighbour lists,
 * normals, force slots, reductions, sort workspace) lives in one 16 MiB static device
 * array that every GPU loading this library holds until the process exits.  Limits:
 * natoms <= 2048 (natoms = 0, an empty subdomain, returns LMFF_OK with zero energies
 * and virials, as lmff_compute_device does), at most 8192 neighbour bins, a box whose
 * periodic images leave the 32-bit list code room for natoms, and the pair list must fit the space
 * left in the array (about 1,600 entries per atom at 2048 atoms); larger requests are
 * rejected with LMFF_EINVAL or LMFF_EOVERFLOW and a message, never truncated.  The
 * engine handle supplies parameters, box, precision and stream.  The first call on a
 * device looks the array's device address up (cudaGetSymbolAddress), so make that
 * first call before capturing any stream.  All calls share the one array and it keeps
 * the previous call's contents: calls that can overlap on the GPU (several streams,
 * threads or handles) race and must be serialised by the caller. */
int lmff_compute_device_noalloc(lmff_engine *e, int natoms, const double *d_x, const int *d_type,
                                const int64_t *d_mol, int which, int eflag, int vflag, double *d_f,
                                lmff_result *res);

/* ---- device-resident system (standalone MD) ---------------------------------------- */
/* mass[t-1] is the mass of type t (amu); v may be NULL (zero). */
int lmff_upload(lmff_engine *e, int natoms, const double *x, const double *v, const int *type,
                const int64_t *mol, const int64_t *tag, const double *mass);
int lmff_compute_resident(lmff_engine *e, int which, int eflag, int vflag, lmff_result *res);
/* nsteps of velocity Verlet (metal units, dt in ps); a thermo sample every
 * thermo_every steps (0: none) into thermo[nsteps/thermo_every + 1] (may be NULL). */
int lmff_run_nve(lmff_engine *e, int nsteps, double dt, int thermo_every, lmff_thermo *thermo);
/* Copies back in the upload order; any pointer may be NULL. */
int lmff_download(lmff_engine *e, double *x, double *v, double *f);

/* Energy minimisation of the resident system: LAMMPS `minimize etol ftol maxiter
 * maxeval` with the default min_style cg (Polak-Ribiere, min_cg.cpp) and quadratic
 * line search (min_linesearch.cpp linemin_quadratic), min_modify dmax (0.1 A in the
 * reference) and norm two.  frozen[natoms] (upload order, may be NULL): nonzero atoms
 * keep zero force, as `fix setforce 0.0 0.0 0.0` on them does.  Positions and forces
 * stay resident (lmff_download).  stop_condition follows min.h: 0 max iterations,
 * 1 max evaluations, 2 energy tolerance, 3 force tolerance, 4 search direction not
 * downhill, 5 linesearch alpha is zero, 6 forces are zero, 7 quadratic factors are zero. */
typedef struct lmff_min_result {
  int niter, neval, stop_condition;
  double einitial, efinal, fnorm2_init, fnorminf_init, fnorm2_final, fnorminf_final, alpha_final;
} lmff_min_result;
int lmff_minimize(lmff_engine *e, double etol, double ftol, int maxiter, int maxeval, double dmax,
                  const int *frozen, lmff_min_result *out);

/* ---- batched independent systems --------------------------------------------------- */
/* A batch holds many independent periodic systems in one flattened device layout and
 * evaluates them in one launch per kernel.  Box per system: lo[3], hi[3], periodic[3]. */
typedef struct lmff_system_desc {
  int natoms;
  const double *x;          /* [natoms*3] */
  const int *type;
  const int64_t *mol;
  double lo[3], hi[3];
  int periodic[3];
  const double *v;          /* [natoms*3] velocities for lmff_run_nve on the batch, or NULL (zero) */
} lmff_system_desc;
/* Makes the batch the engine's resident state: lmff_batch_compute evaluates it,
 * lmff_run_nve integrates every system at once (masses from lmff_set_masses or
 * lmff_upload), lmff_download returns the batch in order.  Atoms of a system are
 * never neighbours of another system's atoms, and each system's forces, energies and
 * virial are bitwise the ones it gets alone. */
int lmff_batch_set(lmff_engine *e, int nsys, const lmff_system_desc *sys);
/* Energies/forces/virials of every system: f_out[sum natoms * 3] in batch order
 * (overwritten), res[nsys]. */
int lmff_batch_compute(lmff_engine *e, double *f_out, lmff_result *res);
/* Per-system energies and virials of the last evaluation that computed them (a
 * lmff_batch_compute, lmff_compute_resident, or a thermo step of lmff_run_nve). */
int lmff_batch_results(lmff_engine *e, int nsys, lmff_result *res);
/* mass[t-1] = mass of type t (amu), used by batches loaded afterwards. */
int lmff_set_masses(lmff_engine *e, int ntypes, const double *mass);
/* A new engine on the same device with the same parameters, precision and tunables
 * (no resident state).  Engines with equal parameters share device constant tables. */
int lmff_clone(const lmff_engine *src, lmff_engine **out);

/* ---- serving: independent requests, continuously batched --------------------------- */
/* No counterpart in the reference (one simulation per process).  A server owns two
 * worker threads, each with an engine cloned from `proto` (parameters, precision,
 * tunables, masses) on its own stream, so both run on the device at once.  Submission
 * is thread-safe and returns at once; requests are admitted in FIFO order while the
 * estimated device bytes of admitted requests stay within hbm_budget_bytes.  One worker
 * evaluates the admitted single points together in one batched launch per kernel; the
 * other advances the admitted NVE requests of equal dt as one resident batch,
 * md_chunk_steps at a time, re-forming it when requests join or leave.  A single
 * point is bitwise the same alone and in any mix; an NVE run in a batch shares the
 * batch's list rebuilds, so it matches the run alone up to summation order.  A failing
 * batch is retried request by request, so an error reaches only its own request. */
typedef struct lmff_request {
  int natoms;
  const double *x;          /* [natoms*3], copied at submission */
  const double *v;          /* [natoms*3] or NULL (zero); NVE only */
  const int *type;          /* [natoms] 1..ntypes */
  const int64_t *mol;       /* [natoms] or NULL (all 0) */
  double lo[3], hi[3];
  int periodic[3];
  int nsteps;               /* 0: single point; > 0: NVE steps */
  double dt;                /* ps, NVE only */
  /* caller-owned outputs, written before the request completes (any may be NULL):
   * forces / energies / virial of the final configuration, final x and v (NVE) */
  double *f_out;
  double *x_out, *v_out;
  lmff_result *res;
} lmff_request;

typedef struct lmff_server_config {
  double hbm_budget_bytes;  /* admission budget (0: 64e9) */
  double bytes_per_atom;    /* starting device-bytes estimate per atom (0: 4096); raised
                             * to what the engines report once batches have run */
  int64_t max_batch_atoms;  /* atoms per batched launch (0: 8M) */
  int md_chunk_steps;       /* NVE steps between batch re-formations (0: 20) */
} lmff_server_config;

typedef struct lmff_server_stats {
  int64_t submitted, completed, failed, queued, active;
  int64_t point_batches, point_systems, md_chunks, md_reforms, md_steps;
  double admitted_bytes, bytes_per_atom;
  double busy_s;              /* busy time summed over the two workers */
  double max_admitted_bytes;  /* high-water mark of admitted_bytes */
} lmff_server_stats;

typedef struct lmff_server lmff_server;
int lmff_server_create(lmff_server **out, const lmff_engine *proto, const lmff_server_config *cfg);
/* Copies the inputs; *ticket identifies the request.  LMFF_ENOMEM if the request alone
 * exceeds the budget. */
int lmff_server_submit(lmff_server *s, const lmff_request *req, int64_t *ticket);
/* Submits reqs[0..nreq) atomically (all queued together, tickets[nreq]); nothing is
 * queued if any request is invalid or alone exceeds the budget. */
int lmff_server_submit_many(lmff_server *s, int nreq, const lmff_request *reqs, int64_t *tickets);
/* Waits up to timeout_s (< 0: forever).  Returns LMFF_PENDING if still running, else
 * the request's status (its message in lmff_server_last_error) and retires the ticket;
 * latency_s = completion - submission time. */
int lmff_server_wait(lmff_server *s, int64_t ticket, double timeout_s, double *latency_s);
int lmff_server_get_stats(lmff_server *s, lmff_server_stats *out);
/* Message of this thread's last failed submit or wait. */
const char *lmff_server_last_error(void);
/* Finishes every submitted request, then stops the worker and frees the engines. */
void lmff_server_destroy(lmff_server *s);

/* ---- diagnostics ------------------------------------------------------------------- */
int lmff_get_stats(lmff_engine *e, lmff_stats *out);
/* Neighbour lists of the last build as (tag_i, tag_j, image) triples with
 * image = sum_d ((s_d + 8) & 15) << (4 d): which = 0 pair list, 1 ILP intralayer list
 * (current step).  Returns the entry count; out may be NULL to query. */
int64_t lmff_export_list(lmff_engine *e, int which, int64_t *out, int64_t cap);
const char *lmff_last_error(const lmff_engine *e);
const char *lmff_strerror(int code);

#ifdef __cplusplus
}
#endif
#endif
