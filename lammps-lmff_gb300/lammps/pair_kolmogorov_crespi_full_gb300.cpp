/* ----------------------------------------------------------------------
   kolmogorov/crespi/full/gb300 -- see pair_kolmogorov_crespi_full_gb300.h
------------------------------------------------------------------------- */

#include "pair_kolmogorov_crespi_full_gb300.h"

#include <cstring>
#include <string>
#include <vector>

#include "atom.h"
#include "comm.h"
#include "domain.h"
#include "error.h"
#include "force.h"
#include "neighbor.h"

using namespace LAMMPS_NS;

PairKolmogorovCrespiFullGB300::PairKolmogorovCrespiFullGB300(LAMMPS *lmp) : PairKolmogorovCrespiFull(lmp)
{
  // exact per-style virial from the engine; no fdotr over ghosts (see tersoff/gb300)
  no_virial_fdotr_compute = 1;
}

/* ----------------------------------------------------------------------
   checks of PairKolmogorovCrespiFull::init_style (pair_kolmogorov_crespi_full.cpp:
   394-399); no neighbour request and no KC pages (the engine builds its own lists)
------------------------------------------------------------------------- */

void PairKolmogorovCrespiFullGB300::init_style()
{
  if (force->newton_pair == 0)
    error->all(FLERR,"Pair style kolmolgorov/crespi/full requires newton pair on");
  if (!atom->molecule_flag)
    error->all(FLERR,"Pair style kolmolgorov/crespi/full requires atom attribute molecule");

  std::vector<lmff_kc_param> kp(nparams);
  for (int m = 0; m < nparams; m++) {
    const Param &q = params[m];
    lmff_kc_param &o = kp[m];
    memset(&o,0,sizeof(o));
    o.z0 = q.z0; o.C0 = q.C0; o.C2 = q.C2; o.C4 = q.C4; o.C = q.C; o.delta = q.delta;
    o.lambda = q.lambda; o.A = q.A; o.S = q.S; o.rcut = q.rcut;
    o.delta2inv = q.delta2inv; o.z06 = q.z06;
    o.ielement = q.ielement; o.jelement = q.jelement;
  }
  int ne = nelements;
  std::vector<int> e2p(ne*ne);
  std::vector<double> cut2(ne*ne);
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < ne; j++) {
      e2p[i*ne+j] = elem2param[i][j];
      cut2[i*ne+j] = cutKCsq[i][j];
    }
  std::vector<int> tmap(atom->ntypes+1);
  for (int t = 0; t <= atom->ntypes; t++) tmap[t] = t ? map[t] : -1;

  lmff_params p;
  memset(&p,0,sizeof(p));
  p.ntypes = atom->ntypes;
  p.ilp_nelements = ne;
  p.ilp_nparams = nparams;
  p.ilp_elem2param = e2p.data();
  p.ilp_map = tmap.data();
  p.ilp_cutILPsq = cut2.data();
  p.ilp_cut_global = cut_global;
  p.ilp_tap_flag = tap_flag;
  p.interlayer_model = LMFF_INTERLAYER_KC;
  p.kc_params = kp.data();
  p.skin = neighbor->skin;
  std::string err;
  if (gb.create(p,lmff_lammps::device_from_env(),lmff_lammps::precision_from_env(),err) != LMFF_OK)
    error->all(FLERR,(std::string("kolmogorov/crespi/full/gb300: ") + err).c_str());
}

/* ----------------------------------------------------------------------
   PairKolmogorovCrespiFull::compute replaced by one engine evaluation
------------------------------------------------------------------------- */

void PairKolmogorovCrespiFullGB300::compute(int eflag, int vflag)
{
  ev_init(eflag,vflag);
  pvector[0] = pvector[1] = 0.0;
  if (comm->nprocs > 1)
    error->all(FLERR,"Pair style kolmogorov/crespi/full/gb300 evaluates the whole periodic system on one GPU: "
               "run it on one MPI rank");
  if (domain->triclinic)
    error->all(FLERR,"Pair style kolmogorov/crespi/full/gb300 requires an orthogonal box");
  if (vflag_atom)
    error->all(FLERR,"Pair style kolmogorov/crespi/full/gb300 does not compute per-atom virials");

  int nlocal = atom->nlocal;
  int periodic[3] = {domain->xperiodic, domain->yperiodic, domain->zperiodic};
  const bool big = sizeof(tagint) == 8;
  lmff_lammps::StyleOut out;
  std::string err;
  int rc = gb.compute(LMFF_ILP, nlocal, nlocal ? &atom->x[0][0] : NULL, atom->type,
                      big ? NULL : (const int32_t *) atom->molecule,
                      big ? (const int64_t *) atom->molecule : NULL,
                      big ? NULL : (const int32_t *) atom->tag, big ? (const int64_t *) atom->tag : NULL,
                      neighbor->ago == 0, domain->boxlo, domain->boxhi, periodic,
                      nlocal ? &atom->f[0][0] : NULL, eflag_atom ? eatom : NULL,
                      eflag, vflag, out, err);
  if (rc != LMFF_OK) error->one(FLERR,(std::string("kolmogorov/crespi/full/gb300: ") + err).c_str());
  if (eflag_global) eng_vdwl += out.eng_vdwl;
  if (vflag_global)
    for (int k = 0; k < 6; k++) virial[k] += out.virial[k];
  pvector[0] = out.pvector[0];
  pvector[1] = out.pvector[1];
}
