/* ----------------------------------------------------------------------
   tersoff/gb300 -- see pair_tersoff_gb300.h
------------------------------------------------------------------------- */

#include "pair_tersoff_gb300.h"

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

PairTersoffGB300::PairTersoffGB300(LAMMPS *lmp) : PairTersoff(lmp)
{
  // the engine returns each style's exact global virial; ghost forces stay zero, so
  // a hybrid fdotr sum over owned+ghost atoms would be wrong (pair_hybrid.cpp:97-102)
  no_virial_fdotr_compute = 1;
}

/* ----------------------------------------------------------------------
   same checks as PairTersoff::init_style (pair_tersoff.cpp:365-377), no neighbour
   request (the engine builds its own lists), then the engine from the parameters
------------------------------------------------------------------------- */

void PairTersoffGB300::init_style()
{
  if (atom->tag_enable == 0)
    error->all(FLERR,"Pair style Tersoff requires atom IDs");
  if (force->newton_pair == 0)
    error->all(FLERR,"Pair style Tersoff requires newton pair on");

  std::vector<lmff_tersoff_param> tp(nparams);
  for (int m = 0; m < nparams; m++) {
    const Param &q = params[m];
    lmff_tersoff_param &o = tp[m];
    memset(&o,0,sizeof(o));
    o.lam1 = q.lam1; o.lam2 = q.lam2; o.lam3 = q.lam3;
    o.c = q.c; o.d = q.d; o.h = q.h; o.gamma = q.gamma; o.powerm = q.powerm;
    o.powern = q.powern; o.beta = q.beta; o.biga = q.biga; o.bigb = q.bigb;
    o.bigd = q.bigd; o.bigr = q.bigr; o.cut = q.cut; o.cutsq = q.cutsq;
    o.c1 = q.c1; o.c2 = q.c2; o.c3 = q.c3; o.c4 = q.c4;
    o.ielement = q.ielement; o.jelement = q.jelement; o.kelement = q.kelement;
    o.powermint = q.powermint;
  }
  int ne = nelements;
  std::vector<int> e2p(ne*ne*ne);
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < ne; j++)
      for (int k = 0; k < ne; k++) e2p[(i*ne+j)*ne+k] = elem2param[i][j][k];
  std::vector<int> tmap(atom->ntypes+1);
  for (int t = 0; t <= atom->ntypes; t++) tmap[t] = t ? map[t] : -1;

  lmff_params p;
  memset(&p,0,sizeof(p));
  p.ntypes = atom->ntypes;
  p.tersoff_nelements = ne;
  p.tersoff_nparams = nparams;
  p.tersoff_params = tp.data();
  p.tersoff_elem2param = e2p.data();
  p.tersoff_map = tmap.data();
  p.tersoff_cutmax = cutmax;
  p.skin = neighbor->skin;
  std::string err;
  if (gb.create(p,lmff_lammps::device_from_env(),lmff_lammps::precision_from_env(),err) != LMFF_OK)
    error->all(FLERR,(std::string("tersoff/gb300: ") + err).c_str());
}

/* ----------------------------------------------------------------------
   PairTersoff::compute replaced by one engine evaluation of the periodic system
------------------------------------------------------------------------- */

void PairTersoffGB300::compute(int eflag, int vflag)
{
  ev_init(eflag,vflag);
  if (comm->nprocs > 1)
    error->all(FLERR,"Pair style tersoff/gb300 evaluates the whole periodic system on one GPU: "
               "run it on one MPI rank");
  if (domain->triclinic)
    error->all(FLERR,"Pair style tersoff/gb300 requires an orthogonal box");
  if (vflag_atom)
    error->all(FLERR,"Pair style tersoff/gb300 does not compute per-atom virials");

  int nlocal = atom->nlocal;
  int periodic[3] = {domain->xperiodic, domain->yperiodic, domain->zperiodic};
  const bool big = sizeof(tagint) == 8;
  lmff_lammps::StyleOut out;
  std::string err;
  int rc = gb.compute(LMFF_TERSOFF, nlocal, nlocal ? &atom->x[0][0] : NULL, atom->type,
                      NULL, NULL,
                      big ? NULL : (const int32_t *) atom->tag, big ? (const int64_t *) atom->tag : NULL,
                      neighbor->ago == 0, domain->boxlo, domain->boxhi, periodic,
                      nlocal ? &atom->f[0][0] : NULL, eflag_atom ? eatom : NULL,
                      eflag, vflag, out, err);
  if (rc != LMFF_OK) error->one(FLERR,(std::string("tersoff/gb300: ") + err).c_str());
  if (eflag_global) eng_vdwl += out.eng_vdwl;
  if (vflag_global)
    for (int k = 0; k < 6; k++) virial[k] += out.virial[k];
}
