/* ----------------------------------------------------------------------
   tersoff/gb300 -- see pair_tersoff_gb300.h
------------------------------------------------------------------------- */

#include "pair_tersoff_gb300.h"

#include <cstring>

#include "atom.h"
#include "error.h"
#include "force.h"
#include "neighbor.h"

using namespace LAMMPS_NS;

PairTersoffGB300::PairTersoffGB300(LAMMPS *lmp) : PairTersoff(lmp)
{
  // the engine returns each style's exact global virial (in the periodic form ghost
  // forces stay zero), so no fdotr sum over owned+ghost atoms (pair_hybrid.cpp:97-102)
  no_virial_fdotr_compute = 1;
}

/* ----------------------------------------------------------------------
   same checks as PairTersoff::init_style (pair_tersoff.cpp:365-377), no neighbour
   request (the engine builds its own lists), then the engine
------------------------------------------------------------------------- */

void PairTersoffGB300::init_style()
{
  if (atom->tag_enable == 0)
    error->all(FLERR,"Pair style Tersoff requires atom IDs");
  if (force->newton_pair == 0)
    error->all(FLERR,"Pair style Tersoff requires newton pair on");
  gb300::setup(lmp,this,this,0,"tersoff/gb300");
}

/* ----------------------------------------------------------------------
   the parameters after coeff(): Param[] as read, elem2param[ne^3], type -> element
------------------------------------------------------------------------- */

void PairTersoffGB300::fill_params(lmff_lammps::StyleParams &sp)
{
  sp.ntypes = atom->ntypes;
  sp.skin = neighbor->skin;
  sp.tersoff = true;
  sp.t_params.resize(nparams);
  for (int m = 0; m < nparams; m++) {
    const Param &q = params[m];
    lmff_tersoff_param &o = sp.t_params[m];
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
  sp.t_nelements = ne;
  sp.t_elem2param.resize(ne*ne*ne);
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < ne; j++)
      for (int k = 0; k < ne; k++) sp.t_elem2param[(i*ne+j)*ne+k] = elem2param[i][j][k];
  sp.t_map.resize(atom->ntypes+1);
  for (int t = 0; t <= atom->ntypes; t++) sp.t_map[t] = t ? map[t] : -1;
  sp.t_cutmax = cutmax;
}

/* ----------------------------------------------------------------------
   PairTersoff::compute replaced by one engine evaluation (shared with the interlayer
   gb300 style under hybrid/overlay)
------------------------------------------------------------------------- */

void PairTersoffGB300::compute(int eflag, int vflag)
{
  ev_init(eflag,vflag);
  lmff_lammps::StyleOut out;
  gb300::compute(lmp,this,this,0,eflag,vflag,eflag_atom,vflag_atom,"tersoff/gb300",out);
  if (eflag_global) eng_vdwl += out.eng_vdwl;
  if (vflag_global)
    for (int k = 0; k < 6; k++) virial[k] += out.virial[k];
}
