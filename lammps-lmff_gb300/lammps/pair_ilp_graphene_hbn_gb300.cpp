/* ----------------------------------------------------------------------
   ilp/graphene/hbn/gb300 -- see pair_ilp_graphene_hbn_gb300.h
------------------------------------------------------------------------- */

#include "pair_ilp_graphene_hbn_gb300.h"

#include <cstring>

#include "atom.h"
#include "error.h"
#include "force.h"
#include "neighbor.h"

using namespace LAMMPS_NS;

PairILPGrapheneHBNGB300::PairILPGrapheneHBNGB300(LAMMPS *lmp) : PairILPGrapheneHBN(lmp)
{
  // exact per-style virial from the engine; no fdotr over ghosts (see tersoff/gb300)
  no_virial_fdotr_compute = 1;
}

/* ----------------------------------------------------------------------
   checks of PairILPGrapheneHBN::init_style (pair_ilp_graphene_hbn.cpp:393-398);
   no neighbour request and no intralayer pages (the engine builds its own lists)
------------------------------------------------------------------------- */

void PairILPGrapheneHBNGB300::init_style()
{
  if (force->newton_pair == 0)
    error->all(FLERR,"Pair style ilp/graphene/hbn requires newton pair on");
  if (!atom->molecule_flag)
    error->all(FLERR,"Pair style ilp/graphene/hbn requires atom attribute molecule");
  gb300::setup(lmp,this,this,1,"ilp/graphene/hbn/gb300");
}

/* ----------------------------------------------------------------------
   the parameters after coeff(): Param[] as read, elem2param[ne^2], the intralayer
   cutoffs, type -> element, cut_global and tap_flag
------------------------------------------------------------------------- */

void PairILPGrapheneHBNGB300::fill_params(lmff_lammps::StyleParams &sp)
{
  sp.ntypes = atom->ntypes;
  sp.skin = neighbor->skin;
  sp.interlayer = true;
  sp.model = LMFF_INTERLAYER_ILP;
  sp.ilp_params.resize(nparams);
  lmff_ilp_param *dst = sp.ilp_params.data();
  for (int m = 0; m < nparams; m++) {
    const Param &q = params[m];
    lmff_ilp_param &o = dst[m];
    memset(&o,0,sizeof(o));
    o.z0 = q.z0; o.alpha = q.alpha; o.epsilon = q.epsilon; o.C = q.C; o.delta = q.delta;
    o.d = q.d; o.sR = q.sR; o.reff = q.reff; o.C6 = q.C6; o.S = q.S;
    o.delta2inv = q.delta2inv; o.seff = q.seff; o.lambda = q.lambda; o.rcut = q.rcut;
    o.ielement = q.ielement; o.jelement = q.jelement;
  }
  int ne = nelements;
  sp.i_nelements = ne;
  sp.i_elem2param.resize(ne*ne);
  sp.i_cutsq.resize(ne*ne);
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < ne; j++) {
      sp.i_elem2param[i*ne+j] = elem2param[i][j];
      sp.i_cutsq[i*ne+j] = cutILPsq[i][j];
    }
  sp.i_map.resize(atom->ntypes+1);
  for (int t = 0; t <= atom->ntypes; t++) sp.i_map[t] = t ? map[t] : -1;
  sp.cut_global = cut_global;
  sp.tap_flag = tap_flag;
}

/* ----------------------------------------------------------------------
   PairILPGrapheneHBN::compute replaced by one engine evaluation (shared with tersoff/gb300
   under hybrid/overlay)
------------------------------------------------------------------------- */

void PairILPGrapheneHBNGB300::compute(int eflag, int vflag)
{
  ev_init(eflag,vflag);
  pvector[0] = pvector[1] = 0.0;
  lmff_lammps::StyleOut out;
  gb300::compute(lmp,this,this,1,eflag,vflag,eflag_atom,vflag_atom,"ilp/graphene/hbn/gb300",out);
  if (eflag_global) eng_vdwl += out.eng_vdwl;
  if (vflag_global)
    for (int k = 0; k < 6; k++) virial[k] += out.virial[k];
  pvector[0] = out.pvector[0];
  pvector[1] = out.pvector[1];
}
