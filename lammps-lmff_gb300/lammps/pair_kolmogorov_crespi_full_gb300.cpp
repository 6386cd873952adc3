/* ----------------------------------------------------------------------
   kolmogorov/crespi/full/gb300 -- see pair_kolmogorov_crespi_full_gb300.h
------------------------------------------------------------------------- */

#include "pair_kolmogorov_crespi_full_gb300.h"

#include <cstring>

#include "atom.h"
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
   checks of PairKolmogorovCrespiFull::init_style (pair_kolmogorov_crespi_full.cpp:394-399);
   no neighbour request and no intralayer pages (the engine builds its own lists)
------------------------------------------------------------------------- */

void PairKolmogorovCrespiFullGB300::init_style()
{
  if (force->newton_pair == 0)
    error->all(FLERR,"Pair style kolmolgorov/crespi/full requires newton pair on");
  if (!atom->molecule_flag)
    error->all(FLERR,"Pair style kolmolgorov/crespi/full requires atom attribute molecule");
  gb300::setup(lmp,this,this,1,"kolmogorov/crespi/full/gb300");
}

/* ----------------------------------------------------------------------
   the parameters after coeff(): Param[] as read, elem2param[ne^2], the intralayer
   cutoffs, type -> element, cut_global and tap_flag
------------------------------------------------------------------------- */

void PairKolmogorovCrespiFullGB300::fill_params(lmff_lammps::StyleParams &sp)
{
  sp.ntypes = atom->ntypes;
  sp.skin = neighbor->skin;
  sp.interlayer = true;
  sp.model = LMFF_INTERLAYER_KC;
  sp.kc_params.resize(nparams);
  lmff_kc_param *dst = sp.kc_params.data();
  for (int m = 0; m < nparams; m++) {
    const Param &q = params[m];
    lmff_kc_param &o = dst[m];
    memset(&o,0,sizeof(o));
    o.z0 = q.z0; o.C0 = q.C0; o.C2 = q.C2; o.C4 = q.C4; o.C = q.C; o.delta = q.delta;
    o.lambda = q.lambda; o.A = q.A; o.S = q.S; o.rcut = q.rcut;
    o.delta2inv = q.delta2inv; o.z06 = q.z06;
    o.ielement = q.ielement; o.jelement = q.jelement;
  }
  int ne = nelements;
  sp.i_nelements = ne;
  sp.i_elem2param.resize(ne*ne);
  sp.i_cutsq.resize(ne*ne);
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < ne; j++) {
      sp.i_elem2param[i*ne+j] = elem2param[i][j];
      sp.i_cutsq[i*ne+j] = cutKCsq[i][j];
    }
  sp.i_map.resize(atom->ntypes+1);
  for (int t = 0; t <= atom->ntypes; t++) sp.i_map[t] = t ? map[t] : -1;
  sp.cut_global = cut_global;
  sp.tap_flag = tap_flag;
}

/* ----------------------------------------------------------------------
   PairKolmogorovCrespiFull::compute replaced by one engine evaluation (shared with tersoff/gb300
   under hybrid/overlay)
------------------------------------------------------------------------- */

void PairKolmogorovCrespiFullGB300::compute(int eflag, int vflag)
{
  ev_init(eflag,vflag);
  pvector[0] = pvector[1] = 0.0;
  lmff_lammps::StyleOut out;
  gb300::compute(lmp,this,this,1,eflag,vflag,eflag_atom,vflag_atom,"kolmogorov/crespi/full/gb300",out);
  if (eflag_global) eng_vdwl += out.eng_vdwl;
  if (vflag_global)
    for (int k = 0; k < 6; k++) virial[k] += out.virial[k];
  pvector[0] = out.pvector[0];
  pvector[1] = out.pvector[1];
}
