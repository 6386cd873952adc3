// Reference harness: runs a LAMMPS input script through the reference's own
// pair styles (Rft/MANYBODY/pair_tersoff.cpp, Rft/USER-MISC/pair_ilp_graphene_hbn.cpp,
// stock hybrid/overlay) and dumps what the parity tests compare against.
//
// Test infrastructure only (built by oracle/ref.mk into oracle/_ref/).
//
//   lmff_ref <input-script> <out.bin> [lists] [min] [-- <LAMMPS command-line arguments>]
//
// Without "--" LAMMPS runs quietly (-log none -screen none); after "--" the given
// arguments are passed to LAMMPS instead (e.g. -sf gb300 -screen stdout).
//
// out.bin is a sequence of records: char name[16], char kind ('d' double, 'q' int64),
// int64 count, then count elements.  Atoms are reported in tag order.
// With "lists", the ILP sub-style's full+ghost list (pair_ilp_graphene_hbn.cpp:402-405)
// and its intralayer list (ILP_neigh, :681-745) are written as (tag_i, tag_j, image)
// triples, image = periodic image of j relative to its owned copy.
// With "min", the last minimize's statistics (Min::niter, neval, stop_condition,
// einitial, efinal, fnorm2_final, fnorminf_final, alpha_final; min.h:23-27) are written.

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>
#include <algorithm>
#include <string>
#include <map>
#include <mpi.h>

#define protected public
#include "lammps.h"
#include "input.h"
#include "atom.h"
#include "force.h"
#include "pair.h"
#include "pair_hybrid.h"
#include "domain.h"
#include "modify.h"
#include "compute.h"
#include "neigh_list.h"
#include "update.h"
#include "min.h"
#include "pair_ilp_graphene_hbn.h"
#undef protected

using namespace LAMMPS_NS;

static FILE *g_out;

static void rec(const char *name, char kind, int64_t n, const void *data) {
  char nm[16];
  memset(nm, 0, 16);
  strncpy(nm, name, 15);
  fwrite(nm, 1, 16, g_out);
  fwrite(&kind, 1, 1, g_out);
  fwrite(&n, sizeof(int64_t), 1, g_out);
  fwrite(data, kind == 'd' ? sizeof(double) : sizeof(int64_t), (size_t)n, g_out);
}

static int64_t image_code(LAMMPS *lmp, int j) {
  // periodic image of atom j relative to its owned copy, each component in [-8,7]
  Atom *atom = lmp->atom;
  Domain *d = lmp->domain;
  int owner = atom->map(atom->tag[j]);
  double prd[3] = {d->xprd, d->yprd, d->zprd};
  int64_t code = 0;
  for (int c = 0; c < 3; c++) {
    long s = 0;
    if (d->periodicity[c]) s = lround((atom->x[j][c] - atom->x[owner][c]) / prd[c]);
    code |= ((s + 8) & 15) << (4 * c);
  }
  return code;
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s in.lmp out.bin [lists]\n", argv[0]);
    return 2;
  }
  bool lists = false, minstats = false;
  for (int a = 3; a < argc && strcmp(argv[a], "--") != 0; a++) {
    if (strcmp(argv[a], "lists") == 0) lists = true;
    if (strcmp(argv[a], "min") == 0) minstats = true;
  }
  std::vector<const char *> largs = {"lmff_ref", "-log", "none", "-screen", "none", "-nocite"};
  for (int a = 3; a < argc; a++)
    if (strcmp(argv[a], "--") == 0) {
      largs.assign(1, "lmff_ref");
      for (int b = a + 1; b < argc; b++) largs.push_back(argv[b]);
      break;
    }
  MPI_Init(&argc, &argv);
  LAMMPS *lmp = new LAMMPS((int)largs.size(), (char **)largs.data(), MPI_COMM_WORLD);
  lmp->input->file(argv[1]);

  g_out = fopen(argv[2], "wb");
  if (!g_out) { perror("open out"); return 1; }
  Atom *atom = lmp->atom;
  int nlocal = atom->nlocal;
  std::vector<int> order(nlocal);
  for (int i = 0; i < nlocal; i++) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return atom->tag[a] < atom->tag[b]; });

  std::vector<double> xs, fs, vs;
  std::vector<int64_t> tags, types, mols;
  for (int ii = 0; ii < nlocal; ii++) {
    int i = order[ii];
    for (int c = 0; c < 3; c++) {
      xs.push_back(atom->x[i][c]);
      fs.push_back(atom->f[i][c]);
      vs.push_back(atom->v[i][c]);
    }
    tags.push_back(atom->tag[i]);
    types.push_back(atom->type[i]);
    mols.push_back(atom->molecule ? atom->molecule[i] : 0);
  }
  rec("x", 'd', xs.size(), xs.data());
  rec("f", 'd', fs.size(), fs.data());
  rec("v", 'd', vs.size(), vs.data());
  rec("tag", 'q', tags.size(), tags.data());
  rec("type", 'q', types.size(), types.data());
  rec("mol", 'q', mols.size(), mols.data());
  int64_t step = lmp->update->ntimestep;
  rec("step", 'q', 1, &step);
  double box[6] = {lmp->domain->boxlo[0], lmp->domain->boxlo[1], lmp->domain->boxlo[2],
                   lmp->domain->boxhi[0], lmp->domain->boxhi[1], lmp->domain->boxhi[2]};
  rec("box", 'd', 6, box);
  if (lmp->domain->triclinic) {
    double tilt[3] = {lmp->domain->xy, lmp->domain->xz, lmp->domain->yz};
    rec("tilt", 'd', 3, tilt);
  }

  Pair *pair = lmp->force->pair;
  rec("virial", 'd', 6, pair->virial);
  double etot = pair->eng_vdwl;
  rec("e_pair", 'd', 1, &etot);

  PairILPGrapheneHBN *ilp = NULL;
  if (strcmp(lmp->force->pair_style, "hybrid/overlay") == 0) {
    PairHybrid *h = (PairHybrid *)pair;
    for (int m = 0; m < h->nstyles; m++) {
      std::string kw = h->keywords[m];
      // the interlayer style (ILP or Kolmogorov-Crespi full) is reported as e_ilp
      bool inter = kw == "ilp/graphene/hbn" || kw == "kolmogorov/crespi/full";
      std::string key = inter ? "e_ilp" : "e_" + kw;
      rec(key.c_str(), 'd', 1, &h->styles[m]->eng_vdwl);
      if (inter) rec("pvector", 'd', 2, h->styles[m]->pvector);
      if (kw == "ilp/graphene/hbn") ilp = (PairILPGrapheneHBN *)h->styles[m];
    }
  }

  int ic = lmp->modify->find_compute("peatom");
  if (ic >= 0 && lmp->modify->compute[ic]->vector_atom) {
    std::vector<double> ea;
    for (int ii = 0; ii < nlocal; ii++) ea.push_back(lmp->modify->compute[ic]->vector_atom[order[ii]]);
    rec("eatom", 'd', ea.size(), ea.data());
  }

  // Per-atom virial of each sub-style (Pair::vatom as its ev_tally / ev_tally_xyz /
  // v_tally3 calls left it), when the script defines a stress/atom compute named
  // "satom" that was invoked on the last step (that sets vflag_atom).  Ghost rows are
  // folded into their owned atoms as Comm::reverse_comm does for compute stress/atom
  // (Atom::map returns the owned copy of a tag); rows are in tag order, 6 per atom
  // (xx yy zz xy xz yz).
  if (lmp->modify->find_compute("satom") >= 0 && strcmp(lmp->force->pair_style, "hybrid/overlay") == 0) {
    PairHybrid *h = (PairHybrid *)pair;
    int nall = nlocal + atom->nghost;
    for (int m = 0; m < h->nstyles; m++) {
      Pair *ps = h->styles[m];
      if (!ps->vatom) continue;
      std::vector<double> fold((size_t)nlocal * 6, 0.0);
      for (int i = 0; i < nall; i++) {
        int o = i < nlocal ? i : atom->map(atom->tag[i]);
        if (o < 0 || o >= nlocal) continue;
        for (int c = 0; c < 6; c++) fold[(size_t)o * 6 + c] += ps->vatom[i][c];
      }
      std::vector<double> va;
      for (int ii = 0; ii < nlocal; ii++)
        for (int c = 0; c < 6; c++) va.push_back(fold[(size_t)order[ii] * 6 + c]);
      std::string kw = h->keywords[m];
      bool inter = kw == "ilp/graphene/hbn" || kw == "kolmogorov/crespi/full";
      rec(inter ? "vatom_ilp" : "vatom_tersoff", 'd', va.size(), va.data());
    }
  }

  if (minstats && lmp->update->minimize) {
    Min *m = lmp->update->minimize;
    int64_t q[3] = {m->niter, m->neval, m->stop_condition};
    rec("min_counts", 'q', 3, q);
    double d[5] = {m->einitial, m->efinal, m->fnorm2_final, m->fnorminf_final, m->alpha_final};
    rec("min_values", 'd', 5, d);
  }

  if (lists && ilp) {
    NeighList *list = ilp->list;
    std::vector<int64_t> nl;
    for (int ii = 0; ii < list->inum; ii++) {
      int i = list->ilist[ii];
      for (int jj = 0; jj < list->numneigh[i]; jj++) {
        int j = list->firstneigh[i][jj] & NEIGHMASK;
        nl.push_back(atom->tag[i]);
        nl.push_back(atom->tag[j]);
        nl.push_back(image_code(lmp, j));
      }
    }
    rec("nlist", 'q', nl.size(), nl.data());
    std::vector<int64_t> il;
    for (int ii = 0; ii < list->inum; ii++) {
      int i = list->ilist[ii];
      for (int kk = 0; kk < ilp->ILP_numneigh[i]; kk++) {
        int k = ilp->ILP_firstneigh[i][kk];
        il.push_back(atom->tag[i]);
        il.push_back(atom->tag[k]);
        il.push_back(image_code(lmp, k));
      }
    }
    rec("ilplist", 'q', il.size(), il.data());
  }
  fclose(g_out);
  delete lmp;
  MPI_Finalize();
  return 0;
}
