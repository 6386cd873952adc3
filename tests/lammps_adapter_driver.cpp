// Drives the LAMMPS-side adapter (lammps-lmff_gb300/lammps/lmff_lammps_adapter.cpp) the
// way the two pair styles do inside LAMMPS, without LAMMPS: one adapter per sub-style
// (tersoff-only and ilp-only parameter sets), 32-bit tagint ids, forces and per-atom
// energies accumulated into contiguous arrays, a first call with reneighbouring and a
// second one without.  Test infrastructure for tests/test_lammps_adapter.py.
//
//   lammps_adapter_driver <potential dir> <in.bin> <out.bin>
// in.bin : int32 n, double box[6], int32 periodic[3], tap_flag; double x[n*3];
//          int32 type[n], mol[n], tag[n]
// out.bin: double f[n*3], eatom[n], e_tersoff, e_ilp, pvector[2], virial[6] (sum of
//          both styles), then the same quantities from the second (same-atoms) call
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lmff_lammps_adapter.h"
#include "potentials.h"

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  std::string pot = argv[1];
  FILE *fi = fopen(argv[2], "rb");
  if (!fi) return 3;
  int n = 0, per[3], tap = 1;
  double box[6];
  if (fread(&n, 4, 1, fi) != 1 || fread(box, 8, 6, fi) != 6 || fread(per, 4, 3, fi) != 3 || fread(&tap, 4, 1, fi) != 1)
    return 3;
  std::vector<double> x(3 * (size_t)n);
  std::vector<int32_t> type(n), mol(n), tag(n);
  if (fread(x.data(), 8, x.size(), fi) != x.size() || fread(type.data(), 4, n, fi) != (size_t)n ||
      fread(mol.data(), 4, n, fi) != (size_t)n || fread(tag.data(), 4, n, fi) != (size_t)n)
    return 3;
  fclose(fi);
  const char *elem[3] = {"C", "B", "N"};
  lmff::HostTersoff ht;
  lmff::HostIlp hi;
  std::string err;
  if (!lmff::parse_tersoff((pot + "/BNC.tersoff").c_str(), 3, elem, ht, err)) { fprintf(stderr, "%s\n", err.c_str()); return 4; }
  if (!lmff::parse_ilp((pot + "/BNCH.ILP").c_str(), 3, elem, hi, err)) { fprintf(stderr, "%s\n", err.c_str()); return 4; }
  lmff_params pt, pi;
  memset(&pt, 0, sizeof pt);
  memset(&pi, 0, sizeof pi);
  pt.ntypes = pi.ntypes = 3;
  pt.tersoff_nelements = (int)ht.elements.size();
  pt.tersoff_nparams = (int)ht.params.size();
  pt.tersoff_params = ht.params.data();
  pt.tersoff_elem2param = ht.elem2param.data();
  pt.tersoff_map = ht.map.data();
  pt.tersoff_cutmax = ht.cutmax;
  pt.skin = 2.0;
  pi.ilp_nelements = (int)hi.elements.size();
  pi.ilp_nparams = (int)hi.params.size();
  pi.ilp_params = hi.params.data();
  pi.ilp_elem2param = hi.elem2param.data();
  pi.ilp_map = hi.map.data();
  pi.ilp_cutILPsq = hi.cutILPsq.data();
  pi.ilp_cut_global = 16.0;
  pi.ilp_tap_flag = tap;
  pi.skin = 2.0;
  lmff_lammps::Adapter at, ai;
  if (at.create(pt, 0, LMFF_FP64, err) || ai.create(pi, 0, LMFF_FP64, err)) { fprintf(stderr, "%s\n", err.c_str()); return 5; }
  FILE *fo = fopen(argv[3], "wb");
  for (int call = 0; call < 2; call++) {
    std::vector<double> f(3 * (size_t)n, 0.0), eatom(n, 0.0);  // force_clear / ev_setup
    lmff_lammps::StyleOut ot, oi;
    bool renei = call == 0;
    if (at.compute(LMFF_TERSOFF, n, x.data(), type.data(), nullptr, nullptr, tag.data(), nullptr, renei, box, box + 3,
                   per, f.data(), eatom.data(), 1, 1, ot, err) ||
        ai.compute(LMFF_ILP, n, x.data(), type.data(), mol.data(), nullptr, tag.data(), nullptr, renei, box, box + 3,
                   per, f.data(), eatom.data(), 1, 1, oi, err)) {
      fprintf(stderr, "%s\n", err.c_str());
      return 6;
    }
    double vir[6];
    for (int k = 0; k < 6; k++) vir[k] = ot.virial[k] + oi.virial[k];
    if (getenv("LMFF_DRIVER_DEBUG")) {
      double fm = 0;
      for (double v : f) fm = fm > fabs(v) ? fm : fabs(v);
      fprintf(stderr, "call %d max|f| %g et %g ei %g\n", call, fm, ot.eng_vdwl, oi.eng_vdwl);
    }
    fwrite(f.data(), 8, f.size(), fo);
    fwrite(eatom.data(), 8, n, fo);
    fwrite(&ot.eng_vdwl, 8, 1, fo);
    fwrite(&oi.eng_vdwl, 8, 1, fo);
    fwrite(oi.pvector, 8, 2, fo);
    fwrite(vir, 8, 6, fo);
  }
  fclose(fo);
  return 0;
}
