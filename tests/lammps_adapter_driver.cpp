// Drives the LAMMPS-side adapter (lammps-lmff_gb300/lammps/lmff_lammps_adapter.cpp) the
// way the pair styles do inside LAMMPS, without LAMMPS: a Tersoff style (slot 0) and an
// ILP style (slot 1) computed one after the other as PairHybrid::compute calls them,
// 32-bit tagint ids, forces and per-atom energies accumulated into contiguous arrays,
// a first call with reneighbouring and a second one without.  Test infrastructure for
// tests/test_lammps_adapter.py.
//
//   lammps_adapter_driver <potential dir> <in.bin> <out.bin>
// in.bin : int32 shared (0: one engine per style, 1: one engine for both, the first
//          style's call evaluating both), int32 nsub (0: the periodic form, one system;
//          k > 0: k subdomains in the subdomain form), double box[6], int32
//          periodic[3], tap_flag; then per system (one, or nsub): int32 nlocal, nall;
//          double x[nall*3]; int32 type[nall], mol[nall], tag[nall]
// out.bin: per call (two) and per system: double f[nall*3], eatom[nall], vatom[nall*6],
//          e_tersoff, e_ilp, pvector[2], virial[6] (sum of both styles)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "lmff_lammps_adapter.h"
#include "potentials.h"

struct Sys {
  int nlocal = 0, nall = 0;
  std::vector<double> x;
  std::vector<int32_t> type, mol, tag;
};

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  std::string pot = argv[1];
  FILE *fi = fopen(argv[2], "rb");
  if (!fi) return 3;
  int shared = 0, nsub = 0, per[3], tap = 1;
  double box[6];
  if (fread(&shared, 4, 1, fi) != 1 || fread(&nsub, 4, 1, fi) != 1 || fread(box, 8, 6, fi) != 6 ||
      fread(per, 4, 3, fi) != 3 || fread(&tap, 4, 1, fi) != 1)
    return 3;
  const bool subdomain = nsub > 0;
  std::vector<Sys> sys(subdomain ? nsub : 1);
  for (Sys &s : sys) {
    if (fread(&s.nlocal, 4, 1, fi) != 1 || fread(&s.nall, 4, 1, fi) != 1) return 3;
    const size_t n = s.nall;
    s.x.resize(3 * n);
    s.type.resize(n);
    s.mol.resize(n);
    s.tag.resize(n);
    if (fread(s.x.data(), 8, 3 * n, fi) != 3 * n || fread(s.type.data(), 4, n, fi) != n ||
        fread(s.mol.data(), 4, n, fi) != n || fread(s.tag.data(), 4, n, fi) != n)
      return 3;
  }
  fclose(fi);
  const char *elem[3] = {"C", "B", "N"};
  lmff::HostTersoff ht;
  lmff::HostIlp hi;
  std::string err;
  if (!lmff::parse_tersoff((pot + "/BNC.tersoff").c_str(), 3, elem, ht, err)) { fprintf(stderr, "%s\n", err.c_str()); return 4; }
  if (!lmff::parse_ilp((pot + "/BNCH.ILP").c_str(), 3, elem, hi, err)) { fprintf(stderr, "%s\n", err.c_str()); return 4; }
  // each style's part, as the styles' fill_params build them from their coeff() data
  lmff_lammps::StyleParams pt, pi;
  pt.ntypes = pi.ntypes = 3;
  pt.skin = pi.skin = 2.0;
  pt.tersoff = true;
  pt.t_nelements = (int)ht.elements.size();
  pt.t_params = ht.params;
  pt.t_elem2param = ht.elem2param;
  pt.t_map = ht.map;
  pt.t_cutmax = ht.cutmax;
  pi.interlayer = true;
  pi.i_nelements = (int)hi.elements.size();
  pi.ilp_params = hi.params;
  pi.i_elem2param = hi.elem2param;
  pi.i_map = hi.map;
  pi.i_cutsq = hi.cutILPsq;
  pi.cut_global = 16.0;
  pi.tap_flag = tap;
  // one engine per system and style (a rank has its own), or one per system shared
  const int nsys = (int)sys.size();
  std::vector<std::shared_ptr<lmff_lammps::Shared>> eng_t(nsys), eng_i(nsys);
  for (int k = 0; k < nsys; k++) {
    if (shared) {
      lmff_lammps::StyleParams both = pt;
      both.merge(pi);
      eng_t[k] = eng_i[k] = std::make_shared<lmff_lammps::Shared>();
      if (eng_t[k]->ad.create(both, 0, LMFF_FP64, err)) { fprintf(stderr, "%s\n", err.c_str()); return 5; }
    } else {
      eng_t[k] = std::make_shared<lmff_lammps::Shared>();
      eng_i[k] = std::make_shared<lmff_lammps::Shared>();
      if (eng_t[k]->ad.create(pt, 0, LMFF_FP64, err) || eng_i[k]->ad.create(pi, 0, LMFF_FP64, err)) {
        fprintf(stderr, "%s\n", err.c_str());
        return 5;
      }
    }
  }
  FILE *fo = fopen(argv[3], "wb");
  for (int call = 0; call < 2; call++) {
    for (int k = 0; k < nsys; k++) {
      Sys &s = sys[k];
      const size_t n = subdomain ? s.nall : s.nlocal;
      std::vector<double> f(3 * n, 0.0), eatom(n, 0.0), vatom(6 * n, 0.0);   // force_clear / ev_setup
      lmff_lammps::StyleOut ot, oi;
      const bool renei = call == 0;
      const bool partner = shared != 0;
      if (eng_t[k]->evaluate(0, partner, s.nlocal, s.nall, subdomain, s.x.data(), s.type.data(), s.mol.data(), nullptr,
                             s.tag.data(), nullptr, renei, box, box + 3, per, f.data(), eatom.data(), vatom.data(), 1,
                             1, ot, err) ||
          eng_i[k]->evaluate(1, partner, s.nlocal, s.nall, subdomain, s.x.data(), s.type.data(), s.mol.data(), nullptr,
                             s.tag.data(), nullptr, renei, box, box + 3, per, f.data(), eatom.data(), vatom.data(), 1,
                             1, oi, err)) {
        fprintf(stderr, "%s\n", err.c_str());
        return 6;
      }
      double vir[6];
      for (int q = 0; q < 6; q++) vir[q] = ot.virial[q] + oi.virial[q];
      fwrite(f.data(), 8, f.size(), fo);
      fwrite(eatom.data(), 8, n, fo);
      fwrite(vatom.data(), 8, 6 * n, fo);
      fwrite(&ot.eng_vdwl, 8, 1, fo);
      fwrite(&oi.eng_vdwl, 8, 1, fo);
      fwrite(oi.pvector, 8, 2, fo);
      fwrite(vir, 8, 6, fo);
    }
  }
  fclose(fo);
  return 0;
}
