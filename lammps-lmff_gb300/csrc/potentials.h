// Host-side potential parameters (parsed files or copied from the LAMMPS pair styles).
#pragma once

#include <functional>
#include <string>
#include <vector>

#include "lmff_gb300.h"

namespace lmff {

struct HostTersoff {
  std::vector<std::string> elements;
  std::vector<int> map;  // [ntypes+1], -1 = NULL
  std::vector<lmff_tersoff_param> params;
  std::vector<int> elem2param;  // ne^3
  double cutmax = 0.0;
};

struct HostIlp {
  std::vector<std::string> elements;
  std::vector<int> map;
  std::vector<lmff_ilp_param> params;
  std::vector<int> elem2param;  // ne^2
  std::vector<double> cutILPsq;  // ne^2 (cutKCsq for Kolmogorov-Crespi)
  int model = LMFF_INTERLAYER_ILP;
  std::vector<lmff_kc_param> kc;  // model KC: the parameters (params stays empty)
};

bool parse_tersoff(const char *path, int ntypes, const char *const *elements, HostTersoff &out, std::string &err);
bool parse_ilp(const char *path, int ntypes, const char *const *elements, HostIlp &out, std::string &err);
bool parse_kc(const char *path, int ntypes, const char *const *elements, HostIlp &out, std::string &err);

}  // namespace lmff
