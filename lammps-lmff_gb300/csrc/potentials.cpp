// Potential-file parsing with the reference's semantics, for callers that do not come
// through LAMMPS (standalone runs, serving, tests).  Inside LAMMPS the pair styles'
// own read_file/setup_params fill lmff_params instead.
//   Tersoff: pair_tersoff.cpp:392-580 (17 words per entry, '#' comments, continuation
//            lines, element filtering, parameter checks, elem2param duplicates/missing,
//            cut/cutsq/c1..c4, cutmax)
//   ILP:     pair_ilp_graphene_hbn.cpp:246-387 (13 words per entry, meV*S scaling,
//            delta2inv/lambda/seff, elem2param, cutILPsq)
#include "potentials.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace lmff {

static int count_words(const char *line) {
  int n = 0, in = 0;
  for (const char *c = line; *c; c++) {
    int ws = (*c == ' ' || *c == '\t' || *c == '\n' || *c == '\r' || *c == '\f');
    if (!ws && !in) n++;
    in = !ws;
  }
  return n;
}

static bool read_entries(const char *path, int per, const char *what, std::string &err,
                         const std::function<bool(std::vector<std::string> &)> &cb) {
  FILE *fp = fopen(path, "r");
  if (!fp) {
    err = std::string("Cannot open ") + what + " potential file " + path;
    return false;
  }
  std::vector<char> line(1024 * 8);
  bool ok = true;
  while (fgets(line.data(), 1024, fp)) {
    char *ptr;
    if ((ptr = strchr(line.data(), '#'))) *ptr = '\0';
    int nwords = count_words(line.data());
    if (nwords == 0) continue;
    while (nwords < per) {
      size_t n = strlen(line.data());
      if (!fgets(line.data() + n, (int)(line.size() - n), fp)) break;
      if ((ptr = strchr(line.data(), '#'))) *ptr = '\0';
      nwords = count_words(line.data());
    }
    if (nwords != per) {
      err = std::string("Incorrect format in ") + what + " potential file";
      ok = false;
      break;
    }
    std::vector<std::string> w;
    char *tok = strtok(line.data(), " \t\n\r\f");
    while (tok) {
      w.emplace_back(tok);
      tok = strtok(nullptr, " \t\n\r\f");
    }
    if (!cb(w)) {
      ok = false;
      break;
    }
  }
  fclose(fp);
  return ok;
}

// element list and type map as PairTersoff::coeff / PairILPGrapheneHBN::coeff build them
static int map_elements(int ntypes, const char *const *elements, std::vector<int> &map, std::vector<std::string> &names) {
  map.assign(ntypes + 1, -1);
  names.clear();
  for (int t = 1; t <= ntypes; t++) {
    const char *e = elements[t - 1];
    if (strcmp(e, "NULL") == 0) continue;
    int j = 0;
    for (; j < (int)names.size(); j++)
      if (names[j] == e) break;
    map[t] = j;
    if (j == (int)names.size()) names.emplace_back(e);
  }
  return (int)names.size();
}

bool parse_tersoff(const char *path, int ntypes, const char *const *elements, HostTersoff &out, std::string &err) {
  out = HostTersoff();
  int ne = map_elements(ntypes, elements, out.map, out.elements);
  if (ne == 0) {
    err = "Incorrect args for pair coefficients";
    return false;
  }
  auto find = [&](const std::string &w) {
    for (int i = 0; i < ne; i++)
      if (out.elements[i] == w) return i;
    return -1;
  };
  bool ok = read_entries(path, 17, "Tersoff", err, [&](std::vector<std::string> &w) {
    int ie = find(w[0]), je = find(w[1]), ke = find(w[2]);
    if (ie < 0 || je < 0 || ke < 0) return true;
    lmff_tersoff_param q;
    memset(&q, 0, sizeof q);
    q.ielement = ie;
    q.jelement = je;
    q.kelement = ke;
    q.powerm = atof(w[3].c_str());
    q.gamma = atof(w[4].c_str());
    q.lam3 = atof(w[5].c_str());
    q.c = atof(w[6].c_str());
    q.d = atof(w[7].c_str());
    q.h = atof(w[8].c_str());
    q.powern = atof(w[9].c_str());
    q.beta = atof(w[10].c_str());
    q.lam2 = atof(w[11].c_str());
    q.bigb = atof(w[12].c_str());
    q.bigr = atof(w[13].c_str());
    q.bigd = atof(w[14].c_str());
    q.lam1 = atof(w[15].c_str());
    q.biga = atof(w[16].c_str());
    q.powermint = (int)q.powerm;
    if (q.c < 0.0 || q.d < 0.0 || q.powern < 0.0 || q.beta < 0.0 || q.lam2 < 0.0 || q.bigb < 0.0 || q.bigr < 0.0 ||
        q.bigd < 0.0 || q.bigd > q.bigr || q.lam1 < 0.0 || q.biga < 0.0 || q.powerm - q.powermint != 0.0 ||
        (q.powermint != 3 && q.powermint != 1) || q.gamma < 0.0) {
      err = "Illegal Tersoff parameter";
      return false;
    }
    out.params.push_back(q);
    return true;
  });
  if (!ok) return false;
  out.elem2param.assign(ne * ne * ne, -1);
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < ne; j++)
      for (int k = 0; k < ne; k++) {
        int n = -1;
        for (int m = 0; m < (int)out.params.size(); m++) {
          const auto &q = out.params[m];
          if (q.ielement == i && q.jelement == j && q.kelement == k) {
            if (n >= 0) {
              err = "Potential file has duplicate entry";
              return false;
            }
            n = m;
          }
        }
        if (n < 0) {
          err = "Potential file is missing an entry";
          return false;
        }
        out.elem2param[(i * ne + j) * ne + k] = n;
      }
  out.cutmax = 0.0;
  for (auto &q : out.params) {
    q.cut = q.bigr + q.bigd;
    q.cutsq = q.cut * q.cut;
    q.c1 = pow(2.0 * q.powern * 1.0e-16, -1.0 / q.powern);
    q.c2 = pow(2.0 * q.powern * 1.0e-8, -1.0 / q.powern);
    q.c3 = 1.0 / q.c2;
    q.c4 = 1.0 / q.c1;
    if (q.cut > out.cutmax) out.cutmax = q.cut;
  }
  return true;
}

bool parse_ilp(const char *path, int ntypes, const char *const *elements, HostIlp &out, std::string &err) {
  out = HostIlp();
  int ne = map_elements(ntypes, elements, out.map, out.elements);
  if (ne == 0) {
    err = "Incorrect args for pair coefficients";
    return false;
  }
  auto find = [&](const std::string &w) {
    for (int i = 0; i < ne; i++)
      if (out.elements[i] == w) return i;
    return -1;
  };
  bool ok = read_entries(path, 13, "ILP", err, [&](std::vector<std::string> &w) {
    int ie = find(w[0]), je = find(w[1]);
    if (ie < 0 || je < 0) return true;
    lmff_ilp_param q;
    memset(&q, 0, sizeof q);
    q.ielement = ie;
    q.jelement = je;
    q.z0 = atof(w[2].c_str());
    q.alpha = atof(w[3].c_str());
    q.delta = atof(w[4].c_str());
    q.epsilon = atof(w[5].c_str());
    q.C = atof(w[6].c_str());
    q.d = atof(w[7].c_str());
    q.sR = atof(w[8].c_str());
    q.reff = atof(w[9].c_str());
    q.C6 = atof(w[10].c_str());
    q.S = atof(w[11].c_str());
    q.rcut = atof(w[12].c_str());
    double meV = 1e-3 * q.S;
    q.C *= meV;
    q.C6 *= meV;
    q.epsilon *= meV;
    q.delta2inv = pow(q.delta, -2.0);
    q.lambda = q.alpha / q.z0;
    q.seff = q.sR * q.reff;
    out.params.push_back(q);
    return true;
  });
  if (!ok) return false;
  out.elem2param.assign(ne * ne, -1);
  out.cutILPsq.assign(ne * ne, 0.0);
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < ne; j++) {
      int n = -1;
      for (int m = 0; m < (int)out.params.size(); m++) {
        if (out.params[m].ielement == i && out.params[m].jelement == j) {
          if (n >= 0) {
            err = "Potential file has duplicate entry";
            return false;
          }
          n = m;
        }
      }
      if (n < 0) {
        err = "Potential file is missing an entry";
        return false;
      }
      out.elem2param[i * ne + j] = n;
      out.cutILPsq[i * ne + j] = out.params[n].rcut * out.params[n].rcut;
    }
  return true;
}

// pair_kolmogorov_crespi_full.cpp read_file (:247-392): 12 words per entry, energies in
// meV scaled by S, every ordered element pair exactly once.
bool parse_kc(const char *path, int ntypes, const char *const *elements, HostIlp &out, std::string &err) {
  out = HostIlp();
  out.model = LMFF_INTERLAYER_KC;
  int ne = map_elements(ntypes, elements, out.map, out.elements);
  if (ne == 0) {
    err = "Incorrect args for pair coefficients";
    return false;
  }
  auto find = [&](const std::string &w) {
    for (int i = 0; i < ne; i++)
      if (out.elements[i] == w) return i;
    return -1;
  };
  bool ok = read_entries(path, 12, "KC", err, [&](std::vector<std::string> &w) {
    int ie = find(w[0]), je = find(w[1]);
    if (ie < 0 || je < 0) return true;
    lmff_kc_param q;
    memset(&q, 0, sizeof q);
    q.ielement = ie;
    q.jelement = je;
    q.z0 = atof(w[2].c_str());
    q.C0 = atof(w[3].c_str());
    q.C2 = atof(w[4].c_str());
    q.C4 = atof(w[5].c_str());
    q.C = atof(w[6].c_str());
    q.delta = atof(w[7].c_str());
    q.lambda = atof(w[8].c_str());
    q.A = atof(w[9].c_str());
    q.S = atof(w[10].c_str());
    q.rcut = atof(w[11].c_str());
    double meV = 1e-3 * q.S;
    q.C *= meV;
    q.A *= meV;
    q.C0 *= meV;
    q.C2 *= meV;
    q.C4 *= meV;
    q.delta2inv = pow(q.delta, -2.0);
    q.z06 = pow(q.z0, 6.0);
    out.kc.push_back(q);
    return true;
  });
  if (!ok) return false;
  out.elem2param.assign(ne * ne, -1);
  out.cutILPsq.assign(ne * ne, 0.0);
  for (int i = 0; i < ne; i++)
    for (int j = 0; j < ne; j++) {
      int n = -1;
      for (int m = 0; m < (int)out.kc.size(); m++) {
        if (out.kc[m].ielement == i && out.kc[m].jelement == j) {
          if (n >= 0) {
            err = "Potential file has duplicate entry";
            return false;
          }
          n = m;
        }
      }
      if (n < 0) {
        err = "Potential file is missing an entry";
        return false;
      }
      out.elem2param[i * ne + j] = n;
      out.cutILPsq[i * ne + j] = out.kc[n].rcut * out.kc[n].rcut;
    }
  return true;
}

}  // namespace lmff
