/* CPU oracle: plain-C restatement of the reference Tersoff + ILP path.
 * TEST INFRASTRUCTURE ONLY -- see lmff_oracle.h for scope and the reference
 * file:line map.  Compiled with -ffp-contract=off so that results agree between x86
 * and Arm hosts and the neighbour-set decisions use the reference's rounding. */
#include "lmff_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Op-count markers: oracle/opcount.cpp compiles this file with an operation-counting
 * floating-point type and defines these to attribute the operations to categories and
 * count the units of each (candidates, pairs, triplets, ...).  Empty here. */
#define ORC_CAT_OTHER 0
#define ORC_CAT_ILP_CAND 1     /* an interlayer candidate's distance and cutoff test */
#define ORC_CAT_ILP_PAIR 2     /* a directed pair in the cutoff: taper, repulsion term, forces */
#define ORC_CAT_ILP_VDW 3      /* the vdW term of the pairs the tag parity selects */
#define ORC_CAT_ILP_KTERM 4    /* calc_FRep's force on one intralayer neighbour k of i */
#define ORC_CAT_NORMAL 5       /* calc_normal of one atom: normal and its Jacobians */
#define ORC_CAT_TERS_CAND 6    /* Tersoff's scan of the full list for short neighbours */
#define ORC_CAT_TERS_REP 7     /* repulsive term of a bond (tag-parity half) */
#define ORC_CAT_TERS_BOND 8    /* force_zeta of a directed bond */
#define ORC_CAT_TERS_ZETA 9    /* zeta term of a triplet */
#define ORC_CAT_TERS_ATTR 10   /* attractive (three-body force) of a triplet */
#define ORC_CAT_ILP_DSELF 11   /* calc_FRep's term of dn_i/dx_i (per pair) */
#define ORC_NCAT 12
#ifndef ORC_OPCAT
#define ORC_OPCAT(cat) ((void)0)
#define ORC_OPUNIT(cat) ((void)0)
#endif

#define MY_PI2 1.57079632679489661923
#define MY_PI4 0.78539816339744830962
#define MAXLINE 1024
#define MAXSHORT 64

/* ===================================================================== params == */

int orc_pot_init(orc_pot *p, int ntypes, double cut_global, int tap_flag, double skin) {
  memset(p, 0, sizeof(*p));
  if (ntypes < 1 || ntypes > ORC_MAXTYPE) {
    snprintf(p->err, sizeof p->err, "ntypes out of range");
    return -1;
  }
  p->ntypes = ntypes;
  p->cut_global = cut_global;
  p->tap_flag = tap_flag;
  p->skin = skin;
  for (int t = 0; t <= ORC_MAXTYPE; t++) p->t_map[t] = p->i_map[t] = -1;
  return 0;
}

const char *orc_pot_error(const orc_pot *p) { return p->err; }

/* element list from the pair_coeff words (pair_tersoff.cpp:312-334) */
static int map_elements(int ntypes, const char *const *elem_of_type, int *map, char names[][16]) {
  int nelem = 0;
  for (int t = 1; t <= ntypes; t++) {
    const char *e = elem_of_type[t - 1];
    if (strcmp(e, "NULL") == 0) {
      map[t] = -1;
      continue;
    }
    int j;
    for (j = 0; j < nelem; j++)
      if (strcmp(e, names[j]) == 0) break;
    map[t] = j;
    if (j == nelem) {
      if (nelem == ORC_MAXELEM) return -1;
      strncpy(names[j], e, 15);
      names[j][15] = 0;
      nelem++;
    }
  }
  return nelem;
}

static int count_words(const char *line) {
  int n = 0, in = 0;
  for (const char *c = line; *c; c++) {
    int ws = (*c == ' ' || *c == '\t' || *c == '\n' || *c == '\r' || *c == '\f');
    if (!ws && !in) n++;
    in = !ws;
  }
  return n;
}

/* Reads entries of nwords_per words each, concatenating lines and stripping '#'
 * comments as pair_tersoff.cpp:420-465 does.  Calls cb for every complete entry. */
typedef int (*entry_cb)(orc_pot *p, char **words, void *ctx);
static int read_entries(orc_pot *p, const char *path, int per, entry_cb cb, void *ctx, const char *what) {
  FILE *fp = fopen(path, "r");
  if (!fp) {
    snprintf(p->err, sizeof p->err, "Cannot open %s potential file %s", what, path);
    return -1;
  }
  char line[MAXLINE * 4];
  char *words[64];
  int rc = 0;
  while (fgets(line, MAXLINE, fp)) {
    char *ptr;
    if ((ptr = strchr(line, '#'))) *ptr = '\0';
    int nwords = count_words(line);
    if (nwords == 0) continue;
    while (nwords < per) {
      size_t n = strlen(line);
      if (!fgets(&line[n], (int)(sizeof line - n), fp)) break;
      if ((ptr = strchr(line, '#'))) *ptr = '\0';
      nwords = count_words(line);
    }
    if (nwords != per) {
      snprintf(p->err, sizeof p->err, "Incorrect format in %s potential file", what);
      rc = -1;
      break;
    }
    int k = 0;
    words[k++] = strtok(line, " \t\n\r\f");
    while ((words[k++] = strtok(NULL, " \t\n\r\f")) && k < 63) continue;
    if ((rc = cb(p, words, ctx)) != 0) break;
  }
  fclose(fp);
  return rc;
}

struct elem_ctx {
  int nelem;
  char names[ORC_MAXELEM][16];
};

static int find_elem(struct elem_ctx *e, const char *w) {
  for (int i = 0; i < e->nelem; i++)
    if (strcmp(w, e->names[i]) == 0) return i;
  return -1;
}

static int ters_entry(orc_pot *p, char **w, void *vctx) {
  struct elem_ctx *e = (struct elem_ctx *)vctx;
  int ie = find_elem(e, w[0]), je = find_elem(e, w[1]), ke = find_elem(e, w[2]);
  if (ie < 0 || je < 0 || ke < 0) return 0;
  if (p->t_nparams >= ORC_MAXELEM * ORC_MAXELEM * ORC_MAXELEM) return -1;
  orc_ters_param *q = &p->t_params[p->t_nparams];
  memset(q, 0, sizeof *q);
  q->ielement = ie;
  q->jelement = je;
  q->kelement = ke;
  q->powerm = atof(w[3]);
  q->gamma = atof(w[4]);
  q->lam3 = atof(w[5]);
  q->c = atof(w[6]);
  q->d = atof(w[7]);
  q->h = atof(w[8]);
  q->powern = atof(w[9]);
  q->beta = atof(w[10]);
  q->lam2 = atof(w[11]);
  q->bigb = atof(w[12]);
  q->bigr = atof(w[13]);
  q->bigd = atof(w[14]);
  q->lam1 = atof(w[15]);
  q->biga = atof(w[16]);
  q->powermint = (int)q->powerm;
  /* pair_tersoff.cpp:511-526 */
  if (q->c < 0.0 || q->d < 0.0 || q->powern < 0.0 || q->beta < 0.0 || q->lam2 < 0.0 ||
      q->bigb < 0.0 || q->bigr < 0.0 || q->bigd < 0.0 || q->bigd > q->bigr || q->lam1 < 0.0 ||
      q->biga < 0.0 || q->powerm - q->powermint != 0.0 ||
      (q->powermint != 3 && q->powermint != 1) || q->gamma < 0.0) {
    snprintf(p->err, sizeof p->err, "Illegal Tersoff parameter");
    return -1;
  }
  p->t_nparams++;
  return 0;
}

int orc_read_tersoff(orc_pot *p, const char *path, const char *const *elem_of_type) {
  struct elem_ctx e;
  memset(&e, 0, sizeof e);
  e.nelem = map_elements(p->ntypes, elem_of_type, p->t_map, e.names);
  if (e.nelem <= 0) {
    snprintf(p->err, sizeof p->err, "Incorrect args for pair coefficients");
    return -1;
  }
  p->t_nelements = e.nelem;
  p->t_nparams = 0;
  if (read_entries(p, path, 17, ters_entry, &e, "Tersoff")) return -1;
  /* setup_params, pair_tersoff.cpp:547-579 */
  for (int i = 0; i < e.nelem; i++)
    for (int j = 0; j < e.nelem; j++)
      for (int k = 0; k < e.nelem; k++) {
        int n = -1;
        for (int m = 0; m < p->t_nparams; m++)
          if (p->t_params[m].ielement == i && p->t_params[m].jelement == j &&
              p->t_params[m].kelement == k) {
            if (n >= 0) {
              snprintf(p->err, sizeof p->err, "Potential file has duplicate entry");
              return -1;
            }
            n = m;
          }
        if (n < 0) {
          snprintf(p->err, sizeof p->err, "Potential file is missing an entry");
          return -1;
        }
        p->t_e2p[i][j][k] = n;
      }
  p->t_cutmax = 0.0;
  for (int m = 0; m < p->t_nparams; m++) {
    orc_ters_param *q = &p->t_params[m];
    q->cut = q->bigr + q->bigd;
    q->cutsq = q->cut * q->cut;
    q->c1 = pow(2.0 * q->powern * 1.0e-16, -1.0 / q->powern);
    q->c2 = pow(2.0 * q->powern * 1.0e-8, -1.0 / q->powern);
    q->c3 = 1.0 / q->c2;
    q->c4 = 1.0 / q->c1;
    if (q->cut > p->t_cutmax) p->t_cutmax = q->cut;
  }
  p->t_enabled = 1;
  return 0;
}

static int ilp_entry(orc_pot *p, char **w, void *vctx) {
  struct elem_ctx *e = (struct elem_ctx *)vctx;
  int ie = find_elem(e, w[0]), je = find_elem(e, w[1]);
  if (ie < 0 || je < 0) return 0;
  if (p->i_nparams >= ORC_MAXELEM * ORC_MAXELEM) return -1;
  orc_ilp_param *q = &p->i_params[p->i_nparams];
  memset(q, 0, sizeof *q);
  q->ielement = ie;
  q->jelement = je;
  q->z0 = atof(w[2]);
  q->alpha = atof(w[3]);
  q->delta = atof(w[4]);
  q->epsilon = atof(w[5]);
  q->C = atof(w[6]);
  q->d = atof(w[7]);
  q->sR = atof(w[8]);
  q->reff = atof(w[9]);
  q->C6 = atof(w[10]);
  q->S = atof(w[11]);
  q->rcut = atof(w[12]);
  /* pair_ilp_graphene_hbn.cpp:354-364 */
  double meV = 1e-3 * q->S;
  q->C *= meV;
  q->C6 *= meV;
  q->epsilon *= meV;
  q->delta2inv = pow(q->delta, -2.0);
  q->lambda = q->alpha / q->z0;
  q->seff = q->sR * q->reff;
  p->i_nparams++;
  return 0;
}

/* pair_kolmogorov_crespi_full.cpp:340-365: 12 words, energies in meV scaled by S */
static int kc_entry(orc_pot *p, char **w, void *vctx) {
  struct elem_ctx *e = (struct elem_ctx *)vctx;
  int ie = find_elem(e, w[0]), je = find_elem(e, w[1]);
  if (ie < 0 || je < 0) return 0;
  if (p->i_nparams >= ORC_MAXELEM * ORC_MAXELEM) return -1;
  orc_ilp_param *q = &p->i_params[p->i_nparams];
  memset(q, 0, sizeof *q);
  q->ielement = ie;
  q->jelement = je;
  q->z0 = atof(w[2]);
  q->C0 = atof(w[3]);
  q->C2 = atof(w[4]);
  q->C4 = atof(w[5]);
  q->C = atof(w[6]);
  q->delta = atof(w[7]);
  q->lambda = atof(w[8]);
  q->A = atof(w[9]);
  q->S = atof(w[10]);
  q->rcut = atof(w[11]);
  double meV = 1e-3 * q->S;
  q->C *= meV;
  q->A *= meV;
  q->C0 *= meV;
  q->C2 *= meV;
  q->C4 *= meV;
  q->delta2inv = pow(q->delta, -2.0);
  q->z06 = pow(q->z0, 6.0);
  p->i_nparams++;
  return 0;
}

static int read_interlayer(orc_pot *p, const char *path, const char *const *elem_of_type, int model) {
  struct elem_ctx e;
  memset(&e, 0, sizeof e);
  e.nelem = map_elements(p->ntypes, elem_of_type, p->i_map, e.names);
  if (e.nelem <= 0) {
    snprintf(p->err, sizeof p->err, "Incorrect args for pair coefficients");
    return -1;
  }
  p->i_nelements = e.nelem;
  p->i_nparams = 0;
  p->i_model = model;
  if (model == 0 && read_entries(p, path, 13, ilp_entry, &e, "ILP")) return -1;
  if (model == 1 && read_entries(p, path, 12, kc_entry, &e, "KC")) return -1;
  for (int i = 0; i < e.nelem; i++)
    for (int j = 0; j < e.nelem; j++) {
      int n = -1;
      for (int m = 0; m < p->i_nparams; m++)
        if (p->i_params[m].ielement == i && p->i_params[m].jelement == j) {
          if (n >= 0) {
            snprintf(p->err, sizeof p->err, "Potential file has duplicate entry");
            return -1;
          }
          n = m;
        }
      if (n < 0) {
        snprintf(p->err, sizeof p->err, "Potential file is missing an entry");
        return -1;
      }
      p->i_e2p[i][j] = n;
      p->i_cutILPsq[i][j] = p->i_params[n].rcut * p->i_params[n].rcut;
    }
  p->i_enabled = 1;
  return 0;
}

int orc_read_ilp(orc_pot *p, const char *path, const char *const *elem_of_type) {
  return read_interlayer(p, path, elem_of_type, 0);
}

int orc_read_kc(orc_pot *p, const char *path, const char *const *elem_of_type) {
  return read_interlayer(p, path, elem_of_type, 1);
}

/* ==================================================================== context == */

struct orc_ctx {
  orc_pot p;
  int nthreads;
  int nlocal, nall, cap_all;
  double *x;          /* nall*3, owned first */
  int *type;
  int64_t *mol, *tag;
  int *owner;         /* owned index of each atom */
  int *shift;         /* nall*3 image of each atom relative to its owner */
  double lo[3], hi[3];
  int per[3];
  double cutneighsq[ORC_MAXTYPE + 1][ORC_MAXTYPE + 1];
  double cutghost;
  double *xhold;      /* owned positions at the last build */
  int64_t *nb_off;    /* nlocal+1 */
  int *nb;
  int64_t nb_cap;
  int ilp_num[1];     /* placeholder so the struct is never empty */
  int *ilpn;          /* nlocal */
  int *ilpnb;         /* nlocal*3 */
  double *normal;     /* nlocal*3 */
  double *dnormdri;   /* nlocal*9   [id*3+ip]   d n[id] / d x_i[ip] */
  double *dnormal;    /* nlocal*27  [(m*3+id)*3+ip] d n[id] / d x_m[ip] */
  double *fthr;       /* nthreads * nall*3 (Tersoff) then ILP */
  double *ethr;       /* nthreads * nall */
  double *vthr;       /* nthreads * nall*6 (per-atom virial) */
  int64_t nrebuild;
  int have_lists;
  char err[256];
};

orc_ctx *orc_new(const orc_pot *p, int nthreads) {
  orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  c->p = *p;
  c->nthreads = nthreads > 0 ? nthreads : 1;
  double cf = 0.0;
  for (int i = 1; i <= p->ntypes; i++)
    for (int j = 1; j <= p->ntypes; j++) {
      double cut = 0.0;
      if (p->i_enabled && p->i_map[i] >= 0 && p->i_map[j] >= 0) cut = p->cut_global;
      if (p->t_enabled && p->t_map[i] >= 0 && p->t_map[j] >= 0 && p->t_cutmax > cut) cut = p->t_cutmax;
      double cn = cut > 0.0 ? cut + p->skin : 0.0;
      c->cutneighsq[i][j] = cn * cn;
      if (cn > cf) cf = cn;
    }
  c->cutghost = cf;
  return c;
}

void orc_free(orc_ctx *c) {
  if (!c) return;
  free(c->x); free(c->type); free(c->mol); free(c->tag); free(c->owner); free(c->shift);
  free(c->xhold); free(c->nb_off); free(c->nb); free(c->ilpn); free(c->ilpnb);
  free(c->normal); free(c->dnormdri); free(c->dnormal); free(c->fthr); free(c->ethr); free(c->vthr);
  free(c);
}

const char *orc_error(const orc_ctx *c) { return c->err; }
int64_t orc_nrebuilds(const orc_ctx *c) { return c->nrebuild; }

static void grow_atoms(orc_ctx *c, int n) {
  if (n <= c->cap_all) return;
  int cap = n + n / 4 + 16;
  c->x = (double *)realloc(c->x, sizeof(double) * 3 * cap);
  c->type = (int *)realloc(c->type, sizeof(int) * cap);
  c->mol = (int64_t *)realloc(c->mol, sizeof(int64_t) * cap);
  c->tag = (int64_t *)realloc(c->tag, sizeof(int64_t) * cap);
  c->owner = (int *)realloc(c->owner, sizeof(int) * cap);
  c->shift = (int *)realloc(c->shift, sizeof(int) * 3 * cap);
  c->cap_all = cap;
}

/* ghost images within cutghost of the box, built like comm_brick borders: each
 * periodic image coordinate is produced by repeated +/- box-length additions. */
static double image_coord(double x, int s, double L) {
  double v = x;
  if (s > 0)
    for (int k = 0; k < s; k++) v = v + L;
  else
    for (int k = 0; k < -s; k++) v = v - L;
  return v;
}

static void make_ghosts(orc_ctx *c) {
  double L[3];
  int R[3];
  for (int d = 0; d < 3; d++) {
    L[d] = c->hi[d] - c->lo[d];
    R[d] = c->per[d] ? (int)ceil(c->cutghost / L[d]) : 0;
  }
  int n = c->nlocal;
  int nall = n;
  for (int sz = -R[2]; sz <= R[2]; sz++)
    for (int sy = -R[1]; sy <= R[1]; sy++)
      for (int sx = -R[0]; sx <= R[0]; sx++) {
        if (!sx && !sy && !sz) continue;
        int s[3] = {sx, sy, sz};
        for (int i = 0; i < n; i++) {
          double xi[3];
          int ok = 1;
          for (int d = 0; d < 3; d++) {
            xi[d] = image_coord(c->x[3 * i + d], s[d], L[d]);
            if (c->per[d] && (xi[d] < c->lo[d] - c->cutghost || xi[d] > c->hi[d] + c->cutghost)) ok = 0;
          }
          if (!ok) continue;
          grow_atoms(c, nall + 1);
          for (int d = 0; d < 3; d++) {
            c->x[3 * nall + d] = xi[d];
            c->shift[3 * nall + d] = s[d];
          }
          c->type[nall] = c->type[i];
          c->mol[nall] = c->mol[i];
          c->tag[nall] = c->tag[i];
          c->owner[nall] = i;
          nall++;
        }
      }
  c->nall = nall;
}

static void refresh_ghosts(orc_ctx *c) {
  double L[3];
  for (int d = 0; d < 3; d++) L[d] = c->hi[d] - c->lo[d];
  for (int g = c->nlocal; g < c->nall; g++) {
    int o = c->owner[g];
    for (int d = 0; d < 3; d++) c->x[3 * g + d] = image_coord(c->x[3 * o + d], c->shift[3 * g + d], L[d]);
  }
}

/* binned full list for owned atoms over owned+ghost (npair_full_bin_ghost.cpp:75-117) */
static int build_list(orc_ctx *c) {
  double bmin[3], bmax[3];
  for (int d = 0; d < 3; d++) {
    bmin[d] = 1e300;
    bmax[d] = -1e300;
  }
  for (int a = 0; a < c->nall; a++)
    for (int d = 0; d < 3; d++) {
      double v = c->x[3 * a + d];
      if (v < bmin[d]) bmin[d] = v;
      if (v > bmax[d]) bmax[d] = v;
    }
  double bs = 0.5 * c->cutghost;
  if (bs <= 0.0) bs = 1.0;
  int nb[3];
  for (int d = 0; d < 3; d++) {
    nb[d] = (int)((bmax[d] - bmin[d]) / bs) + 1;
    if (nb[d] < 1) nb[d] = 1;
  }
  int64_t nbins = (int64_t)nb[0] * nb[1] * nb[2];
  int *head = (int *)malloc(sizeof(int) * nbins);
  int *next = (int *)malloc(sizeof(int) * c->nall);
  int *abin = (int *)malloc(sizeof(int) * 3 * c->nall);
  for (int64_t b = 0; b < nbins; b++) head[b] = -1;
  for (int a = c->nall - 1; a >= 0; a--) {
    int ib[3];
    for (int d = 0; d < 3; d++) {
      ib[d] = (int)((c->x[3 * a + d] - bmin[d]) / bs);
      if (ib[d] >= nb[d]) ib[d] = nb[d] - 1;
      abin[3 * a + d] = ib[d];
    }
    int64_t b = ((int64_t)ib[2] * nb[1] + ib[1]) * nb[0] + ib[0];
    next[a] = head[b];
    head[b] = a;
  }
  int sr = 2;  /* stencil reach in bins: bin size = cutghost/2 */
  int nlocal = c->nlocal;
  c->nb_off = (int64_t *)realloc(c->nb_off, sizeof(int64_t) * (nlocal + 1));
  int64_t *cnt = (int64_t *)calloc(nlocal, sizeof(int64_t));
  /* pass 1 counts, pass 2 fills: keeps the list order identical in both passes */
  for (int pass = 0; pass < 2; pass++) {
    if (pass == 1) {
      c->nb_off[0] = 0;
      for (int i = 0; i < nlocal; i++) c->nb_off[i + 1] = c->nb_off[i] + cnt[i];
      int64_t total = c->nb_off[nlocal];
      if (total > c->nb_cap) {
        c->nb_cap = total + total / 8 + 16;
        c->nb = (int *)realloc(c->nb, sizeof(int) * c->nb_cap);
      }
    }
#pragma omp parallel for schedule(dynamic, 64) num_threads(c->nthreads)
    for (int i = 0; i < nlocal; i++) {
      double xtmp = c->x[3 * i], ytmp = c->x[3 * i + 1], ztmp = c->x[3 * i + 2];
      int itype = c->type[i];
      int64_t n = 0;
      int64_t base = pass ? c->nb_off[i] : 0;
      for (int dz = -sr; dz <= sr; dz++) {
        int bz = abin[3 * i + 2] + dz;
        if (bz < 0 || bz >= nb[2]) continue;
        for (int dy = -sr; dy <= sr; dy++) {
          int by = abin[3 * i + 1] + dy;
          if (by < 0 || by >= nb[1]) continue;
          for (int dx = -sr; dx <= sr; dx++) {
            int bx = abin[3 * i] + dx;
            if (bx < 0 || bx >= nb[0]) continue;
            for (int j = head[((int64_t)bz * nb[1] + by) * nb[0] + bx]; j >= 0; j = next[j]) {
              if (i == j) continue;
              double delx = xtmp - c->x[3 * j];
              double dely = ytmp - c->x[3 * j + 1];
              double delz = ztmp - c->x[3 * j + 2];
              double rsq = delx * delx + dely * dely + delz * delz;
              if (rsq <= c->cutneighsq[itype][c->type[j]]) {
                if (pass) c->nb[base + n] = j;
                n++;
              }
            }
          }
        }
      }
      if (!pass) cnt[i] = n;
    }
  }
  free(cnt);
  free(head);
  free(next);
  free(abin);
  c->have_lists = 1;
  c->nrebuild++;
  return 0;
}

static void wrap_owned(orc_ctx *c) {
  for (int i = 0; i < c->nlocal; i++)
    for (int d = 0; d < 3; d++) {
      if (!c->per[d]) continue;
      double L = c->hi[d] - c->lo[d];
      double v = c->x[3 * i + d];
      while (v < c->lo[d]) v += L;
      while (v >= c->hi[d]) v -= L;
      c->x[3 * i + d] = v;
    }
}

static int rebuild(orc_ctx *c) {
  wrap_owned(c);
  make_ghosts(c);
  c->xhold = (double *)realloc(c->xhold, sizeof(double) * 3 * c->nlocal);
  memcpy(c->xhold, c->x, sizeof(double) * 3 * c->nlocal);
  return build_list(c);
}

int orc_set_atoms(orc_ctx *c, int n, const double *x, const int *type, const int64_t *mol,
                  const int64_t *tag, const double lo[3], const double hi[3], const int periodic[3]) {
  c->nlocal = n;
  c->nall = n;
  grow_atoms(c, n);
  memcpy(c->x, x, sizeof(double) * 3 * n);
  for (int i = 0; i < n; i++) {
    if (type[i] < 1 || type[i] > c->p.ntypes) {
      snprintf(c->err, sizeof c->err, "atom type out of range");
      return -1;
    }
    c->type[i] = type[i];
    c->mol[i] = mol ? mol[i] : 0;
    c->tag[i] = tag ? tag[i] : i + 1;
    c->owner[i] = i;
    c->shift[3 * i] = c->shift[3 * i + 1] = c->shift[3 * i + 2] = 0;
  }
  for (int d = 0; d < 3; d++) {
    c->lo[d] = lo[d];
    c->hi[d] = hi[d];
    c->per[d] = periodic[d];
  }
  c->ilpn = (int *)realloc(c->ilpn, sizeof(int) * n);
  c->ilpnb = (int *)realloc(c->ilpnb, sizeof(int) * 3 * n);
  c->normal = (double *)realloc(c->normal, sizeof(double) * 3 * n);
  c->dnormdri = (double *)realloc(c->dnormdri, sizeof(double) * 9 * n);
  c->dnormal = (double *)realloc(c->dnormal, sizeof(double) * 27 * n);
  return rebuild(c);
}

int orc_update_x(orc_ctx *c, const double *x) {
  double trig = 0.25 * c->p.skin * c->p.skin;  /* (skin/2)^2, neighbor.cpp:1947-1976 */
  int need = 0;
  for (int i = 0; i < c->nlocal && !need; i++) {
    double dx = x[3 * i] - c->xhold[3 * i], dy = x[3 * i + 1] - c->xhold[3 * i + 1],
           dz = x[3 * i + 2] - c->xhold[3 * i + 2];
    if (dx * dx + dy * dy + dz * dz > trig) need = 1;
  }
  memcpy(c->x, x, sizeof(double) * 3 * c->nlocal);
  if (need) return rebuild(c);
  refresh_ghosts(c);
  return 0;
}

/* ======================================================================= ILP == */

/* ILP_neigh, pair_ilp_graphene_hbn.cpp:710-744 (owned atoms) */
static int ilp_neigh(orc_ctx *c) {
  const orc_pot *p = &c->p;
  int bad = 0;
  for (int i = 0; i < c->nlocal; i++) {
    int n = 0;
    int ie = p->i_map[c->type[i]];
    c->ilpn[i] = 0;
    if (ie < 0) continue;
    double xtmp = c->x[3 * i], ytmp = c->x[3 * i + 1], ztmp = c->x[3 * i + 2];
    for (int64_t jj = c->nb_off[i]; jj < c->nb_off[i + 1]; jj++) {
      int j = c->nb[jj];
      int je = p->i_map[c->type[j]];
      if (je < 0) continue;
      double delx = xtmp - c->x[3 * j];
      double dely = ytmp - c->x[3 * j + 1];
      double delz = ztmp - c->x[3 * j + 2];
      double rsq = delx * delx + dely * dely + delz * delz;
      if (rsq != 0 && rsq < p->i_cutILPsq[ie][je] && c->mol[i] == c->mol[j]) {
        if (n < 3) c->ilpnb[3 * i + n] = j;
        n++;
      }
    }
    c->ilpn[i] = n < 3 ? n : 3;
    if (n > 3) bad = 1;
  }
  if (bad) {
    snprintf(c->err, sizeof c->err,
             "There are too many neighbors for some atoms, please check your configuration");
    return -3;
  }
  return 0;
}

/* [u]x : the matrix with [u]x v = u x v */
static void skew(const double u[3], double m[3][3]) {
  m[0][0] = 0.0;   m[0][1] = -u[2]; m[0][2] = u[1];
  m[1][0] = u[2];  m[1][1] = 0.0;   m[1][2] = -u[0];
  m[2][0] = -u[1]; m[2][1] = u[0];  m[2][2] = 0.0;
}

static void cross(const double a[3], const double b[3], double o[3]) {
  o[0] = a[1] * b[2] - b[1] * a[2];
  o[1] = a[2] * b[0] - b[2] * a[0];
  o[2] = a[0] * b[1] - b[0] * a[1];
}

/* calc_normal, pair_ilp_graphene_hbn.cpp:776-1074: unit normal of atom i from its
 * <= 3 intralayer neighbours and its Jacobians w.r.t. x_i and each neighbour.
 * The derivative of a x b is -[b]x w.r.t. a and [a]x w.r.t. b; the unit vector's
 * derivative is (I - n n^T) dn1 / |n1|, the same expression as :893-926 / :1043-1067. */
static int calc_normal(orc_ctx *c) {
  int bad = 0;
  ORC_OPCAT(ORC_CAT_NORMAL);
  for (int i = 0; i < c->nlocal; i++) {
    if (c->p.i_map[c->type[i]] >= 0) ORC_OPUNIT(ORC_CAT_NORMAL);
    double *nrm = &c->normal[3 * i];
    double *dri = &c->dnormdri[9 * i];
    double *dk = &c->dnormal[27 * i];
    memset(dri, 0, sizeof(double) * 9);
    memset(dk, 0, sizeof(double) * 27);
    int cont = c->ilpn[i];
    if (c->p.i_map[c->type[i]] < 0) cont = 0;
    double vet[3][3];
    for (int m = 0; m < cont; m++) {
      int j = c->ilpnb[3 * i + m];
      for (int d = 0; d < 3; d++) vet[m][d] = c->x[3 * j + d] - c->x[3 * i + d];
    }
    if (cont <= 1) {
      nrm[0] = 0.0; nrm[1] = 0.0; nrm[2] = 1.0;
      continue;
    }
    double n1[3], dn1[3][3][3], dn1i[3][3];   /* dn1[m][id][ip] */
    memset(dn1, 0, sizeof dn1);
    memset(dn1i, 0, sizeof dn1i);
    if (cont == 2) {
      double s0[3][3], s1[3][3];
      cross(vet[0], vet[1], n1);
      skew(vet[1], s1);
      skew(vet[0], s0);
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
          dn1[0][a][b] = -s1[a][b];
          dn1[1][a][b] = s0[a][b];
          dn1i[a][b] = s1[a][b] - s0[a][b];     /* = -(dn1/dv1 + dn1/dv2) */
        }
    } else {
      double p12[3], p31[3], p23[3];
      cross(vet[0], vet[1], p12);
      cross(vet[2], vet[0], p31);
      cross(vet[1], vet[2], p23);
      double s0[3][3], s1[3][3], s2[3][3];
      skew(vet[0], s0);
      skew(vet[1], s1);
      skew(vet[2], s2);
      for (int a = 0; a < 3; a++) {
        n1[a] = (p12[a] + p31[a] + p23[a]) / cont;
        for (int b = 0; b < 3; b++) {
          /* d/dv1: p12 -> -[v2], p31 -> [v3];  d/dv2: p12 -> [v1], p23 -> -[v3];
             d/dv3: p31 -> -[v1], p23 -> [v2] */
          dn1[0][a][b] = (-s1[a][b] + s2[a][b]) / cont;
          dn1[1][a][b] = (s0[a][b] - s2[a][b]) / cont;
          dn1[2][a][b] = (-s0[a][b] + s1[a][b]) / cont;
        }
      }
      /* dn1/dx_i vanishes identically for three neighbours (:1036-1041) */
    }
    double nn2 = n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2];
    double nn = sqrt(nn2);
    if (nn == 0) {
      bad = 1;
      nrm[0] = 0.0; nrm[1] = 0.0; nrm[2] = 1.0;
      continue;
    }
    for (int a = 0; a < 3; a++) nrm[a] = n1[a] / nn;
    /* Jacobian of the unit vector: dn1/nn - n1 (n1 . dn1)/nn^3 */
    for (int m = 0; m < cont; m++)
      for (int ip = 0; ip < 3; ip++) {
        double dnn = (n1[0] * dn1[m][0][ip] + n1[1] * dn1[m][1][ip] + n1[2] * dn1[m][2][ip]) / nn;
        for (int id = 0; id < 3; id++) dk[(m * 3 + id) * 3 + ip] = dn1[m][id][ip] / nn - n1[id] * dnn / nn2;
      }
    if (cont == 2)
      for (int ip = 0; ip < 3; ip++) {
        double dni = (n1[0] * dn1i[0][ip] + n1[1] * dn1i[1][ip] + n1[2] * dn1i[2][ip]) / nn;
        for (int id = 0; id < 3; id++) dri[id * 3 + ip] = dn1i[id][ip] / nn - n1[id] * dni / nn2;
      }
  }
  ORC_OPCAT(ORC_CAT_OTHER);
  if (bad) {
    snprintf(c->err, sizeof c->err, "The magnitude of the normal vector is zero");
    return -4;
  }
  return 0;
}

/* taper, pair_ilp_graphene_hbn.h:80-115 */
static inline double calc_Tap(double r_ij, double Rcut) {
  static const double Tap_coeff[8] = {1.0, 0.0, 0.0, 0.0, -35.0, 84.0, -70.0, 20.0};
  double r = r_ij / Rcut;
  if (r >= 1.0) return 0.0;
  double Tap = Tap_coeff[7] * r + Tap_coeff[6];
  Tap = Tap * r + Tap_coeff[5];
  Tap = Tap * r + Tap_coeff[4];
  Tap = Tap * r + Tap_coeff[3];
  Tap = Tap * r + Tap_coeff[2];
  Tap = Tap * r + Tap_coeff[1];
  Tap = Tap * r + Tap_coeff[0];
  return Tap;
}

static inline double calc_dTap(double r_ij, double Rcut) {
  static const double Tap_coeff[8] = {1.0, 0.0, 0.0, 0.0, -35.0, 84.0, -70.0, 20.0};
  double r = r_ij / Rcut;
  if (r >= 1.0) return 0.0;
  double dTap = 7.0 * Tap_coeff[7] * r + 6.0 * Tap_coeff[6];
  dTap = dTap * r + 5.0 * Tap_coeff[5];
  dTap = dTap * r + 4.0 * Tap_coeff[4];
  dTap = dTap * r + 3.0 * Tap_coeff[3];
  dTap = dTap * r + 2.0 * Tap_coeff[2];
  dTap = dTap * r + Tap_coeff[1];
  return dTap / Rcut;
}

/* half-list selection of a full list by tag parity, pair_ilp_graphene_hbn.cpp:488-496
 * (identical in pair_tersoff.cpp:150-158); returns 1 when (i,j) is skipped */
static inline int skip_half(const orc_ctx *c, int i, int j) {
  int64_t itag = c->tag[i], jtag = c->tag[j];
  if (itag > jtag) {
    if ((itag + jtag) % 2 == 0) return 1;
  } else if (itag < jtag) {
    if ((itag + jtag) % 2 == 1) return 1;
  } else {
    if (c->x[3 * j + 2] < c->x[3 * i + 2]) return 1;
    if (c->x[3 * j + 2] == c->x[3 * i + 2] && c->x[3 * j + 1] < c->x[3 * i + 1]) return 1;
    if (c->x[3 * j + 2] == c->x[3 * i + 2] && c->x[3 * j + 1] == c->x[3 * i + 1] &&
        c->x[3 * j] < c->x[3 * i])
      return 1;
  }
  return 0;
}

/* Per-atom virial tallies (pair.cpp): ev_tally (:913-1058) with a scalar pair force
 * fpair along del, ev_tally_xyz (:1060-1153) with a force vector, each half to both
 * atoms with newton on; v_tally3 (:1435-1453) a third to each of three atoms. */
static inline void va_pair(double *va, int i, int j, double fpair, double dx, double dy, double dz) {
  double v[6] = {dx * dx * fpair, dy * dy * fpair, dz * dz * fpair,
                 dx * dy * fpair, dx * dz * fpair, dy * dz * fpair};
  for (int c = 0; c < 6; c++) va[6 * i + c] += 0.5 * v[c];
  for (int c = 0; c < 6; c++) va[6 * j + c] += 0.5 * v[c];
}
static inline void va_xyz(double *va, int i, int j, const double fv[3], double dx, double dy, double dz) {
  double v[6] = {dx * fv[0], dy * fv[1], dz * fv[2], dx * fv[1], dx * fv[2], dy * fv[2]};
  for (int c = 0; c < 6; c++) va[6 * i + c] += 0.5 * v[c];
  for (int c = 0; c < 6; c++) va[6 * j + c] += 0.5 * v[c];
}
static inline void va_three(double *va, int i, int j, int k, const double fj[3], const double fk[3],
                            const double drij[3], const double drik[3]) {
  const double third = 1.0 / 3.0;
  double v[6] = {third * (drij[0] * fj[0] + drik[0] * fk[0]), third * (drij[1] * fj[1] + drik[1] * fk[1]),
                 third * (drij[2] * fj[2] + drik[2] * fk[2]), third * (drij[0] * fj[1] + drik[0] * fk[1]),
                 third * (drij[0] * fj[2] + drik[0] * fk[2]), third * (drij[1] * fj[2] + drik[1] * fk[2])};
  for (int c = 0; c < 6; c++) {
    va[6 * i + c] += v[c];
    va[6 * j + c] += v[c];
    va[6 * k + c] += v[c];
  }
}

/* calc_FvdW (:471-540) and calc_FRep (:577-674) for owned atom i; vatom (nall*6, may be
 * NULL) receives the per-atom virial as the reference tallies it: ev_tally of the vdW
 * pair (:536), ev_tally_xyz of each normal-derivative force on k against x_k - x_j
 * (:667) and of the repulsion's pair force (:671) */
static void ilp_atom(const orc_ctx *c, int i, double *f, double *eatom, double *vatom, double *evdw,
                     double *erep) {
  const orc_pot *p = &c->p;
  int ie = p->i_map[c->type[i]];
  if (ie < 0) return;
  double xtmp = c->x[3 * i], ytmp = c->x[3 * i + 1], ztmp = c->x[3 * i + 2];
  double cutsq = p->cut_global * p->cut_global;
  double Rcut = sqrt(cutsq);
  const double *nrm = &c->normal[3 * i];
  const double *dri = &c->dnormdri[9 * i];
  const double *dk = &c->dnormal[27 * i];
  for (int64_t jj = c->nb_off[i]; jj < c->nb_off[i + 1]; jj++) {
    int j = c->nb[jj];
    int je = p->i_map[c->type[j]];
    if (je < 0) continue;
    if (c->mol[i] == c->mol[j]) continue;
    ORC_OPCAT(ORC_CAT_ILP_CAND);
    ORC_OPUNIT(ORC_CAT_ILP_CAND);
    double delx = xtmp - c->x[3 * j];
    double dely = ytmp - c->x[3 * j + 1];
    double delz = ztmp - c->x[3 * j + 2];
    double rsq = delx * delx + dely * dely + delz * delz;
    if (rsq >= cutsq) continue;
    ORC_OPCAT(ORC_CAT_ILP_PAIR);
    ORC_OPUNIT(ORC_CAT_ILP_PAIR);
    const orc_ilp_param *q = &p->i_params[p->i_e2p[ie][je]];
    double r = sqrt(rsq);
    double Tap, dTap;
    if (p->tap_flag) {
      Tap = calc_Tap(r, Rcut);
      dTap = calc_dTap(r, Rcut);
    } else {
      Tap = 1.0;
      dTap = 0.0;
    }
    /* van der Waals, half of the pairs */
    if (!skip_half(c, i, j)) {
      ORC_OPCAT(ORC_CAT_ILP_VDW);
      ORC_OPUNIT(ORC_CAT_ILP_VDW);
      double r2inv = 1.0 / rsq;
      double r6inv = r2inv * r2inv * r2inv;
      double r8inv = r6inv * r2inv;
      double Vilp, fpair;
      if (p->i_model == 1) {
        /* pair_kolmogorov_crespi_full.cpp:522-526 */
        Vilp = -q->A * q->z06 * r6inv;
        fpair = -6.0 * q->A * q->z06 * r8inv;
      } else {
        double TSvdw = 1.0 + exp(-q->d * (r / q->seff - 1.0));
        double TSvdw2inv = pow(TSvdw, -2.0);
        Vilp = -q->C6 * r6inv / TSvdw;
        fpair = -6.0 * q->C6 * r8inv / TSvdw + q->C6 * q->d / q->seff * (TSvdw - 1.0) * TSvdw2inv * r8inv * r;
      }
      double fsum = fpair * Tap - Vilp * dTap / r;
      f[3 * i] += fsum * delx;
      f[3 * i + 1] += fsum * dely;
      f[3 * i + 2] += fsum * delz;
      f[3 * j] -= fsum * delx;
      f[3 * j + 1] -= fsum * dely;
      f[3 * j + 2] -= fsum * delz;
      double evdwl = Vilp * Tap;
      *evdw += evdwl;
      if (eatom) {
        eatom[i] += 0.5 * evdwl;
        eatom[j] += 0.5 * evdwl;
      }
      if (vatom) va_pair(vatom, i, j, fsum, delx, dely, delz);
      ORC_OPCAT(ORC_CAT_ILP_PAIR);
    }
    /* repulsion with the normal of i, every directed pair */
    double prodnorm1 = nrm[0] * delx + nrm[1] * dely + nrm[2] * delz;
    double rhosq1 = rsq - prodnorm1 * prodnorm1;
    double rdsq1 = rhosq1 * q->delta2inv;
    double exp0 = exp(-q->lambda * (r - q->z0));
    double exp1 = exp(-rdsq1);
    double Vilp, fpair, fpair1;
    if (p->i_model == 1) {
      /* pair_kolmogorov_crespi_full.cpp:615-631 */
      double sumC1 = q->C0 + q->C2 * rdsq1 + q->C4 * rdsq1 * rdsq1;
      double sumC11 = (q->C2 + 2.0 * q->C4 * rdsq1) * q->delta2inv;
      double frho_ij = exp1 * sumC1;
      double sumCff = 0.5 * q->C + frho_ij;
      Vilp = exp0 * sumCff;
      fpair = q->lambda * exp0 / r * sumCff;
      fpair1 = 2.0 * exp0 * exp1 * (q->delta2inv * sumC1 - sumC11);
    } else {
      double frho1 = exp1 * q->C;
      double Erep = 0.5 * q->epsilon + frho1;
      Vilp = exp0 * Erep;
      fpair = q->lambda * exp0 / r * Erep;
      fpair1 = 2.0 * exp0 * frho1 * q->delta2inv;
    }
    double fsum = fpair + fpair1;
    double del[3] = {delx, dely, delz};
    double fkc[3];
    for (int a = 0; a < 3; a++) {
      double fp1 = prodnorm1 * nrm[a] * fpair1;
      fkc[a] = (del[a] * fsum - fp1) * Tap - Vilp * dTap * del[a] / r;
      f[3 * j + a] -= fkc[a];
    }
    /* the term of dn_i/dx_i (a k-term with k = i) */
    ORC_OPCAT(ORC_CAT_ILP_DSELF);
    ORC_OPUNIT(ORC_CAT_ILP_DSELF);
    double dprod[3], fi[3];
    for (int ip = 0; ip < 3; ip++)
      dprod[ip] = dri[0 * 3 + ip] * delx + dri[1 * 3 + ip] * dely + dri[2 * 3 + ip] * delz;
    for (int a = 0; a < 3; a++) {
      double fprod1 = prodnorm1 * dprod[a] * fpair1;
      fi[a] = fkc[a] - fprod1 * Tap;
    }
    ORC_OPCAT(ORC_CAT_ILP_PAIR);
    for (int a = 0; a < 3; a++) f[3 * i + a] += fi[a];
    for (int kk = 0; kk < c->ilpn[i]; kk++) {
      int k = c->ilpnb[3 * i + kk];
      if (k == i) continue;
      ORC_OPCAT(ORC_CAT_ILP_KTERM);
      ORC_OPUNIT(ORC_CAT_ILP_KTERM);
      double fk[3];
      for (int ip = 0; ip < 3; ip++) {
        double dp = dk[(kk * 3 + 0) * 3 + ip] * delx + dk[(kk * 3 + 1) * 3 + ip] * dely +
                    dk[(kk * 3 + 2) * 3 + ip] * delz;
        fk[ip] = (-prodnorm1 * dp * fpair1) * Tap;
        f[3 * k + ip] += fk[ip];
      }
      if (vatom)
        va_xyz(vatom, k, j, fk, c->x[3 * k] - c->x[3 * j], c->x[3 * k + 1] - c->x[3 * j + 1],
               c->x[3 * k + 2] - c->x[3 * j + 2]);
      ORC_OPCAT(ORC_CAT_ILP_PAIR);
    }
    /* KC without the taper tallies V - offset, offset = -A (z0/cut)^6 (init_one :235) */
    double ev = (p->i_model == 1 && !p->tap_flag) ? Vilp + q->A * pow(q->z0 / p->cut_global, 6.0) : Tap * Vilp;
    *erep += ev;
    if (eatom) {
      eatom[i] += 0.5 * ev;
      eatom[j] += 0.5 * ev;
    }
    if (vatom) va_xyz(vatom, i, j, fkc, delx, dely, delz);
  }
  ORC_OPCAT(ORC_CAT_OTHER);
}

/* =================================================================== Tersoff == */

static inline double ters_fc(double r, const orc_ters_param *q) {
  if (r < q->bigr - q->bigd) return 1.0;
  if (r > q->bigr + q->bigd) return 0.0;
  return 0.5 * (1.0 - sin(MY_PI2 * (r - q->bigr) / q->bigd));
}
static inline double ters_fc_d(double r, const orc_ters_param *q) {
  if (r < q->bigr - q->bigd) return 0.0;
  if (r > q->bigr + q->bigd) return 0.0;
  return -(MY_PI4 / q->bigd) * cos(MY_PI2 * (r - q->bigr) / q->bigd);
}
static inline double ters_fa(double r, const orc_ters_param *q) {
  if (r > q->bigr + q->bigd) return 0.0;
  return -q->bigb * exp(-q->lam2 * r) * ters_fc(r, q);
}
static inline double ters_fa_d(double r, const orc_ters_param *q) {
  if (r > q->bigr + q->bigd) return 0.0;
  return q->bigb * exp(-q->lam2 * r) * (q->lam2 * ters_fc(r, q) - ters_fc_d(r, q));
}
static inline double ters_bij(double zeta, const orc_ters_param *q) {
  double tmp = q->beta * zeta;
  if (tmp > q->c1) return 1.0 / sqrt(tmp);
  if (tmp > q->c2) return (1.0 - pow(tmp, -q->powern) / (2.0 * q->powern)) / sqrt(tmp);
  if (tmp < q->c4) return 1.0;
  if (tmp < q->c3) return 1.0 - pow(tmp, q->powern) / (2.0 * q->powern);
  return pow(1.0 + pow(tmp, q->powern), -1.0 / (2.0 * q->powern));
}
static inline double ters_bij_d(double zeta, const orc_ters_param *q) {
  double tmp = q->beta * zeta;
  if (tmp > q->c1) return q->beta * -0.5 * pow(tmp, -1.5);
  if (tmp > q->c2)
    return q->beta * (-0.5 * pow(tmp, -1.5) * (1.0 - (1.0 + 1.0 / (2.0 * q->powern)) * pow(tmp, -q->powern)));
  if (tmp < q->c4) return 0.0;
  if (tmp < q->c3) return -0.5 * q->beta * pow(tmp, q->powern - 1.0);
  double tmp_n = pow(tmp, q->powern);
  return -0.5 * pow(1.0 + tmp_n, -1.0 - (1.0 / (2.0 * q->powern))) * tmp_n / zeta;
}
static inline double ters_gijk(double costheta, const orc_ters_param *q) {
  double tc = q->c * q->c, td = q->d * q->d, hcth = q->h - costheta;
  return q->gamma * (1.0 + tc / td - tc / (td + hcth * hcth));
}
static inline double ters_gijk_d(double costheta, const orc_ters_param *q) {
  double tc = q->c * q->c, td = q->d * q->d, hcth = q->h - costheta;
  double numerator = -2.0 * tc * hcth;
  double denominator = 1.0 / (td + hcth * hcth);
  return q->gamma * numerator * denominator * denominator;
}
static inline double ters_exdelr(const orc_ters_param *q, double rij, double rik) {
  double arg = q->powermint == 3 ? pow(q->lam3 * (rij - rik), 3) : q->lam3 * (rij - rik);
  if (arg > 69.0776) return 1.e30;
  if (arg < -69.0776) return 0.0;
  return exp(arg);
}

/* zeta, pair_tersoff.cpp:599-617 */
static double ters_zeta(const orc_ters_param *q, double rsqij, double rsqik, const double *dij, const double *dik) {
  double rij = sqrt(rsqij), rik = sqrt(rsqik);
  double costheta = (dij[0] * dik[0] + dij[1] * dik[1] + dij[2] * dik[2]) / (rij * rik);
  return ters_fc(rik, q) * ters_gijk(costheta, q) * ters_exdelr(q, rij, rik);
}

/* attractive -> ters_zetaterm_d -> costheta_d, pair_tersoff.cpp:642-659,738-811 */
static void ters_attractive(const orc_ters_param *q, double prefactor, double rsqij, double rsqik,
                            const double *dij, const double *dik, double *fi, double *fj, double *fk) {
  double rij = sqrt(rsqij), rik = sqrt(rsqik);
  double rijinv = 1.0 / rij, rikinv = 1.0 / rik;
  double rh[3], kh[3];
  for (int a = 0; a < 3; a++) {
    rh[a] = dij[a] * rijinv;
    kh[a] = dik[a] * rikinv;
  }
  double fc = ters_fc(rik, q), dfc = ters_fc_d(rik, q);
  double ex_delr = ters_exdelr(q, rij, rik);
  double ex_delr_d = q->powermint == 3 ? 3.0 * pow(q->lam3, 3) * (rij - rik) * (rij - rik) * ex_delr
                                       : q->lam3 * ex_delr;
  double cos_theta = rh[0] * kh[0] + rh[1] * kh[1] + rh[2] * kh[2];
  double gijk = ters_gijk(cos_theta, q), gijk_d = ters_gijk_d(cos_theta, q);
  double dcj[3], dck[3], dci[3];
  for (int a = 0; a < 3; a++) {
    dcj[a] = (-cos_theta * rh[a] + kh[a]) / rij;
    dck[a] = (-cos_theta * kh[a] + rh[a]) / rik;
    dci[a] = -(dcj[a] + dck[a]);
  }
  for (int a = 0; a < 3; a++) {
    double v = -dfc * gijk * ex_delr * kh[a];
    v += fc * gijk_d * ex_delr * dci[a];
    v += fc * gijk * ex_delr_d * kh[a];
    v += -fc * gijk * ex_delr_d * rh[a];
    fi[a] = prefactor * v;
    double w = fc * gijk_d * ex_delr * dcj[a];
    w += fc * gijk * ex_delr_d * rh[a];
    fj[a] = prefactor * w;
    double u = dfc * gijk * ex_delr * kh[a];
    u += fc * gijk_d * ex_delr * dck[a];
    u += -fc * gijk * ex_delr_d * kh[a];
    fk[a] = prefactor * u;
  }
}

/* PairTersoff::compute body for owned atom i, pair_tersoff.cpp:117-262; vatom (nall*6,
 * may be NULL) receives the per-atom virial of its ev_tally (:173, :223) and v_tally3
 * (:253) calls */
static int tersoff_atom(const orc_ctx *c, int i, double *f, double *eatom, double *vatom, double *eng) {
  const orc_pot *p = &c->p;
  int itype = p->t_map[c->type[i]];
  if (itype < 0) return 0;
  double xtmp = c->x[3 * i], ytmp = c->x[3 * i + 1], ztmp = c->x[3 * i + 2];
  double cutshortsq = p->t_cutmax * p->t_cutmax;
  int neighshort[MAXSHORT];
  int numshort = 0;
  double fxtmp = 0.0, fytmp = 0.0, fztmp = 0.0;
  for (int64_t jj = c->nb_off[i]; jj < c->nb_off[i + 1]; jj++) {
    int j = c->nb[jj];
    int jtype = p->t_map[c->type[j]];
    if (jtype < 0) continue;
    ORC_OPCAT(ORC_CAT_TERS_CAND);
    ORC_OPUNIT(ORC_CAT_TERS_CAND);
    double delx = xtmp - c->x[3 * j];
    double dely = ytmp - c->x[3 * j + 1];
    double delz = ztmp - c->x[3 * j + 2];
    double rsq = delx * delx + dely * dely + delz * delz;
    if (rsq < cutshortsq) {
      if (numshort >= MAXSHORT) return -2;
      neighshort[numshort++] = j;
    }
    if (skip_half(c, i, j)) continue;
    const orc_ters_param *q = &p->t_params[p->t_e2p[itype][jtype][jtype]];
    if (rsq >= q->cutsq) continue;
    /* repulsive, :584-595 */
    ORC_OPCAT(ORC_CAT_TERS_REP);
    ORC_OPUNIT(ORC_CAT_TERS_REP);
    double r = sqrt(rsq);
    double tmp_fc = ters_fc(r, q), tmp_fc_d = ters_fc_d(r, q);
    double tmp_exp = exp(-q->lam1 * r);
    double fpair = -q->biga * tmp_exp * (tmp_fc_d - tmp_fc * q->lam1) / r;
    double evdwl = tmp_fc * q->biga * tmp_exp;
    fxtmp += delx * fpair;
    fytmp += dely * fpair;
    fztmp += delz * fpair;
    f[3 * j] -= delx * fpair;
    f[3 * j + 1] -= dely * fpair;
    f[3 * j + 2] -= delz * fpair;
    *eng += evdwl;
    if (eatom) {
      eatom[i] += 0.5 * evdwl;
      eatom[j] += 0.5 * evdwl;
    }
    if (vatom) va_pair(vatom, i, j, fpair, delx, dely, delz);
  }
  for (int jj = 0; jj < numshort; jj++) {
    int j = neighshort[jj];
    int jtype = p->t_map[c->type[j]];
    const orc_ters_param *qij = &p->t_params[p->t_e2p[itype][jtype][jtype]];
    ORC_OPCAT(ORC_CAT_TERS_BOND);
    double delr1[3] = {c->x[3 * j] - xtmp, c->x[3 * j + 1] - ytmp, c->x[3 * j + 2] - ztmp};
    double rsq1 = delr1[0] * delr1[0] + delr1[1] * delr1[1] + delr1[2] * delr1[2];
    if (rsq1 >= qij->cutsq) continue;
    ORC_OPUNIT(ORC_CAT_TERS_BOND);
    double fjx = 0.0, fjy = 0.0, fjz = 0.0;
    double zeta_ij = 0.0;
    ORC_OPCAT(ORC_CAT_TERS_ZETA);
    for (int kk = 0; kk < numshort; kk++) {
      if (jj == kk) continue;
      int k = neighshort[kk];
      int ktype = p->t_map[c->type[k]];
      const orc_ters_param *qijk = &p->t_params[p->t_e2p[itype][jtype][ktype]];
      double delr2[3] = {c->x[3 * k] - xtmp, c->x[3 * k + 1] - ytmp, c->x[3 * k + 2] - ztmp};
      double rsq2 = delr2[0] * delr2[0] + delr2[1] * delr2[1] + delr2[2] * delr2[2];
      if (rsq2 >= qijk->cutsq) continue;
      ORC_OPUNIT(ORC_CAT_TERS_ZETA);
      zeta_ij += ters_zeta(qijk, rsq1, rsq2, delr1, delr2);
    }
    /* force_zeta, :621-634 */
    ORC_OPCAT(ORC_CAT_TERS_BOND);
    double r = sqrt(rsq1);
    double fa = ters_fa(r, qij), fa_d = ters_fa_d(r, qij);
    double bij = ters_bij(zeta_ij, qij);
    double fpair = 0.5 * bij * fa_d / r;
    double prefactor = -0.5 * fa * ters_bij_d(zeta_ij, qij);
    double evdwl = 0.5 * bij * fa;
    fxtmp += delr1[0] * fpair;
    fytmp += delr1[1] * fpair;
    fztmp += delr1[2] * fpair;
    fjx -= delr1[0] * fpair;
    fjy -= delr1[1] * fpair;
    fjz -= delr1[2] * fpair;
    *eng += evdwl;
    if (eatom) {
      eatom[i] += 0.5 * evdwl;
      eatom[j] += 0.5 * evdwl;
    }
    if (vatom) va_pair(vatom, i, j, -fpair, -delr1[0], -delr1[1], -delr1[2]);
    ORC_OPCAT(ORC_CAT_TERS_ATTR);
    for (int kk = 0; kk < numshort; kk++) {
      if (jj == kk) continue;
      int k = neighshort[kk];
      int ktype = p->t_map[c->type[k]];
      const orc_ters_param *qijk = &p->t_params[p->t_e2p[itype][jtype][ktype]];
      double delr2[3] = {c->x[3 * k] - xtmp, c->x[3 * k + 1] - ytmp, c->x[3 * k + 2] - ztmp};
      double rsq2 = delr2[0] * delr2[0] + delr2[1] * delr2[1] + delr2[2] * delr2[2];
      if (rsq2 >= qijk->cutsq) continue;
      ORC_OPUNIT(ORC_CAT_TERS_ATTR);
      double fi[3], fj[3], fk[3];
      ters_attractive(qijk, prefactor, rsq1, rsq2, delr1, delr2, fi, fj, fk);
      fxtmp += fi[0];
      fytmp += fi[1];
      fztmp += fi[2];
      fjx += fj[0];
      fjy += fj[1];
      fjz += fj[2];
      f[3 * k] += fk[0];
      f[3 * k + 1] += fk[1];
      f[3 * k + 2] += fk[2];
      if (vatom) va_three(vatom, i, j, k, fj, fk, delr1, delr2);
    }
    f[3 * j] += fjx;
    f[3 * j + 1] += fjy;
    f[3 * j + 2] += fjz;
  }
  ORC_OPCAT(ORC_CAT_TERS_BOND);
  f[3 * i] += fxtmp;
  f[3 * i + 1] += fytmp;
  f[3 * i + 2] += fztmp;
  ORC_OPCAT(ORC_CAT_OTHER);
  return 0;
}

/* ==================================================================== driver == */

static void fdotr(const orc_ctx *c, const double *f, double *v) {
  for (int a = 0; a < c->nall; a++) {
    const double *x = &c->x[3 * a];
    v[0] += f[3 * a] * x[0];
    v[1] += f[3 * a + 1] * x[1];
    v[2] += f[3 * a + 2] * x[2];
    v[3] += f[3 * a + 1] * x[0];
    v[4] += f[3 * a + 2] * x[0];
    v[5] += f[3 * a + 2] * x[1];
  }
}

static int style_pass(orc_ctx *c, int style, double *ftot, double *eatom, double *vatom, double *eng, double *pv,
                      double *vir) {
  int nall = c->nall, nt = c->nthreads;
  size_t fsz = (size_t)nall * 3, vsz = (size_t)nall * 6;
  c->fthr = (double *)realloc(c->fthr, sizeof(double) * fsz * nt);
  memset(c->fthr, 0, sizeof(double) * fsz * nt);
  if (eatom) {
    c->ethr = (double *)realloc(c->ethr, sizeof(double) * nall * nt);
    memset(c->ethr, 0, sizeof(double) * nall * nt);
  }
  if (vatom) {
    c->vthr = (double *)realloc(c->vthr, sizeof(double) * vsz * nt);
    memset(c->vthr, 0, sizeof(double) * vsz * nt);
  }
  double e0 = 0.0, e1 = 0.0;
  int err = 0;
#pragma omp parallel num_threads(nt) reduction(+ : e0, e1)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double *ft = c->fthr + fsz * tid;
    double *et = eatom ? c->ethr + (size_t)nall * tid : NULL;
    double *vt = vatom ? c->vthr + vsz * tid : NULL;
#pragma omp for schedule(dynamic, 32)
    for (int i = 0; i < c->nlocal; i++) {
      if (style == 1) {
        if (tersoff_atom(c, i, ft, et, vt, &e0)) err = 1;
      } else {
        ilp_atom(c, i, ft, et, vt, &e0, &e1);
      }
    }
  }
  if (err) {
    snprintf(c->err, sizeof c->err, "Tersoff short list overflow");
    return -2;
  }
  double *f = c->fthr;
  for (int t = 1; t < nt; t++)
    for (size_t k = 0; k < fsz; k++) f[k] += c->fthr[fsz * t + k];
  fdotr(c, f, vir);
  for (int a = 0; a < nall; a++) {
    int o = c->owner[a];
    for (int d = 0; d < 3; d++) ftot[3 * o + d] += f[3 * a + d];
    if (eatom) {
      double e = 0.0;
      for (int t = 0; t < nt; t++) e += c->ethr[(size_t)nall * t + a];
      eatom[o] += e;
    }
    if (vatom)
      for (int k = 0; k < 6; k++) {
        double v = 0.0;
        for (int t = 0; t < nt; t++) v += c->vthr[vsz * t + 6 * (size_t)a + k];
        vatom[6 * o + k] += v;
      }
  }
  if (style == 1) {
    *eng = e0;
  } else {
    pv[0] = e0;
    pv[1] = e1;
    *eng = e0 + e1;
  }
  return 0;
}

int orc_forces(orc_ctx *c, int which, double *f, double *eatom, orc_result *r) {
  return orc_forces_va(c, which, f, eatom, NULL, NULL, r);
}

int orc_forces_va(orc_ctx *c, int which, double *f, double *eatom, double *vatom_ters, double *vatom_ilp,
                  orc_result *r) {
  memset(r, 0, sizeof *r);
  memset(f, 0, sizeof(double) * 3 * c->nlocal);
  if (eatom) memset(eatom, 0, sizeof(double) * c->nlocal);
  if (vatom_ters) memset(vatom_ters, 0, sizeof(double) * 6 * c->nlocal);
  if (vatom_ilp) memset(vatom_ilp, 0, sizeof(double) * 6 * c->nlocal);
  int rc;
  if ((which & 1) && c->p.t_enabled) {
    rc = style_pass(c, 1, f, eatom, vatom_ters, &r->e_tersoff, NULL, r->virial_tersoff);
    if (rc) return rc;
  }
  if ((which & 2) && c->p.i_enabled) {
    if ((rc = ilp_neigh(c))) return rc;
    if ((rc = calc_normal(c))) return rc;
    rc = style_pass(c, 2, f, eatom, vatom_ilp, &r->e_ilp, r->pvector, r->virial_ilp);
    if (rc) return rc;
  }
  for (int k = 0; k < 6; k++) r->virial[k] = r->virial_tersoff[k] + r->virial_ilp[k];
  r->nghost = c->nall - c->nlocal;
  r->nlist = c->nb_off[c->nlocal];
  return 0;
}

int orc_nve(orc_ctx *c, int nsteps, double dt, const double *mass_of_type, double *x, double *v,
            double *f, orc_result *r) {
  const double ftm2v = 1.0 / 1.0364269e-4;
  double dtv = dt, dtf = 0.5 * dt * ftm2v;
  int n = c->nlocal;
  for (int s = 0; s < nsteps; s++) {
    for (int i = 0; i < n; i++) {
      double dtfm = dtf / mass_of_type[c->type[i] - 1];
      for (int d = 0; d < 3; d++) {
        v[3 * i + d] += dtfm * f[3 * i + d];
        x[3 * i + d] += dtv * v[3 * i + d];
      }
    }
    int rc = orc_update_x(c, x);
    if (rc) return rc;
    rc = orc_forces(c, 3, f, NULL, r);
    if (rc) return rc;
    for (int i = 0; i < n; i++) {
      double dtfm = dtf / mass_of_type[c->type[i] - 1];
      for (int d = 0; d < 3; d++) v[3 * i + d] += dtfm * f[3 * i + d];
    }
  }
  return 0;
}

/* ===================================================================== lists == */

static int64_t img_code(const orc_ctx *c, int j) {
  int64_t code = 0;
  for (int d = 0; d < 3; d++) code |= (int64_t)((c->shift[3 * j + d] + 8) & 15) << (4 * d);
  return code;
}

int64_t orc_full_list(orc_ctx *c, int64_t *out, int64_t cap) {
  int64_t n = 0;
  for (int i = 0; i < c->nlocal; i++)
    for (int64_t jj = c->nb_off[i]; jj < c->nb_off[i + 1]; jj++) {
      int j = c->nb[jj];
      if (out && n < cap) {
        out[3 * n] = c->tag[i];
        out[3 * n + 1] = c->tag[j];
        out[3 * n + 2] = img_code(c, j);
      }
      n++;
    }
  return n;
}

int64_t orc_ilp_list(orc_ctx *c, int64_t *out, int64_t cap) {
  if (ilp_neigh(c)) return -1;
  int64_t n = 0;
  for (int i = 0; i < c->nlocal; i++)
    for (int kk = 0; kk < c->ilpn[i]; kk++) {
      int j = c->ilpnb[3 * i + kk];
      if (out && n < cap) {
        out[3 * n] = c->tag[i];
        out[3 * n + 1] = c->tag[j];
        out[3 * n + 2] = img_code(c, j);
      }
      n++;
    }
  return n;
}
