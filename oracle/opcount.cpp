// Operation count of the oracle (TEST INFRASTRUCTURE, like the oracle itself): the
// oracle's C source (lmff_oracle.c) compiled as C++ with its floating-point type
// replaced by OpD, a double that counts the arithmetic done on it.  The categories and
// units are the markers ORC_OPCAT / ORC_OPUNIT in lmff_oracle.c.
//
// Counting convention (the one the benchmark's roofline uses): add, subtract, multiply,
// divide = 1; a*b + c = 2 (the oracle is compiled without contraction, so a fused
// multiply-add of the kernels counts the same 2); sqrt = 1; each call of exp, pow,
// sin, cos = 1 (its internals are not counted; they are tallied separately as
// "calls").  Negation, comparisons, conversions and loads are free.
//
// Built and run by oracle/opcount.py, which writes bench/flops.h.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static int g_cat = 0;
static uint64_t g_ops[16];
static uint64_t g_calls[16];
static uint64_t g_units[16];

struct OpD {
  double v;
  OpD() = default;
  constexpr OpD(double x) : v(x) {}
  explicit operator int() const { return (int)v; }
  explicit operator long() const { return (long)v; }
  explicit operator long long() const { return (long long)v; }
  explicit operator float() const { return (float)v; }
  explicit operator bool() const { return v != 0.0; }
};
static inline void tick() { g_ops[g_cat] += 1; }
static inline void call() {
  g_calls[g_cat] += 1;
  g_ops[g_cat] += 1;
}

static inline OpD operator+(OpD a, OpD b) { tick(); return OpD(a.v + b.v); }
static inline OpD operator-(OpD a, OpD b) { tick(); return OpD(a.v - b.v); }
static inline OpD operator*(OpD a, OpD b) { tick(); return OpD(a.v * b.v); }
static inline OpD operator/(OpD a, OpD b) { tick(); return OpD(a.v / b.v); }
static inline OpD operator-(OpD a) { return OpD(-a.v); }
static inline OpD operator+(OpD a) { return a; }
static inline OpD &operator+=(OpD &a, OpD b) { tick(); a.v += b.v; return a; }
static inline OpD &operator-=(OpD &a, OpD b) { tick(); a.v -= b.v; return a; }
static inline OpD &operator*=(OpD &a, OpD b) { tick(); a.v *= b.v; return a; }
static inline OpD &operator/=(OpD &a, OpD b) { tick(); a.v /= b.v; return a; }
static inline bool operator<(OpD a, OpD b) { return a.v < b.v; }
static inline bool operator>(OpD a, OpD b) { return a.v > b.v; }
static inline bool operator<=(OpD a, OpD b) { return a.v <= b.v; }
static inline bool operator>=(OpD a, OpD b) { return a.v >= b.v; }
static inline bool operator==(OpD a, OpD b) { return a.v == b.v; }
static inline bool operator!=(OpD a, OpD b) { return a.v != b.v; }
static inline bool operator!(OpD a) { return a.v == 0.0; }
// plain double (literals) and integer operands, counted like OpD ones
#define OPD_MIXED_OPS(T)                                                                 \
  static inline OpD operator+(OpD a, T b) { return a + OpD((double)b); }                \
  static inline OpD operator+(T a, OpD b) { return OpD((double)a) + b; }                \
  static inline OpD operator-(OpD a, T b) { return a - OpD((double)b); }                \
  static inline OpD operator-(T a, OpD b) { return OpD((double)a) - b; }                \
  static inline OpD operator*(OpD a, T b) { return a * OpD((double)b); }                \
  static inline OpD operator*(T a, OpD b) { return OpD((double)a) * b; }                \
  static inline OpD operator/(OpD a, T b) { return a / OpD((double)b); }                \
  static inline OpD operator/(T a, OpD b) { return OpD((double)a) / b; }                \
  static inline bool operator<(OpD a, T b) { return a.v < (double)b; }                  \
  static inline bool operator>(OpD a, T b) { return a.v > (double)b; }                  \
  static inline bool operator<=(OpD a, T b) { return a.v <= (double)b; }                \
  static inline bool operator>=(OpD a, T b) { return a.v >= (double)b; }                \
  static inline bool operator==(OpD a, T b) { return a.v == (double)b; }                \
  static inline bool operator!=(OpD a, T b) { return a.v != (double)b; }
OPD_MIXED_OPS(double)
OPD_MIXED_OPS(int)
OPD_MIXED_OPS(long)
OPD_MIXED_OPS(long long)
OPD_MIXED_OPS(unsigned long)
#undef OPD_MIXED_OPS

static inline OpD sqrt(OpD a) { tick(); return OpD(::sqrt(a.v)); }
static inline OpD exp(OpD a) { call(); return OpD(::exp(a.v)); }
static inline OpD pow(OpD a, OpD b) { call(); return OpD(::pow(a.v, b.v)); }
static inline OpD pow(OpD a, double b) { call(); return OpD(::pow(a.v, b)); }
static inline OpD pow(OpD a, int b) { call(); return OpD(::pow(a.v, (double)b)); }
static inline OpD sin(OpD a) { call(); return OpD(::sin(a.v)); }
static inline OpD cos(OpD a) { call(); return OpD(::cos(a.v)); }
static inline OpD fabs(OpD a) { return OpD(::fabs(a.v)); }
static inline OpD floor(OpD a) { return OpD(::floor(a.v)); }
static inline OpD ceil(OpD a) { return OpD(::ceil(a.v)); }
static inline OpD atof_opd(const char *s) { return OpD(::atof(s)); }

#define ORC_OPCAT(cat) (g_cat = (cat))
#define ORC_OPUNIT(cat) (g_units[(cat)] += 1)
#define double OpD
#define atof atof_opd
#include "lmff_oracle.c"
#undef atof
#undef double

// Counts of one force evaluation (which: 1 Tersoff, 2 ILP, 3 both) of the owned atoms
// x[n*3] (plain doubles, as the oracle's C interface takes them) in an orthogonal box,
// single-threaded.  ops/calls/units[ORC_NCAT] out.  Returns 0 or the oracle's error.
extern "C" int opc_count(const char *tersoff_file, const char *ilp_file, int ntypes, const char *const *elements,
                         double cut_global, int tap_flag, int n, const double *x, const int *type, const int64_t *mol,
                         const int64_t *tag, const double *lo, const double *hi, const int *periodic, int which,
                         uint64_t *ops, uint64_t *calls, uint64_t *units, char *err, int errlen) {
  static orc_pot pot;
  int rc = orc_pot_init(&pot, ntypes, OpD(cut_global), tap_flag, OpD(2.0));
  if (!rc && tersoff_file) rc = orc_read_tersoff(&pot, tersoff_file, elements);
  if (!rc && ilp_file) rc = orc_read_ilp(&pot, ilp_file, elements);
  if (rc) {
    snprintf(err, errlen, "%s", orc_pot_error(&pot));
    return rc;
  }
  orc_ctx *c = orc_new(&pot, 1);
  rc = orc_set_atoms(c, n, reinterpret_cast<const OpD *>(x), type, mol, tag, reinterpret_cast<const OpD *>(lo),
                     reinterpret_cast<const OpD *>(hi), periodic);
  if (rc) {
    snprintf(err, errlen, "%s", orc_error(c));
    orc_free(c);
    return rc;
  }
  OpD *f = (OpD *)calloc((size_t)3 * n, sizeof(OpD));
  orc_result r;
  memset(g_ops, 0, sizeof g_ops);
  memset(g_calls, 0, sizeof g_calls);
  memset(g_units, 0, sizeof g_units);
  g_cat = ORC_CAT_OTHER;
  rc = orc_forces(c, which, f, nullptr, &r);
  if (rc) snprintf(err, errlen, "%s", orc_error(c));
  for (int k = 0; k < ORC_NCAT; k++) {
    ops[k] = g_ops[k];
    calls[k] = g_calls[k];
    units[k] = g_units[k];
  }
  free(f);
  orc_free(c);
  return rc;
}
