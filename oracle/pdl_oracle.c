/*
 * pdl_oracle.c -- TEST INFRASTRUCTURE ONLY.  A CPU restatement of the
 * reference's algorithms for the broadcast-loop hot path, used by tests/ as
 * the parity checker and by bench.py as the timed CPU baseline.  It is never
 * linked into, loaded by, or called from the product library.
 *
 * What is restated (file:line in PDL 2.106):
 *   - type selection and output typing: pdl__transtype_select and
 *     PDL_TYPE_ADJUST_FROM_TRANS, lib/PDL/Core/pdlapi.c:1169-1236, 1240-1259;
 *     input conversion lib/PDL/Core/pdlconv.c:163-172 (bad -> bad,
 *     unsigned targets through intmax_t);
 *   - the broadcast engine for implicit broadcasting:
 *     pdl_initbroadcaststruct lib/PDL/Core/pdlbroadcast.c:340-488,
 *     pdl_broadcast_dim_checks :275-327, pdl_dim_checks :211-273,
 *     pdl_broadcast_create_parameter :490-523, pdl_redodims_default
 *     lib/PDL/Core/pdlapi.c:829-869, the error text of pdl_param_error
 *     lib/PDL/Core/pdlutil.c:65-147;
 *   - the auto-pthread split of one broadcast dim: pdl_find_max_pthread
 *     lib/PDL/Core/pdlbroadcast.c:95-159, chunking :469-484 and
 *     PDL_BRC_OFFSET lib/PDL/Core/pdlbroadcast.h:63;
 *   - the per-element Code of each op, in the reference's sequential order:
 *     sumover/prodover (+d) lib/PDL/Ufunc.pd:94-118, cumusumover (+d)
 *     :120-140, average (+d) :413-444, minimum/maximum(+_ind) :446-500,
 *     plus/mult and the other binary ops lib/PDL/Ops.pd:133-153,288-307,
 *     inner lib/PDL/Primitive.pd:48-76,
 *     matmult lib/PDL/Primitive.pd:211-248 (same t-tile order);
 *   - badflag propagation to outputs lib/PDL/Core/pdlapi.c:760-808.
 *
 * Integer arithmetic wraps (the reference is compiled with -fwrapv) and
 * floating point is not contracted to FMA (-ffp-contract=off, as the
 * reference's x86-64 build has no FMA): see oracle/Makefile.
 * `inner` accumulates in long double, as the reference does.
 */
#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/pdlgb300.h"

#define MAXP 5
#define MAXB (PDLGB300_MAXDIMS + 2)

/* ------------------------------------------------------------------ types */

#define O_REAL_TYPES(X)                                   \
  X(PDLGB300_SB, int8_t, A, int32_t, 0, 0)                \
  X(PDLGB300_B, uint8_t, B, int32_t, 0, 1)                \
  X(PDLGB300_S, int16_t, S, int32_t, 0, 0)                \
  X(PDLGB300_US, uint16_t, U, int32_t, 0, 1)              \
  X(PDLGB300_L, int32_t, L, int32_t, 0, 0)                \
  X(PDLGB300_UL, uint32_t, K, uint32_t, 0, 1)             \
  X(PDLGB300_IND, int64_t, N, int64_t, 0, 0)              \
  X(PDLGB300_ULL, uint64_t, P, uint64_t, 0, 1)            \
  X(PDLGB300_LL, int64_t, Q, int64_t, 0, 0)               \
  X(PDLGB300_F, float, F, float, 1, 0)                    \
  X(PDLGB300_D, double, D, double, 1, 0)
/* the same list, for nesting inside an O_REAL_TYPES expansion */
#define O_REAL_TYPES2(X)                                  \
  X(PDLGB300_SB, int8_t, A, int32_t, 0, 0)                \
  X(PDLGB300_B, uint8_t, B, int32_t, 0, 1)                \
  X(PDLGB300_S, int16_t, S, int32_t, 0, 0)                \
  X(PDLGB300_US, uint16_t, U, int32_t, 0, 1)              \
  X(PDLGB300_L, int32_t, L, int32_t, 0, 0)                \
  X(PDLGB300_UL, uint32_t, K, uint32_t, 0, 1)             \
  X(PDLGB300_IND, int64_t, N, int64_t, 0, 0)              \
  X(PDLGB300_ULL, uint64_t, P, uint64_t, 0, 1)            \
  X(PDLGB300_LL, int64_t, Q, int64_t, 0, 0)               \
  X(PDLGB300_F, float, F, float, 1, 0)                    \
  X(PDLGB300_D, double, D, double, 1, 0)

static const char *type_names[] = {"sbyte", "byte", "short", "ushort", "long",
                                   "ulong", "indx", "ulonglong", "longlong",
                                   "float", "double", "ldouble", "cfloat",
                                   "cdouble", "cldouble"};
static size_t type_size(int t) {
  static const size_t s[] = {1, 1, 2, 2, 4, 4, 8, 8, 8, 4, 8, 16, 8, 16, 32};
  return (t >= 0 && t < PDLGB300_NTYPES) ? s[t] : 0;
}

/* per-type default badvalues, Types.pm defbval */
static pdlgb300_value default_bad(int t) {
  pdlgb300_value v;
  memset(&v, 0, sizeof v);
  switch (t) {
    case PDLGB300_SB: v.A = INT8_MIN; break;
    case PDLGB300_B: v.B = UINT8_MAX; break;
    case PDLGB300_S: v.S = INT16_MIN; break;
    case PDLGB300_US: v.U = UINT16_MAX; break;
    case PDLGB300_L: v.L = INT32_MIN; break;
    case PDLGB300_UL: v.K = UINT32_MAX; break;
    case PDLGB300_IND: v.N = INT64_MIN; break;
    case PDLGB300_ULL: v.P = UINT64_MAX; break;
    case PDLGB300_LL: v.Q = INT64_MIN; break;
    case PDLGB300_F: v.F = -3.40282346638528859812e+38F; break;
    case PDLGB300_D: v.D = -1.79769313486231570815e+308; break;
  }
  return v;
}

static pdlgb300_value badval_of(const pdlgb300_ndarray *x) {
  return x->has_badvalue ? x->badvalue.value : default_bad(x->datatype);
}

/* ---------------------------------------------------------------- op table */

enum {
  OP_SUMOVER, OP_DSUMOVER, OP_PRODOVER, OP_DPRODOVER, OP_CUMUSUMOVER,
  OP_DCUMUSUMOVER, OP_AVERAGE, OP_DAVERAGE, OP_MINIMUM, OP_MAXIMUM,
  OP_MINIMUM_IND, OP_MAXIMUM_IND, OP_PLUS, OP_MULT, OP_INNER, OP_MATMULT,
  OP_MINUS, OP_DIVIDE, OP_GT, OP_LT, OP_LE, OP_GE, OP_EQ, OP_NE, OP_SHIFTLEFT,
  OP_SHIFTRIGHT, OP_OR2, OP_AND2, OP_XOR,
  OP_ANDOVER, OP_OROVER, OP_XOROVER, OP_ZCOVER, OP_BANDOVER, OP_BOROVER,
  OP_BXOROVER, OP_FIRSTNONZEROOVER, OP_CUMUPRODOVER, OP_DCUMUPRODOVER,
  OP_MINMAXIMUM, OP_QSORT, OP_QSORTI, OP_MEDOVER, OP_ODDMEDOVER, OP_PCTOVER,
  OP_ODDPCTOVER, OP_MODEOVER, OP_QSORTVEC, OP_QSORTVECI,
  OP_N
};
#define IS_BIOP(op) ((op) == OP_PLUS || (op) == OP_MULT || ((op) >= OP_MINUS && (op) <= OP_XOR))

#define TYPED 1  /* typed output */
#define TPLUS 2  /* "int+" */

typedef struct {
  const char *name;
  int npdls, nparents;
  const char *par_names[MAXP];
  int realdims[MAXP];
  int ind[MAXP][2];     /* index id per real dim */
  const char *ind_names[3];
  int out_typed;        /* 0, TYPED, TYPED|TPLUS for the output */
  int out_type;         /* typed output type */
  int int_only;         /* GenericTypes = the integer types (bit ops) */
  int idx_from;         /* > 0: outputs from this parameter on are indx */
} opdef;

static const opdef OPS[OP_N] = {
  {"sumover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, TYPED | TPLUS, PDLGB300_L},
  {"dsumover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, TYPED, PDLGB300_D},
  {"prodover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, TYPED | TPLUS, PDLGB300_L},
  {"dprodover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, TYPED, PDLGB300_D},
  {"cumusumover", 2, 1, {"a", "b"}, {1, 1}, {{0}, {0}}, {"n"}, TYPED | TPLUS, PDLGB300_L},
  {"dcumusumover", 2, 1, {"a", "b"}, {1, 1}, {{0}, {0}}, {"n"}, TYPED, PDLGB300_D},
  {"average", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, TYPED | TPLUS, PDLGB300_L},
  {"daverage", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, TYPED, PDLGB300_D},
  {"minimum", 2, 1, {"a", "c"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1},
  {"maximum", 2, 1, {"a", "c"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1},
  {"minimum_ind", 2, 1, {"a", "c"}, {1, 0}, {{0}, {0}}, {"n"}, TYPED, PDLGB300_IND},
  {"maximum_ind", 2, 1, {"a", "c"}, {1, 0}, {{0}, {0}}, {"n"}, TYPED, PDLGB300_IND},
  {"plus", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1},
  {"mult", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1},
  {"inner", 3, 2, {"a", "b", "c"}, {1, 1, 0}, {{0}, {0}, {0}}, {"n"}, 0, -1},
  {"matmult", 3, 2, {"a", "b", "c"}, {2, 2, 2}, {{0, 1}, {2, 0}, {2, 1}},
   {"t", "h", "w"}, 0, -1},
  /* lib/PDL/Ops.pd:290-307 */
  {"minus", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1},
  {"divide", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1},
  {"gt", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1},
  {"lt", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1},
  {"le", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1},
  {"ge", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1},
  {"eq", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1},
  {"ne", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1},
  {"shiftleft", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1, 1},
  {"shiftright", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1, 1},
  {"or2", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1, 1},
  {"and2", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1, 1},
  {"xor", 3, 2, {"a", "b", "c"}, {0, 0, 0}, {{0}, {0}, {0}}, {0}, 0, -1, 1},
  /* lib/PDL/Ufunc.pd:143-187: a(n); [o] b() in the generic type */
  {"andover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1},
  {"orover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1},
  {"xorover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1},
  {"zcover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1},
  {"bandover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1, 1},
  {"borover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1, 1},
  {"bxorover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1, 1},
  {"firstnonzeroover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1},
  {"cumuprodover", 2, 1, {"a", "b"}, {1, 1}, {{0}, {0}}, {"n"}, TYPED | TPLUS, PDLGB300_L},
  {"dcumuprodover", 2, 1, {"a", "b"}, {1, 1}, {{0}, {0}}, {"n"}, TYPED, PDLGB300_D},
  /* lib/PDL/Ufunc.pd:563-613 */
  {"minmaximum", 5, 1, {"a", "cmin", "cmax", "cmin_ind", "cmax_ind"}, {1, 0, 0, 0, 0},
   {{0}, {0}, {0}, {0}, {0}}, {"n"}, 0, -1, 0, 3},
  /* lib/PDL/Ufunc.pd:878-1115: the sort-based functions */
  {"qsort", 2, 1, {"a", "b"}, {1, 1}, {{0}, {0}}, {"n"}, 0, -1},
  {"qsorti", 2, 1, {"a", "indx"}, {1, 1}, {{0}, {0}}, {"n"}, TYPED, PDLGB300_IND},
  {"medover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1},
  {"oddmedover", 2, 1, {"a", "b"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1},
  {"pctover", 3, 2, {"a", "p", "b"}, {1, 0, 0}, {{0}, {0}, {0}}, {"n"}, 0, -1},
  {"oddpctover", 3, 2, {"a", "p", "b"}, {1, 0, 0}, {{0}, {0}, {0}}, {"n"}, 0, -1},
  {"modeover", 2, 1, {"data", "out"}, {1, 0}, {{0}, {0}}, {"n"}, 0, -1, 1},
  /* lib/PDL/Ufunc.pd:1115-1230: a list of m vectors of n, sorted lexicographically */
  {"qsortvec", 2, 1, {"a", "b"}, {2, 2}, {{0, 1}, {0, 1}}, {"n", "m"}, 0, -1},
  {"qsortveci", 2, 1, {"a", "indx"}, {2, 1}, {{0, 1}, {1}}, {"n", "m"}, TYPED, PDLGB300_IND},
};

static int find_op(const char *name) {
  for (int i = 0; i < OP_N; i++)
    if (!strcmp(OPS[i].name, name)) return i;
  return -1;
}

/* ------------------------------------------------------------------ errors */

typedef struct {
  char *buf;
  size_t len;
} errbuf;

static int set_err(errbuf *e, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  if (e->buf && e->len) vsnprintf(e->buf, e->len, fmt, ap);
  va_end(ap);
  return 1;
}

/* pdl_param_error, lib/PDL/Core/pdlutil.c:65-147 */
/* The package defining an op: pdl_param_error uses the package-qualified
 * vtable name ("PDL::Ops::plus"; PDL's pp_def vtables). */
static const char *op_package(const char *name) {
  static const char *const ops[] = {"plus", "mult", "minus", "divide", "gt", "lt", "le", "ge",
                                    "eq", "ne", "shiftleft", "shiftright", "or2", "and2", "xor"};
  for (size_t k = 0; k < sizeof ops / sizeof ops[0]; k++)
    if (!strcmp(name, ops[k])) return "PDL::Ops::";
  if (!strcmp(name, "inner") || !strcmp(name, "matmult")) return "PDL::Primitive::";
  return "PDL::Ufunc::";
}

const char *oracle_op_package(const char *name) { return op_package(name); }

static int param_error(errbuf *e, const opdef *op, int param,
                       pdlgb300_ndarray *const *pdls, int64_t nimpl,
                       const int *creating, const char *fmt, ...) {
  char msg[4096];
  size_t off = 0;
#define ADV() off = strlen(msg)
  msg[0] = 0;
  if (param < 0 || param >= op->npdls) {
    snprintf(msg, sizeof msg, "ERROR: UNKNOWN PARAMETER");
  } else {
    snprintf(msg, sizeof msg, "%s%s(", op_package(op->name), op->name);
    for (int i = 0; i < op->npdls; i++) {
      ADV();
      snprintf(msg + off, sizeof msg - off, "%s%s", op->par_names[i],
               i < op->npdls - 1 ? "," : "");
    }
    ADV();
    snprintf(msg + off, sizeof msg - off, "): parameter '%s': ",
             op->par_names[param]);
  }
  ADV();
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg + off, sizeof msg - off, fmt, ap);
  va_end(ap);
  ADV();
  snprintf(msg + off, sizeof msg - off,
           "\nThere are %d PDLs in the expression; %lld broadcast dim%s.\n",
           op->npdls, (long long)nimpl, nimpl == 1 ? "" : "s");
  int maxreal = 0;
  for (int i = 0; i < op->npdls; i++)
    if (op->realdims[i] > maxreal) maxreal = op->realdims[i];
  ADV();
  snprintf(msg + off, sizeof msg - off, "   PDL IN EXPR.    ");
  if (maxreal > 0) {
    char fmt2[32];
    snprintf(fmt2, sizeof fmt2, "%%%ds", 8 * maxreal + 3);
    ADV();
    snprintf(msg + off, sizeof msg - off, fmt2, "ACTIVE DIMS | ");
  }
  ADV();
  snprintf(msg + off, sizeof msg - off, "BROADCAST DIMS\n");
  for (int i = 0; i < op->npdls; i++) {
    ADV();
    snprintf(msg + off, sizeof msg - off, "   #%3d (%s", i,
             creating[i] ? "null)\n" : "normal): ");
    if (creating[i]) continue;
    if (maxreal == 1) {
      ADV();
      snprintf(msg + off, sizeof msg - off, "    ");
    }
    for (int j = 0; j < maxreal - op->realdims[i]; j++) {
      ADV();
      snprintf(msg + off, sizeof msg - off, "%8s", " ");
    }
    for (int j = 0; j < op->realdims[i]; j++) {
      ADV();
      snprintf(msg + off, sizeof msg - off, "%8lld",
               (long long)(j < pdls[i]->ndims ? pdls[i]->dims[j] : 1));
    }
    if (maxreal) {
      ADV();
      snprintf(msg + off, sizeof msg - off, " | ");
    }
    for (int j = 0; j < nimpl && j + op->realdims[i] < pdls[i]->ndims; j++) {
      ADV();
      snprintf(msg + off, sizeof msg - off, "%8lld",
               (long long)pdls[i]->dims[j + op->realdims[i]]);
    }
    ADV();
    snprintf(msg + off, sizeof msg - off, "\n");
  }
#undef ADV
  return set_err(e, "%s", msg);
}

/* -------------------------------------------------------- type selection */

/* pdl__transtype_select (lib/PDL/Core/pdlapi.c:1208-1235) with GenericTypes
 * = all real types (ldouble and the complex types are not computed by this
 * path), or the integer types for the bit ops: the largest allowed type
 * among the untyped parameters, outputs first; a type above the last
 * allowed one, or none, gives the last allowed type. */
static int transtype_select(const opdef *op, pdlgb300_ndarray *const *pdls) {
  const int last = op->int_only ? PDLGB300_LL : PDLGB300_D;
  int ret = -1, use_last = 0;
  for (int i = op->npdls - 1; i >= 0; i--) {
    const pdlgb300_ndarray *p = pdls[i];
    int is_typed = (i >= op->nparents) && (op->out_typed || (op->idx_from && i >= op->idx_from));
    if (!(p->state & PDLGB300_NOMYDIMS) && !is_typed) {
      int t = p->datatype;
      int avail = t <= last;
      if (!avail && t > last) use_last = 1;
      if (avail && ret < t) ret = t;
    }
    if (i == op->nparents && ret != -1) return ret;
  }
  if (use_last || ret < 0) ret = last;
  return ret;
}

static int out_type_for(const opdef *op, int ttype, int j) {
  if (op->idx_from && j >= op->idx_from) return PDLGB300_IND;
  if (!op->out_typed) return ttype;
  if (op->out_typed & TPLUS) return op->out_type > ttype ? op->out_type : ttype;
  return op->out_type;
}

/* ---------------------------------------------------------- broadcasting */

typedef struct {
  int npdls, ndims, nimpl;
  int64_t dims[MAXB];
  int64_t incs[MAXB][MAXP]; /* PDL_BRC_INC */
  int64_t ind_sizes[3];
  int64_t inc_sizes[MAXP][2];
} obrc;

/* a dummy (broadcast) dim of a view: increment 0 (PDL tests the view's
 * vafftrans increments; an empty ndarray is never a view of anything) */
static int is_dummy(const pdlgb300_ndarray *p, int d) {
  if (d >= p->ndims || p->incs[d] != 0) return 0;
  for (int i = 0; i < p->ndims; i++)
    if (p->dims[i] == 0) return 0;
  return 1;
}

static void default_incs(pdlgb300_ndarray *p) {
  int64_t s = 1;
  for (int i = 0; i < p->ndims; i++) {
    p->incs[i] = s;
    s *= p->dims[i];
  }
}

/* Fill brc and shape null outputs.  pdls are not modified except the
 * creating (null) outputs. */
static int do_redodims(errbuf *e, const opdef *op, pdlgb300_ndarray *const *pdls,
                       obrc *b) {
  int creating[MAXP];
  int np = op->npdls;
  memset(b, 0, sizeof *b);
  b->npdls = np;
  int64_t nimpl = 0;
  for (int j = 0; j < np; j++) {
    creating[j] = (j >= op->nparents) && (pdls[j]->state & PDLGB300_NOMYDIMS);
    if (j < op->nparents && (pdls[j]->state & PDLGB300_NOMYDIMS))
      return set_err(e, "Error in %s%s: input parameter '%s' is null", op_package(op->name),
                     op->name, op->par_names[j]);
    if (creating[j]) continue;
    int64_t k = pdls[j]->ndims - op->realdims[j];
    if (k > nimpl) nimpl = k;
  }
  if (nimpl > PDLGB300_MAXDIMS) return set_err(e, "too many dims");
  int64_t ndims = nimpl + (nimpl < 2 ? 2 - nimpl : 0);
  b->ndims = (int)ndims;
  b->nimpl = (int)nimpl;
  for (int k = 0; k < ndims; k++) b->dims[k] = 1;
  /* pdl_broadcast_dim_checks */
  for (int nth = 0; nth < nimpl; nth++) {
    for (int j = 0; j < np; j++) {
      if (creating[j]) continue;
      const pdlgb300_ndarray *p = pdls[j];
      int isout = j >= op->nparents;
      if (nth >= p->ndims - op->realdims[j]) {
        if (isout && b->dims[nth] != 1)
          return param_error(e, op, nth, pdls, nimpl, creating,
                             "implicit dim %lld size %lld, can't broadcast over output ndarray with size > 1",
                             (long long)nth, (long long)b->dims[nth]);
        continue;
      }
      int64_t cur = p->dims[nth + op->realdims[j]];
      if (isout && cur == 1 && cur != b->dims[nth])
        return param_error(e, op, nth, pdls, nimpl, creating,
                           "implicit dim %lld size %lld, but dim has size %lld",
                           (long long)nth, (long long)b->dims[nth], (long long)cur);
      if (isout && cur != 1 && is_dummy(p, nth + op->realdims[j]))
        return param_error(e, op, nth, pdls, nimpl, creating,
                           "implicit dim %lld size %lld, but dim is dummy",
                           (long long)nth, (long long)b->dims[nth]);
      if (cur != 1) {
        if (b->dims[nth] != 1) {
          if (b->dims[nth] != cur)
            return param_error(e, op, j, pdls, nimpl, creating,
                               "Mismatched implicit broadcast dimension %lld: size %lld vs. %lld",
                               (long long)nth, (long long)b->dims[nth], (long long)cur);
        } else {
          b->dims[nth] = cur;
        }
        b->incs[nth][j] = p->incs[nth + op->realdims[j]];
      }
    }
  }
  /* pdl_dim_checks */
  for (int i = 0; i < 3; i++) b->ind_sizes[i] = -1;
  for (int i = 0; i < np; i++) {
    if (creating[i]) continue;
    const pdlgb300_ndarray *p = pdls[i];
    int isout = i >= op->nparents;
    for (int j = 0; j < op->realdims[i]; j++) {
      int id = op->ind[i][j];
      int64_t sz = b->ind_sizes[id];
      if (j >= p->ndims && sz == -1) sz = b->ind_sizes[id] = 1;
      if (sz == -1 || (j < p->ndims && sz == 1)) {
        b->ind_sizes[id] = j < p->ndims ? p->dims[j] : 1;
        continue;
      }
      if (j >= p->ndims && isout && sz != 1)
        return param_error(e, op, i, pdls, nimpl, creating,
                           "index '%s' size %lld, can't broadcast over output ndarray with size > 1",
                           op->ind_names[id], (long long)sz);
      if (isout && sz != 1 && is_dummy(p, j))
        return param_error(e, op, i, pdls, nimpl, creating,
                           "index '%s' size %lld, can't broadcast over dummy dim with size > 1",
                           op->ind_names[id], (long long)sz);
      if (j < p->ndims && sz != p->dims[j] && (isout || p->dims[j] != 1))
        return param_error(e, op, i, pdls, nimpl, creating,
                           "index '%s' size %lld, but ndarray dim has size %lld",
                           op->ind_names[id], (long long)sz, (long long)p->dims[j]);
    }
  }
  /* pdl_broadcast_create_parameter for null outputs */
  for (int j = 0; j < np; j++) {
    if (!creating[j]) continue;
    pdlgb300_ndarray *p = pdls[j];
    int nd = op->realdims[j] + (int)nimpl;
    if (nd > PDLGB300_MAXDIMS) return set_err(e, "too many dims");
    p->ndims = nd;
    for (int i = 0; i < op->realdims[j]; i++) {
      int64_t s = b->ind_sizes[op->ind[j][i]];
      p->dims[i] = s < 0 ? 1 : s;
    }
    for (int i = 0; i < nimpl; i++) p->dims[i + op->realdims[j]] = b->dims[i];
    default_incs(p);
    p->offs = 0;
    for (int i = 0; i < nimpl; i++) b->incs[i][j] = p->incs[i + op->realdims[j]];
  }
  /* inc_sizes */
  for (int i = 0; i < np; i++) {
    const pdlgb300_ndarray *p = pdls[i];
    for (int j = 0; j < op->realdims[i]; j++)
      b->inc_sizes[i][j] = (p->ndims <= j || p->dims[j] <= 1) ? 0 : p->incs[j];
  }
  for (int i = 0; i < 3; i++)
    if (b->ind_sizes[i] < 0) b->ind_sizes[i] = 1;
  return 0;
}

void oracle_ndarray_init(pdlgb300_ndarray *x, int32_t datatype, int32_t ndims,
                         const int64_t *dims, void *data, void *ddata);

/* ------------------------------------------------------------ conversion */

#define O_GET(ctype, p) (*(const ctype *)(p))

/* Convert one element (C conversion; unsigned targets via intmax_t). */
static void convert_elem(int from, const void *src, int to, void *dst) {
  switch (from) {
#define X_FROM(E, CT, SYM, IP, ISF, UNS) \
  case E: {                              \
    CT v = O_GET(CT, src);               \
    switch (to) {                        \
      X_TO_LIST                          \
    }                                    \
    break;                               \
  }
#define X_TO(E2, CT2, SYM2, IP2, ISF2, UNS2)                               \
  case E2:                                                                  \
    *(CT2 *)dst = UNS2 ? (CT2)(intmax_t)v : (CT2)v;                         \
    break;
#define X_TO_LIST O_REAL_TYPES2(X_TO)
    O_REAL_TYPES(X_FROM)
#undef X_TO_LIST
#undef X_TO
#undef X_FROM
  }
}

static int value_isbad(int t, const void *p, pdlgb300_value bv) {
  switch (t) {
#define X(E, CT, SYM, IP, ISF, UNS)                                 \
  case E: {                                                          \
    CT v = O_GET(CT, p);                                             \
    if (ISF && isnan((double)bv.SYM)) return isnan((double)v);       \
    return v == bv.SYM;                                              \
  }
    O_REAL_TYPES(X)
#undef X
  }
  return 0;
}

static void store_value(int t, void *p, pdlgb300_value v) {
  memcpy(p, &v, type_size(t));
}

/* Make a contiguous converted copy of x (type `to`), applying the bad-value
 * mapping when bad != 0.  Returns malloc'd data. */
static void *converted_copy(const pdlgb300_ndarray *x, int to, int bad) {
  int64_t n = 1;
  for (int i = 0; i < x->ndims; i++) n *= x->dims[i];
  size_t ts = type_size(to), fs = type_size(x->datatype);
  char *out = malloc(n * ts + 16);
  pdlgb300_value fb = badval_of(x), tb = default_bad(to);
  int64_t idx[PDLGB300_MAXDIMS] = {0};
  for (int64_t k = 0; k < n; k++) {
    int64_t off = x->offs;
    for (int d = 0; d < x->ndims; d++) off += idx[d] * x->incs[d];
    const char *src = (const char *)x->data + off * (int64_t)fs;
    if (bad && value_isbad(x->datatype, src, fb))
      store_value(to, out + k * ts, tb);
    else
      convert_elem(x->datatype, src, to, out + k * ts);
    for (int d = 0; d < x->ndims; d++) {
      if (++idx[d] < x->dims[d]) break;
      idx[d] = 0;
    }
  }
  return out;
}

/* -------------------------------------------------------------- op bodies */

typedef struct {
  int op, ttype;
  int bvalflag;
  char *base[MAXP];       /* byte pointers to element 0 of each pdl's data */
  int64_t inc_sizes[MAXP][2];
  int64_t ind_sizes[3];
  int statebad[MAXP];     /* PDLSTATEISBAD per param */
  pdlgb300_value bad[MAXP];
  volatile int setbad_out; /* PDLSTATESETBAD(output) requested */
  const int64_t *other;
} octx;

typedef void (*body_fn)(octx *c, const int64_t *offs, int64_t n0,
                        const int64_t *inc0);

#define ISBADV(v, bv, ISF) ((ISF) && isnan((double)(bv)) ? isnan((double)(v)) : (v) == (bv))

/* reductions over n: a(n); [o]b() ---------------------------------------- */
#define DEF_OVER(NAME, TA, SYMA, TB, SYMB, ISFA, INIT, OPSTMT, LEFTZERO)           \
  static void NAME(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    const TA *a0 = (const TA *)c->base[0] + offs[0];                                 \
    TB *b0 = (TB *)c->base[1] + offs[1];                                             \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0];                            \
    TA abad = c->bad[0].SYMA;                                                        \
    TB bbad = c->bad[1].SYMB;                                                        \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const TA *a = a0 + i0 * inc0[0];                                               \
      TB tmp = INIT;                                                                 \
      int flag = 0;                                                                  \
      if (c->bvalflag) {                                                             \
        for (int64_t n = 0; n < N; n++) {                                            \
          TA v = a[n * ia];                                                          \
          if (ISBADV(v, abad, ISFA)) continue;                                       \
          flag = 1;                                                                  \
          OPSTMT;                                                                    \
          if (LEFTZERO) break;                                                       \
        }                                                                            \
        b0[i0 * inc0[1]] = flag ? tmp : bbad;                                        \
      } else {                                                                       \
        for (int64_t n = 0; n < N; n++) {                                            \
          TA v = a[n * ia];                                                          \
          OPSTMT;                                                                    \
          if (LEFTZERO) break;                                                       \
        }                                                                            \
        b0[i0 * inc0[1]] = tmp;                                                      \
      }                                                                              \
      (void)flag;                                                                    \
    }                                                                                \
  }

#define DEF_SUMS(E, CT, SYM, IP, ISF, UNS)                                                  \
  DEF_OVER(sumover_##SYM, CT, SYM, IP, SYM##_ip, ISF, 0, tmp += v, 0)                         \
  DEF_OVER(dsumover_##SYM, CT, SYM, double, D, ISF, 0, tmp += v, 0)                           \
  DEF_OVER(prodover_##SYM, CT, SYM, IP, SYM##_ip, ISF, 1, tmp *= v, tmp == 0)                 \
  DEF_OVER(dprodover_##SYM, CT, SYM, double, D, ISF, 1, tmp *= v, tmp == 0)

/* lib/PDL/Ufunc.pd:143-187 (the reference's `char tmp` of the logical ones
 * holds the same 0/1 as a tmp of the output type) */
#define DEF_LOGICS(E, CT, SYM, IP, ISF, UNS)                                              \
  DEF_OVER(andover_##SYM, CT, SYM, CT, SYM, ISF, 1, tmp = (CT)((tmp != 0) & (v != 0)), !tmp) \
  DEF_OVER(orover_##SYM, CT, SYM, CT, SYM, ISF, 0, tmp = (CT)((tmp != 0) | (v != 0)), tmp)   \
  DEF_OVER(xorover_##SYM, CT, SYM, CT, SYM, ISF, 0, tmp = (CT)((tmp != 0) ^ (v != 0)), 0)  \
  DEF_OVER(zcover_##SYM, CT, SYM, CT, SYM, ISF, 1, tmp = (CT)((tmp != 0) & (v == 0)), !tmp) \
  DEF_OVER(firstnonzeroover_##SYM, CT, SYM, CT, SYM, ISF, 0, tmp = v, tmp)
#define DEF_BITOVERS(E, CT, SYM, IP, ISF, UNS)                              \
  DEF_OVER(bandover_##SYM, CT, SYM, CT, SYM, 0, ~0, tmp &= v, !tmp)         \
  DEF_OVER(borover_##SYM, CT, SYM, CT, SYM, 0, 0, tmp |= v, !~tmp)          \
  DEF_OVER(bxorover_##SYM, CT, SYM, CT, SYM, 0, 0, tmp ^= v, 0)

/* the int+ output's value-union member per input type */
#define A_ip L
#define B_ip L
#define S_ip L
#define U_ip L
#define L_ip L
#define K_ip K
#define N_ip N
#define P_ip P
#define Q_ip Q
#define F_ip F
#define D_ip D
O_REAL_TYPES(DEF_SUMS)
O_REAL_TYPES(DEF_LOGICS)

/* cumusumover: a(n); [o]b(n) */
#define DEF_CUMU(NAME, TA, SYMA, TB, SYMB, ISFA) DEF_CUMU_OP(NAME, TA, SYMA, TB, SYMB, ISFA, 0, +=)
#define DEF_CUMU_OP(NAME, TA, SYMA, TB, SYMB, ISFA, INIT, OP)                          \
  static void NAME(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0], ib = c->inc_sizes[1][0];   \
    TA abad = c->bad[0].SYMA;                                                        \
    TB bbad = c->bad[1].SYMB;                                                        \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const TA *a = (const TA *)c->base[0] + offs[0] + i0 * inc0[0];                 \
      TB *b = (TB *)c->base[1] + offs[1] + i0 * inc0[1];                             \
      TB tmp = INIT;                                                                 \
      for (int64_t n = 0; n < N; n++) {                                              \
        TA v = a[n * ia];                                                            \
        if (c->bvalflag && ISBADV(v, abad, ISFA)) {                                  \
          b[n * ib] = bbad;                                                          \
          continue;                                                                  \
        }                                                                            \
        tmp OP v;                                                                    \
        b[n * ib] = tmp;                                                             \
      }                                                                              \
    }                                                                                \
  }
#define DEF_CUMUS(E, CT, SYM, IP, ISF, UNS)                           \
  DEF_CUMU(cumusumover_##SYM, CT, SYM, IP, SYM##_ip, ISF)              \
  DEF_CUMU(dcumusumover_##SYM, CT, SYM, double, D, ISF)                \
  DEF_CUMU_OP(cumuprodover_##SYM, CT, SYM, IP, SYM##_ip, ISF, 1, *=)   \
  DEF_CUMU_OP(dcumuprodover_##SYM, CT, SYM, double, D, ISF, 1, *=)
O_REAL_TYPES(DEF_CUMUS)

/* average: tmp/cnt with cnt a PDL_Indx (C's usual conversions) */
#define DEF_AVG(NAME, TA, SYMA, TB, SYMB, ISFA, ISFB)                                   \
  static void NAME(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0];                            \
    TA abad = c->bad[0].SYMA;                                                        \
    TB bbad = c->bad[1].SYMB;                                                        \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const TA *a = (const TA *)c->base[0] + offs[0] + i0 * inc0[0];                 \
      TB *b = (TB *)c->base[1] + offs[1] + i0 * inc0[1];                             \
      TB tmp = 0;                                                                    \
      int64_t cnt = 0;                                                               \
      for (int64_t n = 0; n < N; n++) {                                              \
        TA v = a[n * ia];                                                            \
        if (c->bvalflag && ISBADV(v, abad, ISFA)) continue;                          \
        cnt++;                                                                       \
        tmp += v;                                                                    \
      }                                                                              \
      if (!cnt) {                                                                    \
        if (c->bvalflag) *b = bbad;                                                  \
        else *b = ISFB ? (TB)NAN : (TB)0;                                            \
      } else                                                                         \
        *b = tmp / cnt;                                                              \
    }                                                                                \
  }
#define DEF_AVGS(E, CT, SYM, IP, ISF, UNS)               \
  DEF_AVG(average_##SYM, CT, SYM, IP, SYM##_ip, ISF, ISF) \
  DEF_AVG(daverage_##SYM, CT, SYM, double, D, ISF, 1)
O_REAL_TYPES(DEF_AVGS)

/* minimum/maximum(+_ind): replace when first, when a OP cur, or cur is NaN */
#define DEF_MM(NAME, TA, SYMA, ISFA, CMP, IND)                                          \
  static void NAME(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0];                            \
    TA abad = c->bad[0].SYMA;                                                        \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const TA *a = (const TA *)c->base[0] + offs[0] + i0 * inc0[0];                 \
      TA cur = 0;                                                                    \
      int64_t curind = -1;                                                           \
      for (int64_t n = 0; n < N; n++) {                                              \
        TA v = a[n * ia];                                                            \
        if (c->bvalflag && ISBADV(v, abad, ISFA)) continue;                          \
        if (curind != -1 && !(v CMP cur) && !(ISFA && isnan((double)cur))) continue; \
        cur = v;                                                                     \
        curind = n;                                                                  \
      }                                                                              \
      if (IND) {                                                                     \
        int64_t *o = (int64_t *)c->base[1] + offs[1] + i0 * inc0[1];                 \
        if (curind != -1) *o = curind;                                               \
        else { *o = c->bad[1].N; c->setbad_out = 1; }                                \
      } else {                                                                       \
        TA *o = (TA *)c->base[1] + offs[1] + i0 * inc0[1];                           \
        if (curind != -1) *o = cur;                                                  \
        else { *o = c->bad[1].SYMA; c->setbad_out = 1; }                             \
      }                                                                              \
    }                                                                                \
  }
#define DEF_MMS(E, CT, SYM, IP, ISF, UNS)            \
  DEF_MM(minimum_##SYM, CT, SYM, ISF, <, 0)          \
  DEF_MM(maximum_##SYM, CT, SYM, ISF, >, 0)          \
  DEF_MM(minimum_ind_##SYM, CT, SYM, ISF, <, 1)      \
  DEF_MM(maximum_ind_##SYM, CT, SYM, ISF, >, 1)
O_REAL_TYPES(DEF_MMS)

/* minmaximum: skip bad (bad mode) and NaN; strict < / > keep the first
 * index; nothing left sets all four outputs bad (and their bad state) */
#define DEF_MINMAXIMUM(NAME, T, SYM, ISF)                                                \
  static void NAME(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0];                            \
    T abad = c->bad[0].SYM;                                                          \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *a = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      T *cmin = (T *)c->base[1] + offs[1] + i0 * inc0[1];                            \
      T *cmax = (T *)c->base[2] + offs[2] + i0 * inc0[2];                            \
      int64_t *imin = (int64_t *)c->base[3] + offs[3] + i0 * inc0[3];                \
      int64_t *imax = (int64_t *)c->base[4] + offs[4] + i0 * inc0[4];                \
      T curmin = 0, curmax = 0;                                                      \
      int64_t curmin_ind = 0, curmax_ind = 0;                                        \
      int flag = 0;                                                                  \
      for (int64_t n = 0; n < N; n++) {                                              \
        T v = a[n * ia];                                                             \
        if (c->bvalflag && ISBADV(v, abad, ISF)) continue;                           \
        if (ISF && isnan((double)v)) continue;                                       \
        if (!flag) {                                                                 \
          curmin = curmax = v;                                                       \
          curmin_ind = curmax_ind = n;                                               \
          flag = 1;                                                                  \
        } else {                                                                     \
          if (v < curmin) { curmin = v; curmin_ind = n; }                            \
          if (v > curmax) { curmax = v; curmax_ind = n; }                            \
        }                                                                            \
      }                                                                              \
      if (!flag) {                                                                   \
        *cmin = c->bad[1].SYM;                                                       \
        *cmax = c->bad[2].SYM;                                                       \
        *imin = c->bad[3].N;                                                         \
        *imax = c->bad[4].N;                                                         \
        c->setbad_out = 1;                                                           \
      } else {                                                                       \
        *cmin = curmin; *cmax = curmax; *imin = curmin_ind; *imax = curmax_ind;      \
      }                                                                              \
    }                                                                                \
  }
#define DEF_MINMAXIMUMS(E, CT, SYM, IP, ISF, UNS) DEF_MINMAXIMUM(minmaximum_##SYM, CT, SYM, ISF)
O_REAL_TYPES(DEF_MINMAXIMUMS)

/* plus/mult: a(); b(); [o]c() */
#define DEF_BIOP(NAME, T, SYM, ISF, OP)                                                 \
  static void NAME(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    const T *a = (const T *)c->base[0] + offs[0];                                    \
    const T *b = (const T *)c->base[1] + offs[1];                                    \
    T *o = (T *)c->base[2] + offs[2];                                                \
    if (!c->bvalflag) {                                                              \
      for (int64_t i = 0; i < n0; i++)                                               \
        o[i * inc0[2]] = (T)(a[i * inc0[0]] OP b[i * inc0[1]]);                      \
      return;                                                                        \
    }                                                                                \
    T abad = c->bad[0].SYM, bbad = c->bad[1].SYM, obad = c->bad[2].SYM;              \
    int anybad = 0;                                                                  \
    for (int64_t i = 0; i < n0; i++) {                                               \
      T va = a[i * inc0[0]], vb = b[i * inc0[1]];                                    \
      if ((c->statebad[0] && ISBADV(va, abad, ISF)) ||                               \
          (c->statebad[1] && ISBADV(vb, bbad, ISF))) {                               \
        o[i * inc0[2]] = obad;                                                       \
        anybad = 1;                                                                  \
      } else                                                                         \
        o[i * inc0[2]] = (T)(va OP vb);                                              \
    }                                                                                \
    if (anybad) c->setbad_out = 1;                                                   \
  }
#define DEF_BIOPS(E, CT, SYM, IP, ISF, UNS) \
  DEF_BIOP(plus_##SYM, CT, SYM, ISF, +)     \
  DEF_BIOP(mult_##SYM, CT, SYM, ISF, *)     \
  DEF_BIOP(minus_##SYM, CT, SYM, ISF, -)    \
  DEF_BIOP(divide_##SYM, CT, SYM, ISF, /)   \
  DEF_BIOP(gt_##SYM, CT, SYM, ISF, >)       \
  DEF_BIOP(lt_##SYM, CT, SYM, ISF, <)       \
  DEF_BIOP(le_##SYM, CT, SYM, ISF, <=)      \
  DEF_BIOP(ge_##SYM, CT, SYM, ISF, >=)      \
  DEF_BIOP(eq_##SYM, CT, SYM, ISF, ==)      \
  DEF_BIOP(ne_##SYM, CT, SYM, ISF, !=)
O_REAL_TYPES(DEF_BIOPS)
/* shifts and bit ops: the integer types only (GenericTypes $T) */
#define DEF_BITOPS(E, CT, SYM, IP, ISF, UNS) \
  DEF_BIOP(shiftleft_##SYM, CT, SYM, 0, <<)  \
  DEF_BIOP(shiftright_##SYM, CT, SYM, 0, >>) \
  DEF_BIOP(or2_##SYM, CT, SYM, 0, |)         \
  DEF_BIOP(and2_##SYM, CT, SYM, 0, &)        \
  DEF_BIOP(xor_##SYM, CT, SYM, 0, ^)
#define O_INT_TYPES(X)                        \
  X(PDLGB300_SB, int8_t, A, int32_t, 0, 0)    \
  X(PDLGB300_B, uint8_t, B, int32_t, 0, 1)    \
  X(PDLGB300_S, int16_t, S, int32_t, 0, 0)    \
  X(PDLGB300_US, uint16_t, U, int32_t, 0, 1)  \
  X(PDLGB300_L, int32_t, L, int32_t, 0, 0)    \
  X(PDLGB300_UL, uint32_t, K, uint32_t, 0, 1) \
  X(PDLGB300_IND, int64_t, N, int64_t, 0, 0)  \
  X(PDLGB300_ULL, uint64_t, P, uint64_t, 0, 1)\
  X(PDLGB300_LL, int64_t, Q, int64_t, 0, 0)
O_INT_TYPES(DEF_BITOPS)
O_INT_TYPES(DEF_BITOVERS)
#define bandover_F NULL
#define bandover_D NULL
#define borover_F NULL
#define borover_D NULL
#define bxorover_F NULL
#define bxorover_D NULL
#define shiftleft_F NULL
#define shiftleft_D NULL
#define shiftright_F NULL
#define shiftright_D NULL
#define or2_F NULL
#define or2_D NULL
#define and2_F NULL
#define and2_D NULL
#define xor_F NULL
#define xor_D NULL

/* inner: long double accumulator, product in the generic type */
#define DEF_INNER(NAME, T, SYM, ISF)                                                    \
  static void NAME(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0], ib = c->inc_sizes[1][0];   \
    T abad = c->bad[0].SYM, bbad = c->bad[1].SYM;                                    \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *a = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      const T *b = (const T *)c->base[1] + offs[1] + i0 * inc0[1];                   \
      T *o = (T *)c->base[2] + offs[2] + i0 * inc0[2];                               \
      long double tmp = 0;                                                           \
      int badflag = 0;                                                               \
      for (int64_t n = 0; n < N; n++) {                                              \
        T va = a[n * ia], vb = b[n * ib];                                            \
        if (c->bvalflag && (ISBADV(va, abad, ISF) || ISBADV(vb, bbad, ISF))) {       \
          badflag = 1;                                                               \
          break;                                                                     \
        }                                                                            \
        __typeof__(va * vb) prod = va * vb; /* C promotion, as the reference */     \
        tmp += (T)prod;                                                              \
      }                                                                              \
      if (badflag) {                                                                 \
        *o = c->bad[2].SYM;                                                          \
        c->setbad_out = 1;                                                           \
      } else                                                                         \
        *o = (T)tmp;                                                                 \
    }                                                                                \
  }
#define DEF_INNERS(E, CT, SYM, IP, ISF, UNS) DEF_INNER(inner_##SYM, CT, SYM, ISF)
O_REAL_TYPES(DEF_INNERS)

/* matmult: tiles of tsiz = 8*sizeof(double)/sizeof(T), Primitive.pd:211-248 */
#define DEF_MATMULT(NAME, T, SYM, ISF)                                                  \
  static void NAME(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t TT = c->ind_sizes[0], H = c->ind_sizes[1], W = c->ind_sizes[2];          \
    int64_t tsiz = 8 * sizeof(double) / sizeof(T);                                   \
    int64_t at = c->inc_sizes[0][0], ah = c->inc_sizes[0][1];                        \
    int64_t bw = c->inc_sizes[1][0], bt = c->inc_sizes[1][1];                        \
    int64_t cw = c->inc_sizes[2][0], ch = c->inc_sizes[2][1];                        \
    T abad = c->bad[0].SYM, bbad = c->bad[1].SYM, cbad = c->bad[2].SYM;              \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *A = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      const T *B = (const T *)c->base[1] + offs[1] + i0 * inc0[1];                   \
      T *C = (T *)c->base[2] + offs[2] + i0 * inc0[2];                               \
      for (int64_t ho = 0; ho < H; ho += tsiz)                                       \
        for (int64_t wo = 0; wo < W; wo += tsiz) {                                   \
          int64_t he = ho + tsiz < H ? ho + tsiz : H;                                \
          int64_t we = wo + tsiz < W ? wo + tsiz : W;                                \
          for (int64_t h = ho; h < he; h++)                                          \
            for (int64_t w = wo; w < we; w++) C[h * ch + w * cw] = 0;                \
          for (int64_t to = 0; to < TT; to += tsiz) {                                \
            int64_t te = to + tsiz < TT ? to + tsiz : TT;                            \
            for (int64_t h = ho; h < he; h++)                                        \
              for (int64_t w = wo; w < we; w++) {                                    \
                T cc = C[h * ch + w * cw];                                           \
                if (c->bvalflag && ISBADV(cc, cbad, ISF)) continue;                  \
                const T *ad = A + to * at + h * ah;                                  \
                const T *bd = B + w * bw + to * bt;                                  \
                int c_isbad = 0;                                                     \
                for (int64_t t = to; t < te; t++) {                                  \
                  if (c->bvalflag &&                                                 \
                      (ISBADV(*ad, abad, ISF) || ISBADV(*bd, bbad, ISF))) {          \
                    c_isbad = 1;                                                     \
                    break;                                                           \
                  }                                                                  \
                  cc = (T)(cc + (T)(*ad * *bd));                                     \
                  ad += at;                                                          \
                  bd += bt;                                                          \
                }                                                                    \
                if (c_isbad) {                                                       \
                  C[h * ch + w * cw] = cbad;                                         \
                  continue;                                                          \
                }                                                                    \
                C[h * ch + w * cw] = cc;                                             \
              }                                                                      \
          }                                                                          \
        }                                                                            \
    }                                                                                \
  }
#define DEF_MATMULTS(E, CT, SYM, IP, ISF, UNS) DEF_MATMULT(matmult_##SYM, CT, SYM, ISF)
O_REAL_TYPES(DEF_MATMULTS)

/* ------------------------------------------------ sort-based (Ufunc.pd:744-1115)
 * The sort is the quicksort of lib/PDL/Core/pdl.h.PL:618-640 (middle
 * element as pivot, the two scans, swap, recurse on [a,j] then [i,b]); the
 * two sub-ranges are disjoint, so recursing on the smaller one first and
 * looping on the larger gives the same array with a bounded stack. */
#define DEF_QSORT(T, SYM)                                                            \
  static void oq_##SYM(T *xx, int64_t a, int64_t b) {                               \
    while (a < b) {                                                                  \
      int64_t i = a, j = b;                                                          \
      T median = xx[(i + j) / 2];                                                    \
      do {                                                                           \
        while (xx[i] < median) i++;                                                  \
        while (median < xx[j]) j--;                                                  \
        if (i <= j) {                                                                \
          T t = xx[i]; xx[i] = xx[j]; xx[j] = t;                                     \
          i++; j--;                                                                  \
        }                                                                            \
      } while (i <= j);                                                              \
      if (j - a < b - i) {                                                           \
        if (a < j) oq_##SYM(xx, a, j);                                               \
        a = i;                                                                       \
      } else {                                                                       \
        if (i < b) oq_##SYM(xx, i, b);                                               \
        b = j;                                                                       \
      }                                                                              \
    }                                                                                \
  }                                                                                  \
  /* Ufunc.pd:745-767: the same on an index vector */                             \
  static void oqi_##SYM(const T *xx, int64_t *ix, int64_t a, int64_t b) {           \
    while (a < b) {                                                                  \
      int64_t i = a, j = b;                                                          \
      T median = xx[ix[(i + j) / 2]];                                                \
      do {                                                                           \
        while (xx[ix[i]] < median) i++;                                              \
        while (median < xx[ix[j]]) j--;                                              \
        if (i <= j) {                                                                \
          int64_t t = ix[i]; ix[i] = ix[j]; ix[j] = t;                               \
          i++; j--;                                                                  \
        }                                                                            \
      } while (i <= j);                                                              \
      if (j - a < b - i) {                                                           \
        if (a < j) oqi_##SYM(xx, ix, a, j);                                          \
        a = i;                                                                       \
      } else {                                                                       \
        if (i < b) oqi_##SYM(xx, ix, i, b);                                          \
        b = j;                                                                       \
      }                                                                              \
    }                                                                                \
  }
#define DEF_QSORTS(E, CT, SYM, IP, ISF, UNS) DEF_QSORT(CT, SYM)
O_REAL_TYPES(DEF_QSORTS)

/* the good elements of a row into tmp (all of them without bad values);
 * returns their count (Ufunc.pd:857-867, $copy_to_temp) */
#define DEF_SORTRED(T, SYM, ISF, UNS)                                                \
  static int64_t sr_copy_##SYM(octx *c, const T *a, int64_t N, int64_t ia, T *tmp) { \
    T abad = c->bad[0].SYM;                                                          \
    int64_t nn = 0;                                                                  \
    for (int64_t n = 0; n < N; n++) {                                                \
      T v = a[n * ia];                                                               \
      if (c->bvalflag && ISBADV(v, abad, ISF)) continue;                             \
      tmp[nn++] = v;                                                                 \
    }                                                                                \
    return nn;                                                                       \
  }                                                                                  \
  static void qsort_##SYM(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0], ib = c->inc_sizes[1][0];   \
    T *tmp = (T *)malloc(sizeof(T) * (N ? N : 1));                                   \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *a = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      T *b = (T *)c->base[1] + offs[1] + i0 * inc0[1];                               \
      int64_t nn = sr_copy_##SYM(c, a, N, ia, tmp);                                  \
      if (nn > 0) oq_##SYM(tmp, 0, nn - 1);                                          \
      for (int64_t n = 0; n < N; n++) b[n * ib] = n < nn ? tmp[n] : c->bad[1].SYM;   \
    }                                                                                \
    free(tmp);                                                                       \
  }                                                                                  \
  /* Ufunc.pd:1079-1112: good indices in order, bad ones from the end */          \
  static void qsorti_##SYM(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0], ib = c->inc_sizes[1][0];   \
    T abad = c->bad[0].SYM;                                                          \
    T *row = (T *)malloc(sizeof(T) * (N ? N : 1));                                   \
    int64_t *ix = (int64_t *)malloc(sizeof(int64_t) * (N ? N : 1));                 \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *a = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      int64_t *b = (int64_t *)c->base[1] + offs[1] + i0 * inc0[1];                   \
      int64_t nn = 0, nb = N - 1;                                                    \
      for (int64_t n = 0; n < N; n++) {                                              \
        row[n] = a[n * ia];                                                          \
        if (c->bvalflag && ISBADV(row[n], abad, ISF)) ix[nb--] = n;                  \
        else ix[nn++] = n;                                                           \
      }                                                                              \
      if (nn > 0) oqi_##SYM(row, ix, 0, nn - 1);                                     \
      for (int64_t n = 0; n < N; n++) b[n * ib] = ix[n];                             \
    }                                                                                \
    free(row);                                                                       \
    free(ix);                                                                        \
  }                                                                                  \
  /* Ufunc.pd:857-884: the average of the two middle elements for an even count */ \
  static void medover_##SYM(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0];                            \
    T *tmp = (T *)malloc(sizeof(T) * (N ? N : 1));                                   \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *a = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      T *b = (T *)c->base[1] + offs[1] + i0 * inc0[1];                               \
      int64_t nn = sr_copy_##SYM(c, a, N, ia, tmp);                                  \
      if (nn == 0) { *b = c->bad[1].SYM; continue; }                                 \
      nn -= 1;                                                                       \
      oq_##SYM(tmp, 0, nn);                                                          \
      int64_t nn1 = nn / 2, nn2 = nn1 + 1;                                           \
      if (nn % 2 == 0) *b = tmp[nn1];                                                \
      else *b = (T)(0.5 * (tmp[nn1] + tmp[nn2]));                                    \
    }                                                                                \
    free(tmp);                                                                       \
  }                                                                                  \
  static void oddmedover_##SYM(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0];                            \
    T *tmp = (T *)malloc(sizeof(T) * (N ? N : 1));                                   \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *a = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      T *b = (T *)c->base[1] + offs[1] + i0 * inc0[1];                               \
      int64_t nn = sr_copy_##SYM(c, a, N, ia, tmp);                                  \
      if (nn == 0) { *b = c->bad[1].SYM; continue; }                                 \
      nn -= 1;                                                                       \
      oq_##SYM(tmp, 0, nn);                                                          \
      *b = tmp[nn / 2];                                                              \
    }                                                                                \
    free(tmp);                                                                       \
  }                                                                                  \
  /* Ufunc.pd:941-973: interpolated percentile, p clipped to [0, 1] */             \
  static void pctover_##SYM(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0];                            \
    T *tmp = (T *)malloc(sizeof(T) * (N ? N : 1));                                   \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *a = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      T p = *((const T *)c->base[1] + offs[1] + i0 * inc0[1]);                       \
      T *b = (T *)c->base[2] + offs[2] + i0 * inc0[2];                               \
      int64_t nn = sr_copy_##SYM(c, a, N, ia, tmp);                                  \
      if (nn == 0) { *b = c->bad[2].SYM; continue; }                                 \
      nn -= 1;                                                                       \
      oq_##SYM(tmp, 0, nn);                                                          \
      double np = nn * p, pp1, pp2;                                                  \
      int64_t nn1 = (int64_t)(nn < (0 > np ? 0 : np) ? nn : (0 > np ? 0 : np));      \
      int64_t nn2 = (int64_t)(nn < (0 > np + 1 ? 0 : np + 1) ? nn : (0 > np + 1 ? 0 : np + 1)); \
      if (nn == 0) { pp1 = 0; pp2 = 0; }                                             \
      else { pp1 = (double)nn1 / (double)nn; pp2 = (double)nn2 / (double)nn; }       \
      if (np <= 0.0) *b = tmp[0];                                                    \
      else if (np >= nn) *b = tmp[nn];                                               \
      else if (tmp[nn2] == tmp[nn1]) *b = tmp[nn1];                                  \
      else if (p == pp1) *b = tmp[nn1];                                              \
      else if (p == pp2) *b = tmp[nn2];                                              \
      else *b = (T)((np - nn1) * (tmp[nn2] - tmp[nn1]) + tmp[nn1]);                  \
    }                                                                                \
    free(tmp);                                                                       \
  }                                                                                  \
  /* Ufunc.pd:991-1005: the nearest data value */                                  \
  static void oddpctover_##SYM(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0];                            \
    T *tmp = (T *)malloc(sizeof(T) * (N ? N : 1));                                   \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *a = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      T p = *((const T *)c->base[1] + offs[1] + i0 * inc0[1]);                       \
      T *b = (T *)c->base[2] + offs[2] + i0 * inc0[2];                               \
      int64_t nn = sr_copy_##SYM(c, a, N, ia, tmp);                                  \
      if (nn == 0) { *b = c->bad[2].SYM; continue; }                                 \
      nn -= 1;                                                                       \
      oq_##SYM(tmp, 0, nn);                                                          \
      int64_t np = (int64_t)(0 > (nn < (nn + 1) * p ? nn : (nn + 1) * p)             \
                                 ? 0 : (nn < (nn + 1) * p ? nn : (nn + 1) * p));      \
      *b = tmp[np];                                                                  \
    }                                                                                \
    free(tmp);                                                                       \
  }
#define DEF_SORTREDS(E, CT, SYM, IP, ISF, UNS) DEF_SORTRED(CT, SYM, ISF, UNS)
O_REAL_TYPES(DEF_SORTREDS)

/* Ufunc.pd:905-939: the most frequent value of the sorted row (a value must
 * repeat to count; bad values are values like any other) */
#define DEF_MODEOVER(T, SYM)                                                         \
  static void modeover_##SYM(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], ia = c->inc_sizes[0][0];                            \
    T *tmp = (T *)malloc(sizeof(T) * (N ? N : 1));                                   \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *a = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      T *o = (T *)c->base[1] + offs[1] + i0 * inc0[1];                               \
      for (int64_t n = 0; n < N; n++) tmp[n] = a[n * ia];                            \
      if (N > 0) oq_##SYM(tmp, 0, N - 1);                                            \
      int64_t i = 0, most = 0;                                                       \
      T curmode = 0, curval = 0;                                                     \
      for (int64_t n = 0; n < N; n++) {                                              \
        if (n == 0 || curval != tmp[n]) { curval = tmp[n]; i = 0; }                  \
        else { i++; if (i > most) { most = i; curmode = curval; } }                  \
      }                                                                              \
      *o = curmode;                                                                  \
    }                                                                                \
    free(tmp);                                                                       \
  }
#define DEF_MODEOVERS(E, CT, SYM, IP, ISF, UNS) DEF_MODEOVER(CT, SYM)
O_INT_TYPES(DEF_MODEOVERS)
#define modeover_F NULL
#define modeover_D NULL

/* ------------------------------------------ vector sorts (Ufunc.pd:769-851)
 * PDL_QSORTVEC: the pivot is the vector at position median_ind, compared
 * in place (not copied), and median_ind follows that vector when a swap
 * moves it; vectors compare lexicographically (pdl_cmpvec).  The two
 * ranges after a partition are disjoint, so their order does not matter. */
#define DEF_QSORTVEC(T, SYM, ISF)                                                    \
  static int ocmpvec_##SYM(const T *a, const T *b, int64_t n) {                     \
    for (int64_t i = 0; i < n; i++) {                                                \
      if (a[i] < b[i]) return -1;                                                    \
      if (a[i] > b[i]) return 1;                                                     \
    }                                                                                \
    return 0;                                                                        \
  }                                                                                  \
  static void oqv_##SYM(T *xx, int64_t n, int64_t a, int64_t b) {                   \
    int64_t i = a, j = b, med = (i + j) / 2;                                         \
    do {                                                                             \
      while (ocmpvec_##SYM(xx + n * i, xx + n * med, n) < 0) i++;                    \
      while (ocmpvec_##SYM(xx + n * j, xx + n * med, n) > 0) j--;                    \
      if (i <= j) {                                                                  \
        for (int64_t k = 0; k < n; k++) {                                            \
          T z = xx[n * i + k]; xx[n * i + k] = xx[n * j + k]; xx[n * j + k] = z;     \
        }                                                                            \
        if (med == i) med = j;                                                       \
        else if (med == j) med = i;                                                  \
        i++; j--;                                                                    \
      }                                                                              \
    } while (i <= j);                                                                \
    if (a < j) oqv_##SYM(xx, n, a, j);                                               \
    if (i < b) oqv_##SYM(xx, n, i, b);                                               \
  }                                                                                  \
  static void oqvi_##SYM(const T *xx, int64_t *ix, int64_t n, int64_t a, int64_t b) { \
    int64_t i = a, j = b, med = (i + j) / 2;                                         \
    do {                                                                             \
      while (ocmpvec_##SYM(xx + n * ix[i], xx + n * ix[med], n) < 0) i++;            \
      while (ocmpvec_##SYM(xx + n * ix[j], xx + n * ix[med], n) > 0) j--;            \
      if (i <= j) {                                                                  \
        int64_t z = ix[i]; ix[i] = ix[j]; ix[j] = z;                                 \
        if (med == i) med = j;                                                       \
        else if (med == j) med = i;                                                  \
        i++; j--;                                                                    \
      }                                                                              \
    } while (i <= j);                                                                \
    if (a < j) oqvi_##SYM(xx, ix, n, a, j);                                          \
    if (i < b) oqvi_##SYM(xx, ix, n, i, b);                                          \
  }                                                                                  \
  /* qsortvec: good vectors in order, vectors with a bad element from the end */  \
  static void qsortvec_##SYM(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], M = c->ind_sizes[1];                                \
    int64_t ian = c->inc_sizes[0][0], iam = c->inc_sizes[0][1];                      \
    int64_t ibn = c->inc_sizes[1][0], ibm = c->inc_sizes[1][1];                      \
    T abad = c->bad[0].SYM, bbad = c->bad[1].SYM;                                    \
    T *tmp = (T *)malloc(sizeof(T) * (N * M > 0 ? N * M : 1));                           \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *a = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      T *b = (T *)c->base[1] + offs[1] + i0 * inc0[1];                               \
      if (N * M == 0) continue;                                                      \
      int64_t nn = 0, nb = M - 1;                                                    \
      for (int64_t m = 0; m < M; m++) {                                              \
        int good = 1;                                                                \
        if (c->bvalflag)                                                             \
          for (int64_t k = 0; k < N; k++)                                            \
            if (ISBADV(a[k * ian + m * iam], abad, ISF)) { good = 0; break; }        \
        int64_t d = good ? nn++ : nb--;                                              \
        for (int64_t k = 0; k < N; k++) {                                            \
          T v = a[k * ian + m * iam];                                                \
          tmp[d * N + k] = (c->bvalflag && ISBADV(v, abad, ISF)) ? bbad : v;         \
        }                                                                            \
      }                                                                              \
      if (nn > 0) oqv_##SYM(tmp, N, 0, nn - 1);                                      \
      for (int64_t m = 0; m < M; m++)                                                \
        for (int64_t k = 0; k < N; k++) b[k * ibn + m * ibm] = tmp[m * N + k];       \
    }                                                                                \
    free(tmp);                                                                       \
  }                                                                                  \
  static void qsortveci_##SYM(octx *c, const int64_t *offs, int64_t n0, const int64_t *inc0) { \
    int64_t N = c->ind_sizes[0], M = c->ind_sizes[1];                                \
    int64_t ian = c->inc_sizes[0][0], iam = c->inc_sizes[0][1];                      \
    int64_t ibm = c->inc_sizes[1][0];                                                \
    T abad = c->bad[0].SYM;                                                          \
    T *tmp = (T *)malloc(sizeof(T) * (N * M > 0 ? N * M : 1));                           \
    int64_t *ix = (int64_t *)malloc(sizeof(int64_t) * (M ? M : 1));                 \
    for (int64_t i0 = 0; i0 < n0; i0++) {                                            \
      const T *a = (const T *)c->base[0] + offs[0] + i0 * inc0[0];                   \
      int64_t *b = (int64_t *)c->base[1] + offs[1] + i0 * inc0[1];                   \
      if (N * M == 0) continue;                                                      \
      int64_t nn = 0, nb = M - 1;                                                    \
      for (int64_t m = 0; m < M; m++) {                                              \
        int good = 1;                                                                \
        for (int64_t k = 0; k < N; k++) {                                            \
          T v = a[k * ian + m * iam];                                                \
          tmp[m * N + k] = v;                                                        \
          if (c->bvalflag && ISBADV(v, abad, ISF)) good = 0;                         \
        }                                                                            \
        ix[good ? nn++ : nb--] = m;                                                  \
      }                                                                              \
      if (nn > 0) oqvi_##SYM(tmp, ix, N, 0, nn - 1);                                 \
      for (int64_t m = 0; m < M; m++) b[m * ibm] = ix[m];                            \
    }                                                                                \
    free(tmp);                                                                       \
    free(ix);                                                                        \
  }
#define DEF_QSORTVECS(E, CT, SYM, IP, ISF, UNS) DEF_QSORTVEC(CT, SYM, ISF)
O_REAL_TYPES(DEF_QSORTVECS)

static body_fn pick_body(int op, int t) {
#define CASE(OPID, PFX)                                                   \
  case OPID:                                                               \
    switch (t) {                                                           \
      case PDLGB300_SB: return PFX##_A; case PDLGB300_B: return PFX##_B;   \
      case PDLGB300_S: return PFX##_S; case PDLGB300_US: return PFX##_U;   \
      case PDLGB300_L: return PFX##_L; case PDLGB300_UL: return PFX##_K;   \
      case PDLGB300_IND: return PFX##_N; case PDLGB300_ULL: return PFX##_P;\
      case PDLGB300_LL: return PFX##_Q; case PDLGB300_F: return PFX##_F;   \
      case PDLGB300_D: return PFX##_D;                                     \
    }                                                                      \
    return NULL;
  switch (op) {
    CASE(OP_SUMOVER, sumover)
    CASE(OP_DSUMOVER, dsumover)
    CASE(OP_PRODOVER, prodover)
    CASE(OP_DPRODOVER, dprodover)
    CASE(OP_CUMUSUMOVER, cumusumover)
    CASE(OP_DCUMUSUMOVER, dcumusumover)
    CASE(OP_AVERAGE, average)
    CASE(OP_DAVERAGE, daverage)
    CASE(OP_MINIMUM, minimum)
    CASE(OP_MAXIMUM, maximum)
    CASE(OP_MINIMUM_IND, minimum_ind)
    CASE(OP_MAXIMUM_IND, maximum_ind)
    CASE(OP_PLUS, plus)
    CASE(OP_MULT, mult)
    CASE(OP_INNER, inner)
    CASE(OP_MATMULT, matmult)
    CASE(OP_MINUS, minus)
    CASE(OP_DIVIDE, divide)
    CASE(OP_GT, gt)
    CASE(OP_LT, lt)
    CASE(OP_LE, le)
    CASE(OP_GE, ge)
    CASE(OP_EQ, eq)
    CASE(OP_NE, ne)
    CASE(OP_SHIFTLEFT, shiftleft)
    CASE(OP_SHIFTRIGHT, shiftright)
    CASE(OP_OR2, or2)
    CASE(OP_AND2, and2)
    CASE(OP_XOR, xor)
    CASE(OP_ANDOVER, andover)
    CASE(OP_OROVER, orover)
    CASE(OP_XOROVER, xorover)
    CASE(OP_ZCOVER, zcover)
    CASE(OP_BANDOVER, bandover)
    CASE(OP_BOROVER, borover)
    CASE(OP_BXOROVER, bxorover)
    CASE(OP_FIRSTNONZEROOVER, firstnonzeroover)
    CASE(OP_CUMUPRODOVER, cumuprodover)
    CASE(OP_DCUMUPRODOVER, dcumuprodover)
    CASE(OP_MINMAXIMUM, minmaximum)
    CASE(OP_QSORT, qsort)
    CASE(OP_QSORTI, qsorti)
    CASE(OP_MEDOVER, medover)
    CASE(OP_ODDMEDOVER, oddmedover)
    CASE(OP_PCTOVER, pctover)
    CASE(OP_ODDPCTOVER, oddpctover)
    CASE(OP_MODEOVER, modeover)
    CASE(OP_QSORTVEC, qsortvec)
    CASE(OP_QSORTVECI, qsortveci)
  }
#undef CASE
  return NULL;
}

/* --------------------------------------------------------- broadcast loop */

typedef struct {
  octx *c;
  body_fn fn;
  const obrc *b;
  int mag;          /* split broadcast dim (-1: none) */
  int64_t start, count;
} tjob;

static void run_range(octx *c, body_fn fn, const obrc *b, int mag, int64_t start,
                      int64_t count) {
  int64_t dims[MAXB], inds[MAXB] = {0}, offs[MAXP], base[MAXP];
  int np = b->npdls, nd = b->ndims;
  for (int k = 0; k < nd; k++) dims[k] = b->dims[k];
  for (int j = 0; j < np; j++) base[j] = 0;
  if (mag >= 0) {
    dims[mag] = count;
    for (int j = 0; j < np; j++) base[j] += start * b->incs[mag][j];
  }
  for (int k = 0; k < nd; k++)
    if (dims[k] == 0) return; /* empty: nothing runs, pdlbroadcast.c:560 */
  int64_t inc0[MAXP];
  for (int j = 0; j < np; j++) inc0[j] = b->incs[0][j];
  for (;;) {
    for (int j = 0; j < np; j++) {
      offs[j] = base[j];
      for (int k = 1; k < nd; k++) offs[j] += inds[k] * b->incs[k][j];
    }
    fn(c, offs, dims[0], inc0);
    int k = 1;
    for (; k < nd; k++) {
      if (++inds[k] < dims[k]) break;
      inds[k] = 0;
    }
    if (k >= nd) break;
  }
}

static void *thread_main(void *arg) {
  tjob *j = arg;
  run_range(j->c, j->fn, j->b, j->mag, j->start, j->count);
  return NULL;
}

/* pdl_find_max_pthread over the broadcast dims of the non-created pdls */
static int choose_pthread_dim(const opdef *op, pdlgb300_ndarray *const *pdls,
                              const int *creating, int target, int *nthr) {
  int best = 0, bestdim = -1;
  int64_t max_rem = 0;
  for (int j = 0; j < op->npdls && best != target; j++) {
    if (creating[j]) continue;
    for (int t = op->realdims[j]; t < pdls[j]->ndims; t++) {
      int64_t sz = pdls[j]->dims[t], rem = sz % target;
      if (rem == 0) {
        best = target;
        bestdim = t - op->realdims[j];
        break;
      }
      if (sz > best && rem > max_rem) {
        max_rem = rem;
        best = (int)(sz < target ? sz : target);
        bestdim = t - op->realdims[j];
      }
    }
  }
  *nthr = best;
  return bestdim;
}

/* ---------------------------------------------------------------- public */

const char *oracle_type_name(int t) {
  return (t >= 0 && t < PDLGB300_NTYPES) ? type_names[t] : "?";
}

void oracle_default_badvalue(int t, pdlgb300_value *out) { *out = default_bad(t); }

/* Shape null outputs and set their datatype; returns 0 or 1 with msg. */
int oracle_redodims(const char *opname, pdlgb300_ndarray **pdls, char *msg,
                    size_t msglen) {
  errbuf e = {msg, msglen};
  int op = find_op(opname);
  if (op < 0) return set_err(&e, "unknown op %s", opname);
  const opdef *d = &OPS[op];
  int tt = transtype_select(d, pdls);
  obrc b;
  if (do_redodims(&e, d, pdls, &b)) return 1;
  for (int j = d->nparents; j < d->npdls; j++)
    if (pdls[j]->state & PDLGB300_NOMYDIMS) {
      pdls[j]->datatype = out_type_for(d, tt, j);
      pdls[j]->state &= ~PDLGB300_NOMYDIMS;
    }
  return 0;
}

/* Run an op.  Null outputs are shaped and malloc'd (release with
 * oracle_free).  Inputs of another type are converted; supplied outputs
 * must already have the op's output type.  other: swap for plus/mult.
 * nthreads <= 1 runs single-threaded; otherwise the reference's
 * auto-pthread split (only when some pdl has >= 2^20 elements, the default
 * PDL_AUTOPTHREAD_SIZE of 1 Mi elements). */
/* Number of ndarray arguments (parents + children) of an op, -1 if unknown:
   callers size the argument array with it. */
int oracle_npdls(const char *opname) {
  int op = find_op(opname);
  return op < 0 ? -1 : OPS[op].npdls;
}

/* Number of input ndarrays of an op, -1 if unknown. */
int oracle_nparents(const char *opname) {
  int op = find_op(opname);
  return op < 0 ? -1 : OPS[op].nparents;
}

/* Name of an op's parameter j (the pp_def signature's), or NULL. */
const char *oracle_par_name(const char *opname, int j) {
  int op = find_op(opname);
  return op < 0 || j < 0 || j >= OPS[op].npdls ? NULL : OPS[op].par_names[j];
}

int oracle_run(const char *opname, pdlgb300_ndarray **pdls_in, const int64_t *other,
               int nthreads, char *msg, size_t msglen) {
  errbuf e = {msg, msglen};
  int op = find_op(opname);
  if (op < 0) return set_err(&e, "unknown op %s", opname);
  const opdef *d = &OPS[op];
  pdlgb300_ndarray local[MAXP], *pdls[MAXP];
  for (int j = 0; j < d->npdls; j++) {
    local[j] = *pdls_in[j];
    pdls[j] = &local[j];
  }
  if (IS_BIOP(op) && other && other[0]) {
    pdlgb300_ndarray t = local[0];
    local[0] = local[1];
    local[1] = t;
  }
  for (int j = 0; j < d->npdls; j++)
    if (!(pdls[j]->state & PDLGB300_NOMYDIMS) && pdls[j]->datatype > PDLGB300_D)
      return set_err(&e, "%s: type %s not supported", d->name,
                     oracle_type_name(pdls[j]->datatype));
  int tt = transtype_select(d, pdls);
  int creating[MAXP];
  for (int j = 0; j < d->npdls; j++)
    creating[j] = j >= d->nparents && (pdls[j]->state & PDLGB300_NOMYDIMS);
  int bvalflag = 0;
  for (int j = 0; j < d->nparents; j++)
    if (pdls[j]->state & PDLGB300_BADVAL) bvalflag = 1;
  obrc b;
  if (do_redodims(&e, d, pdls, &b)) return 1;
  void *tofree[MAXP] = {0};
  for (int j = 0; j < d->npdls; j++) {
    pdlgb300_ndarray *p = pdls[j];
    int want = j < d->nparents ? tt : out_type_for(d, tt, j);
    if (creating[j]) {
      int64_t n = 1;
      for (int i = 0; i < p->ndims; i++) n *= p->dims[i];
      p->datatype = want;
      p->data = calloc(n ? n : 1, type_size(want));
      p->has_badvalue = 0;
      p->state &= ~PDLGB300_NOMYDIMS;
      *pdls_in[j] = *p; /* the caller gets the shape and data back */
    } else if (p->datatype != want) {
      /* pdl_get_convertedpdl (pdlapi.c:141-165) makes a converttypei child:
       * its CHILD parameter is PDL_PARAM_ISIGNORE, so the child keeps
       * has_badvalue = 0 (pdlapi.c:1240-1258) and its badvalue is the new
       * type's default; COPYCONVERT maps the parent's bad elements to it
       * (pdlconv.c:163-174). */
      void *cp = converted_copy(p, want, bvalflag && (p->state & PDLGB300_BADVAL));
      pdlgb300_value nb = default_bad(want);
      tofree[j] = cp;
      int64_t dims[PDLGB300_MAXDIMS];
      memcpy(dims, p->dims, sizeof dims);
      int nd = p->ndims;
      uint32_t st = p->state;
      oracle_ndarray_init(p, want, nd, dims, cp, NULL);
      p->state = st;
      p->has_badvalue = 0;
      p->badvalue.type = want;
      p->badvalue.value = nb;
      /* strides changed: recompute the broadcast increments */
      if (do_redodims(&e, d, pdls, &b)) return 1;
    }
  }
  octx c;
  memset(&c, 0, sizeof c);
  c.op = op;
  c.ttype = tt;
  c.bvalflag = bvalflag;
  c.other = other;
  for (int j = 0; j < d->npdls; j++) {
    c.base[j] = (char *)pdls[j]->data + pdls[j]->offs * (int64_t)type_size(pdls[j]->datatype);
    c.statebad[j] = !!(pdls[j]->state & PDLGB300_BADVAL);
    c.bad[j] = badval_of(pdls[j]);
    for (int k = 0; k < 2; k++) c.inc_sizes[j][k] = b.inc_sizes[j][k];
  }
  for (int k = 0; k < 3; k++) c.ind_sizes[k] = b.ind_sizes[k];
  body_fn fn = pick_body(op, tt);
  if (!fn) return set_err(&e, "no body for %s type %d", d->name, tt);
  if (op == OP_MEDOVER || op == OP_ODDMEDOVER || op == OP_PCTOVER || op == OP_ODDPCTOVER) {
    /* Ufunc.pd:857-858, $copy_to_temp: $CROAK("cannot process empty ndarray") */
    int64_t nv = 1;
    for (int k = 0; k < pdls[0]->ndims; k++) nv *= pdls[0]->dims[k];
    if (nv == 0) return set_err(&e, "Error in %s:cannot process empty ndarray", d->name);
  }

  int64_t maxvals = 0;
  for (int j = 0; j < d->npdls; j++) {
    int64_t n = 1;
    for (int i = 0; i < pdls[j]->ndims; i++) n *= pdls[j]->dims[i];
    if (n > maxvals) maxvals = n;
  }
  int nthr = 0, mag = -1;
  if (nthreads > 1 && maxvals >= (1 << 20))
    mag = choose_pthread_dim(d, pdls, creating, nthreads, &nthr);
  if (mag < 0 || nthr <= 1 || mag >= b.ndims) {
    run_range(&c, fn, &b, -1, 0, 0);
  } else {
    int64_t md = b.dims[mag], n1 = md / nthr, n2 = md % nthr;
    pthread_t th[256];
    tjob jobs[256];
    if (nthr > 256) nthr = 256;
    for (int t = 0; t < nthr; t++) {
      int64_t start = t * n1 + (t < n2 ? t : n2);
      int64_t cnt = n1 + (t < n2 ? 1 : 0);
      jobs[t] = (tjob){&c, fn, &b, mag, start, cnt};
      pthread_create(&th[t], NULL, thread_main, &jobs[t]);
    }
    for (int t = 0; t < nthr; t++) pthread_join(th[t], NULL);
  }
  /* badflag propagation (pdlapi.c:806-808) and PDLSTATESETBAD */
  for (int j = d->nparents; j < d->npdls; j++) {
    if (bvalflag || c.setbad_out) pdls_in[j]->state |= PDLGB300_BADVAL;
  }
  /* A supplied output of another type got a converted child above; its
   * values flow back into the output (converttypei's writeback, pdlconv.c
   * COPYCONVERT), a bad value becoming the output's badvalue. */
  for (int j = d->nparents; j < d->npdls; j++) {
    if (!tofree[j]) continue;
    const pdlgb300_ndarray *u = pdls_in[j], *w = pdls[j];
    int64_t n = 1;
    for (int i = 0; i < u->ndims; i++) n *= u->dims[i];
    const size_t ws = type_size(w->datatype), us = type_size(u->datatype);
    const pdlgb300_value wb = badval_of(w), ub = badval_of(u);
    int64_t idx[PDLGB300_MAXDIMS] = {0};
    for (int64_t k = 0; k < n; k++) {
      int64_t off = u->offs;
      for (int i = 0; i < u->ndims; i++) off += idx[i] * u->incs[i];
      char *dst = (char *)u->data + off * (int64_t)us;
      const char *src = (const char *)w->data + k * (int64_t)ws;
      if (bvalflag && value_isbad(w->datatype, src, wb))
        store_value(u->datatype, dst, ub);
      else
        convert_elem(w->datatype, src, u->datatype, dst);
      for (int i = 0; i < u->ndims; i++) {
        if (++idx[i] < u->dims[i]) break;
        idx[i] = 0;
      }
    }
  }
  for (int j = 0; j < d->npdls; j++) free(tofree[j]);
  return 0;
}

void oracle_free(void *p) { free(p); }

/* A contiguous descriptor (PDL's default increments). */
void oracle_ndarray_init(pdlgb300_ndarray *x, int32_t datatype, int32_t ndims,
                         const int64_t *dims, void *data, void *ddata) {
  memset(x, 0, sizeof *x);
  x->datatype = datatype;
  x->ndims = ndims;
  x->badvalue.type = -1;
  for (int i = 0; i < ndims; i++) x->dims[i] = dims[i];
  default_incs(x);
  x->data = data;
  x->ddata = ddata;
}

/* ---------------------------------------------------- hand-derived adjoints
 * Gradients of the hot-path ops written out by hand, in double precision,
 * for contiguous float64 operands (the checker of the GPU adjoint kernels).
 * Shapes follow PDL dims (dim 0 fastest). */

/* ga(n, R) = gb(R) */
void oracle_sumover_bwd(const double *gb, double *ga, int64_t n, int64_t R) {
  for (int64_t r = 0; r < R; r++)
    for (int64_t i = 0; i < n; i++) ga[r * n + i] = gb[r];
}

void oracle_average_bwd(const double *gb, double *ga, int64_t n, int64_t R) {
  for (int64_t r = 0; r < R; r++)
    for (int64_t i = 0; i < n; i++) ga[r * n + i] = gb[r] / (double)n;
}

/* c(w,h,B) = sum_t a(t,h,Ba) b(w,t,Bb); batch broadcast when Ba or Bb is 1.
 * ga(t,h,Ba) = sum_w gc(w,h) b(w,t); gb(w,t,Bb) = sum_h gc(w,h) a(t,h). */
void oracle_matmult_bwd(const double *gc, const double *a, const double *b,
                        double *ga, double *gb, int64_t T, int64_t H, int64_t W,
                        int64_t B, int64_t Ba, int64_t Bb) {
  if (ga) memset(ga, 0, sizeof(double) * T * H * Ba);
  if (gb) memset(gb, 0, sizeof(double) * W * T * Bb);
  for (int64_t z = 0; z < B; z++) {
    const double *A = a + (Ba == 1 ? 0 : z) * T * H;
    const double *Bm = b + (Bb == 1 ? 0 : z) * W * T;
    const double *G = gc + z * W * H;
    double *GA = ga ? ga + (Ba == 1 ? 0 : z) * T * H : NULL;
    double *GB = gb ? gb + (Bb == 1 ? 0 : z) * W * T : NULL;
    for (int64_t h = 0; h < H; h++)
      for (int64_t t = 0; t < T; t++) {
        double s = 0;
        for (int64_t w = 0; w < W; w++) s += G[h * W + w] * Bm[t * W + w];
        if (GA) GA[h * T + t] += s;
      }
    if (GB)
      for (int64_t t = 0; t < T; t++)
        for (int64_t w = 0; w < W; w++) {
          double s = 0;
          for (int64_t h = 0; h < H; h++) s += G[h * W + w] * A[h * T + t];
          GB[t * W + w] += s;
        }
  }
}
