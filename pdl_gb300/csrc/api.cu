// api.cpp -- the C ABI of libpdlgb300: op vtables, the launch planner, device
// staging, type conversion and the per-op dispatch.
//
// The planner restates PDL's broadcast engine for implicit broadcasting:
// dim unification and increments (pdl_initbroadcaststruct /
// pdl_broadcast_dim_checks, lib/PDL/Core/pdlbroadcast.c:275-488), the real-
// dim checks (pdl_dim_checks :211-273), creation of null outputs
// (pdl_broadcast_create_parameter :490-523, pdl_redodims_default
// lib/PDL/Core/pdlapi.c:829-869), with the error text of pdl_param_error
// (lib/PDL/Core/pdlutil.c:65-147).  Instead of an odometer walked by the
// CPU (pdl_broadcast_nd_step, pdlbroadcast.h:72-84) the broadcast dims are
// collapsed (adjacent dims whose increments chain for every ndarray merge)
// and mapped onto the CUDA grid.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "biop.cuh"

// ================================================================ helpers
namespace {
thread_local std::string tl_msg;
thread_local pdlgb300_launch_info tl_info;
thread_local pdlgb300_launch_info tl_last;
cudaStream_t g_stream = nullptr;
int g_timing = 0;
int64_t g_opt_mm_mode = PDLGB300_MATMULT_BF16X6;
int64_t g_opt_comp = 1;
int64_t g_opt_debug = 0;
int g_nsm = 0;

pdlgb300_value g_defbad[PDLGB300_NTYPES];
std::once_flag g_defbad_once;

void init_defbad() {
  memset(g_defbad, 0, sizeof g_defbad);
  g_defbad[PDLGB300_SB].A = INT8_MIN;
  g_defbad[PDLGB300_B].B = UINT8_MAX;
  g_defbad[PDLGB300_S].S = INT16_MIN;
  g_defbad[PDLGB300_US].U = UINT16_MAX;
  g_defbad[PDLGB300_L].L = INT32_MIN;
  g_defbad[PDLGB300_UL].K = UINT32_MAX;
  g_defbad[PDLGB300_IND].N = INT64_MIN;
  g_defbad[PDLGB300_ULL].P = UINT64_MAX;
  g_defbad[PDLGB300_LL].Q = INT64_MIN;
  g_defbad[PDLGB300_F].F = -3.40282346638528859812e+38F;
  g_defbad[PDLGB300_D].D = -1.79769313486231570815e+308;
}
pdlgb300_value defbad(int t) {
  std::call_once(g_defbad_once, init_defbad);
  return g_defbad[t];
}
const char *TNAMES[] = {"sbyte", "byte", "short", "ushort", "long", "ulong",
                        "indx", "ulonglong", "longlong", "float", "double",
                        "ldouble", "cfloat", "cdouble", "cldouble"};
const size_t TSIZES[] = {1, 1, 2, 2, 4, 4, 8, 8, 8, 4, 8, 16, 8, 16, 32};
}  // namespace

namespace pgh {
pdlgb300_error ok() { return pdlgb300_error{0, 0, nullptr}; }
static pdlgb300_error verr(int kind, const char *fmt, va_list ap) {
  char buf[8192];
  vsnprintf(buf, sizeof buf, fmt, ap);
  tl_msg = buf;
  return pdlgb300_error{kind, 0, tl_msg.c_str()};
}
pdlgb300_error err(int kind, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  pdlgb300_error e = verr(kind, fmt, ap);
  va_end(ap);
  return e;
}
cudaStream_t stream() { return g_stream; }
bool cuda_check(cudaError_t e, pdlgb300_error *out, const char *what) {
  if (e == cudaSuccess) return true;
  *out = err(PDLGB300_EFATAL, "CUDA error in %s: %s", what, cudaGetErrorString(e));
  return false;
}
void record_kernel(const char *name, int64_t grid, int64_t block) {
  tl_info.nlaunches++;
  snprintf(tl_info.kernel, sizeof tl_info.kernel, "%s", name);
  tl_info.grid = grid;
  tl_info.block = block;
}
int num_sms() {
  if (!g_nsm) {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0)
      g_nsm = n;
    else
      g_nsm = pg::NSM_GB300;
  }
  return g_nsm;
}
}  // namespace pgh

using pgh::err;
using pgh::ok;
using namespace pg;

#define RET_IF(e) do { pdlgb300_error _e = (e); if (_e.error) return _e; } while (0)

// ================================================================ vtables
namespace {

enum OpId {
  O_SUMOVER, O_DSUMOVER, O_PRODOVER, O_DPRODOVER, O_CUMUSUMOVER, O_DCUMUSUMOVER,
  O_AVERAGE, O_DAVERAGE, O_MINIMUM, O_MAXIMUM, O_MINIMUM_IND, O_MAXIMUM_IND,
  O_PLUS, O_MULT, O_INNER, O_MATMULT, O_SMP,
  O_MINUS, O_DIVIDE, O_GT, O_LT, O_LE, O_GE, O_EQ, O_NE,
  O_SHIFTLEFT, O_SHIFTRIGHT, O_OR2, O_AND2, O_XOR,
  O_ANDOVER, O_OROVER, O_XOROVER, O_ZCOVER, O_BANDOVER, O_BOROVER, O_BXOROVER,
  O_FIRSTNONZEROOVER, O_CUMUPRODOVER, O_DCUMUPRODOVER, O_MINMAXIMUM,
  O_QSORT, O_QSORTI, O_MEDOVER, O_ODDMEDOVER, O_PCTOVER, O_ODDPCTOVER, O_MODEOVER,
  O_QSORTVEC, O_QSORTVECI, O_NOPS
};

// binary ops (a(); b(); [o]c(); int swap) and their kernel codes
bool is_biop(int op) { return op == O_PLUS || op == O_MULT || (op >= O_MINUS && op <= O_XOR); }
int biop_code_of(int op) {
  switch (op) {
    case O_PLUS: return 0;
    case O_MULT: return 1;
    default: return 2 + (op - O_MINUS);  // minus, divide, gt .. xor in kernel order
  }
}

const int32_t GENTYPES[] = {PDLGB300_SB, PDLGB300_B,   PDLGB300_S,   PDLGB300_US,
                            PDLGB300_L,  PDLGB300_UL,  PDLGB300_IND, PDLGB300_ULL,
                            PDLGB300_LL, PDLGB300_F,   PDLGB300_D,   PDLGB300_LD,
                            PDLGB300_CF, PDLGB300_CD,  PDLGB300_CLD, -1};
// GenericTypes of the bit ops: the integer types (lib/PDL/Ops.pd:296-307)
const int32_t INTTYPES[] = {PDLGB300_SB, PDLGB300_B,   PDLGB300_S,   PDLGB300_US, PDLGB300_L,
                            PDLGB300_UL, PDLGB300_IND, PDLGB300_ULL, PDLGB300_LL, -1};
const int32_t REALTYPES[] = {PDLGB300_SB, PDLGB300_B,  PDLGB300_S,   PDLGB300_US,
                             PDLGB300_L,  PDLGB300_UL, PDLGB300_IND, PDLGB300_ULL,
                             PDLGB300_LL, PDLGB300_F,  PDLGB300_D,   PDLGB300_LD, -1};

#define OUT_C (PDLGB300_PARAM_ISOUT | PDLGB300_PARAM_ISCREAT)
#define OUT_T (OUT_C | PDLGB300_PARAM_ISTYPED)
#define OUT_TP (OUT_T | PDLGB300_PARAM_ISTPLUS)

const char *const N_AB[] = {"a", "b"};
const char *const N_AC[] = {"a", "c"};
const char *const N_ABC[] = {"a", "b", "c"};
const char *const N_ABDC[] = {"a", "b", "d", "c"};
const char *const I_N[] = {"n"};
const char *const N_MM4[] = {"a", "cmin", "cmax", "cmin_ind", "cmax_ind"};
const char *const I_THW[] = {"t", "h", "w"};
const char *const N_AI[] = {"a", "indx"};
const char *const N_APB[] = {"a", "p", "b"};
const char *const N_DO[] = {"data", "out"};
const char *const I_NM[] = {"n", "m"};

const int32_t RD_10[] = {1, 0}, RD_11[] = {1, 1}, RD_000[] = {0, 0, 0},
              RD_110[] = {1, 1, 0}, RD_222[] = {2, 2, 2}, RD_1110[] = {1, 1, 1, 0};
const int32_t F_TP[] = {0, OUT_TP}, F_T[] = {0, OUT_T}, F_C[] = {0, OUT_C},
              F_ABC[] = {0, 0, OUT_C}, F_SMP[] = {0, 0, 0, OUT_TP};
const int32_t PT_L[] = {-1, PDLGB300_L}, PT_D[] = {-1, PDLGB300_D},
              PT_N[] = {-1, PDLGB300_IND}, PT_NONE[] = {-1, -1, -1, -1},
              PT_SMP[] = {-1, -1, -1, PDLGB300_L};
const int32_t RD_10000[] = {1, 0, 0, 0, 0}, F_MM4[] = {0, OUT_C, OUT_C, OUT_T, OUT_T},
              PT_MM4[] = {-1, -1, -1, PDLGB300_IND, PDLGB300_IND};
const int32_t RD_100[] = {1, 0, 0}, F_APB[] = {0, 0, OUT_C};
const int32_t RD_22[] = {2, 2}, RD_21[] = {2, 1}, ID_NMNM[] = {0, 1, 0, 1}, ID_NMM[] = {0, 1, 1};
const int32_t ID_N0[] = {0}, ID_NN[] = {0, 0}, ID_NNN[] = {0, 0, 0},
              ID_MM[] = {0, 1, 2, 0, 2, 1}, ID_NONE[] = {0};

const pdlgb300_vtable VT[O_NOPS] = {
    {"sumover", 2, 1, 1, 0, N_AB, RD_10, F_TP, PT_L, ID_N0, I_N, GENTYPES},
    {"dsumover", 2, 1, 1, 0, N_AB, RD_10, F_T, PT_D, ID_N0, I_N, REALTYPES},
    {"prodover", 2, 1, 1, 0, N_AB, RD_10, F_TP, PT_L, ID_N0, I_N, GENTYPES},
    {"dprodover", 2, 1, 1, 0, N_AB, RD_10, F_T, PT_D, ID_N0, I_N, REALTYPES},
    {"cumusumover", 2, 1, 1, 0, N_AB, RD_11, F_TP, PT_L, ID_NN, I_N, GENTYPES},
    {"dcumusumover", 2, 1, 1, 0, N_AB, RD_11, F_T, PT_D, ID_NN, I_N, REALTYPES},
    {"average", 2, 1, 1, 0, N_AB, RD_10, F_TP, PT_L, ID_N0, I_N, REALTYPES},
    {"daverage", 2, 1, 1, 0, N_AB, RD_10, F_T, PT_D, ID_N0, I_N, REALTYPES},
    {"minimum", 2, 1, 1, 0, N_AC, RD_10, F_C, PT_NONE, ID_N0, I_N, REALTYPES},
    {"maximum", 2, 1, 1, 0, N_AC, RD_10, F_C, PT_NONE, ID_N0, I_N, REALTYPES},
    {"minimum_ind", 2, 1, 1, 0, N_AC, RD_10, F_T, PT_N, ID_N0, I_N, REALTYPES},
    {"maximum_ind", 2, 1, 1, 0, N_AC, RD_10, F_T, PT_N, ID_N0, I_N, REALTYPES},
    {"plus", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, GENTYPES},
    {"mult", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, GENTYPES},
    {"inner", 3, 2, 1, 0, N_ABC, RD_110, F_ABC, PT_NONE, ID_NN, I_N, GENTYPES},
    {"matmult", 3, 2, 3, 0, N_ABC, RD_222, F_ABC, PT_NONE, ID_MM, I_THW, GENTYPES},
    {"sumover_mult_plus", 4, 3, 1, 0, N_ABDC, RD_1110, F_SMP, PT_SMP, ID_NNN, I_N, GENTYPES},
    {"minus", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, GENTYPES},
    {"divide", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, GENTYPES},
    {"gt", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, GENTYPES},
    {"lt", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, GENTYPES},
    {"le", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, GENTYPES},
    {"ge", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, GENTYPES},
    {"eq", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, GENTYPES},
    {"ne", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, GENTYPES},
    {"shiftleft", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, INTTYPES},
    {"shiftright", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, INTTYPES},
    {"or2", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, INTTYPES},
    {"and2", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, INTTYPES},
    {"xor", 3, 2, 0, 1, N_ABC, RD_000, F_ABC, PT_NONE, ID_NONE, nullptr, INTTYPES},
    // lib/PDL/Ufunc.pd:143-187: a(n); [o] b() in a's type
    {"andover", 2, 1, 1, 0, N_AB, RD_10, F_C, PT_NONE, ID_N0, I_N, GENTYPES},
    {"orover", 2, 1, 1, 0, N_AB, RD_10, F_C, PT_NONE, ID_N0, I_N, GENTYPES},
    {"xorover", 2, 1, 1, 0, N_AB, RD_10, F_C, PT_NONE, ID_N0, I_N, GENTYPES},
    {"zcover", 2, 1, 1, 0, N_AB, RD_10, F_C, PT_NONE, ID_N0, I_N, GENTYPES},
    {"bandover", 2, 1, 1, 0, N_AB, RD_10, F_C, PT_NONE, ID_N0, I_N, INTTYPES},
    {"borover", 2, 1, 1, 0, N_AB, RD_10, F_C, PT_NONE, ID_N0, I_N, INTTYPES},
    {"bxorover", 2, 1, 1, 0, N_AB, RD_10, F_C, PT_NONE, ID_N0, I_N, INTTYPES},
    {"firstnonzeroover", 2, 1, 1, 0, N_AB, RD_10, F_C, PT_NONE, ID_N0, I_N, GENTYPES},
    // lib/PDL/Ufunc.pd:120-140 with `*=`: a(n); int+ [o]b(n) / double [o]b(n)
    {"cumuprodover", 2, 1, 1, 0, N_AB, RD_11, F_TP, PT_L, ID_NN, I_N, GENTYPES},
    {"dcumuprodover", 2, 1, 1, 0, N_AB, RD_11, F_T, PT_D, ID_NN, I_N, REALTYPES},
    // lib/PDL/Ufunc.pd:563-613
    {"minmaximum", 5, 1, 1, 0, N_MM4, RD_10000, F_MM4, PT_MM4, ID_N0, I_N, REALTYPES},
    // lib/PDL/Ufunc.pd:878-1112: the sort-based functions (real types;
    // modeover the integer types)
    {"qsort", 2, 1, 1, 0, N_AB, RD_11, F_C, PT_NONE, ID_NN, I_N, REALTYPES},
    {"qsorti", 2, 1, 1, 0, N_AI, RD_11, F_T, PT_N, ID_NN, I_N, REALTYPES},
    {"medover", 2, 1, 1, 0, N_AB, RD_10, F_C, PT_NONE, ID_N0, I_N, REALTYPES},
    {"oddmedover", 2, 1, 1, 0, N_AB, RD_10, F_C, PT_NONE, ID_N0, I_N, REALTYPES},
    {"pctover", 3, 2, 1, 0, N_APB, RD_100, F_APB, PT_NONE, ID_NNN, I_N, REALTYPES},
    {"oddpctover", 3, 2, 1, 0, N_APB, RD_100, F_APB, PT_NONE, ID_NNN, I_N, REALTYPES},
    {"modeover", 2, 1, 1, 0, N_DO, RD_10, F_C, PT_NONE, ID_N0, I_N, INTTYPES},
    // lib/PDL/Ufunc.pd:1115-1231: a(n,m); [o]b(n,m) / indx [o]indx(m)
    {"qsortvec", 2, 1, 2, 0, N_AB, RD_22, F_C, PT_NONE, ID_NMNM, I_NM, REALTYPES},
    {"qsortveci", 2, 1, 2, 0, N_AI, RD_21, F_T, PT_N, ID_NMM, I_NM, REALTYPES},
};

int op_of(const pdlgb300_vtable *vt) {
  for (int i = 0; i < O_NOPS; i++)
    if (vt == &VT[i]) return i;
  return -1;
}

// index id of real dim j of parameter i
int ind_id(const pdlgb300_vtable *vt, int i, int j) {
  int k = 0;
  for (int p = 0; p < i; p++) k += vt->par_realdims[p];
  return vt->ind_ids[k + j];
}

// ================================================================ planner

struct Brc {
  int np = 0, nimpl = 0, ndims = 0;
  int creating[MAXP] = {0};
  int64_t dims[MAXB];
  int64_t incs[MAXB][MAXP];  // PDL_BRC_INC(incs, npdls, p, d) == incs[d][p]
  int64_t ind_sizes[4];
  int64_t inc_sizes[MAXP][2];
};

int64_t nvals(const pdlgb300_ndarray *x) {
  int64_t n = 1;
  for (int i = 0; i < x->ndims; i++) n *= x->dims[i];
  return n;
}

void default_incs(pdlgb300_ndarray *x) {
  int64_t s = 1;
  for (int i = 0; i < x->ndims; i++) {
    x->incs[i] = s;
    s *= x->dims[i];
  }
}

// The package that defines an op: pdl_param_error names the op by its
// vtable name, which is package-qualified ("PDL::Ops::plus").
const char *op_package(const char *name) {
  static const char *const ops[] = {"plus", "mult", "minus", "divide", "gt", "lt", "le", "ge",
                                    "eq", "ne", "shiftleft", "shiftright", "or2", "and2",
                                    "xor"};
  for (const char *o : ops)
    if (!strcmp(name, o)) return "PDL::Ops::";
  if (!strcmp(name, "inner") || !strcmp(name, "matmult")) return "PDL::Primitive::";
  if (!strcmp(name, "sumover_mult_plus")) return "";  // no PDL counterpart
  return "PDL::Ufunc::";
}

// pdl_param_error's message: "PDL::Pkg::op(a,b,c): parameter 'b': <msg>"
// followed by the table of active and broadcast dims.
pdlgb300_error param_error(const pdlgb300_vtable *vt, int param, pdlgb300_ndarray *const *pdls,
                           int nimpl, const int *creating, const char *fmt, ...) {
  std::string m;
  char tmp[1024];
  if (param < 0 || param >= vt->npdls) {
    m = "ERROR: UNKNOWN PARAMETER";
  } else {
    m = std::string(op_package(vt->name)) + vt->name + "(";
    for (int i = 0; i < vt->npdls; i++) {
      m += vt->par_names[i];
      if (i < vt->npdls - 1) m += ",";
    }
    m += std::string("): parameter '") + vt->par_names[param] + "': ";
  }
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(tmp, sizeof tmp, fmt, ap);
  va_end(ap);
  m += tmp;
  snprintf(tmp, sizeof tmp, "\nThere are %d PDLs in the expression; %d broadcast dim%s.\n",
           vt->npdls, nimpl, nimpl == 1 ? "" : "s");
  m += tmp;
  int maxreal = 0;
  for (int i = 0; i < vt->npdls; i++) maxreal = std::max(maxreal, (int)vt->par_realdims[i]);
  m += "   PDL IN EXPR.    ";
  if (maxreal > 0) {
    snprintf(tmp, sizeof tmp, "%*s", 8 * maxreal + 3, "ACTIVE DIMS | ");
    m += tmp;
  }
  m += "BROADCAST DIMS\n";
  for (int i = 0; i < vt->npdls; i++) {
    snprintf(tmp, sizeof tmp, "   #%3d (%s", i, creating[i] ? "null)\n" : "normal): ");
    m += tmp;
    if (creating[i]) continue;
    if (maxreal == 1) m += "    ";
    for (int j = 0; j < maxreal - vt->par_realdims[i]; j++) {
      snprintf(tmp, sizeof tmp, "%8s", " ");
      m += tmp;
    }
    for (int j = 0; j < vt->par_realdims[i]; j++) {
      snprintf(tmp, sizeof tmp, "%8lld", (long long)(j < pdls[i]->ndims ? pdls[i]->dims[j] : 1));
      m += tmp;
    }
    if (maxreal) m += " | ";
    for (int j = 0; j < nimpl && j + vt->par_realdims[i] < pdls[i]->ndims; j++) {
      snprintf(tmp, sizeof tmp, "%8lld", (long long)pdls[i]->dims[j + vt->par_realdims[i]]);
      m += tmp;
    }
    m += "\n";
  }
  return err(PDLGB300_EUSERERROR, "%s", m.c_str());
}

// A dummy (broadcast) dim of a view has increment 0.  An empty ndarray's
// default increments can be 0 too, and it holds nothing to write, so it is
// never treated as a dummy.
bool dummy_dim(const pdlgb300_ndarray *p, int d) {
  if (d >= p->ndims || p->incs[d] != 0) return false;
  for (int i = 0; i < p->ndims; i++)
    if (p->dims[i] == 0) return false;
  return true;
}

// Broadcast dims and increments, real-dim sizes, and the shapes of null
// outputs (which get default increments).
pdlgb300_error plan_broadcast(const pdlgb300_vtable *vt, pdlgb300_ndarray *const *pdls, Brc &b) {
  const int np = vt->npdls;
  b = Brc();
  b.np = np;
  int nimpl = 0;
  for (int j = 0; j < np; j++) {
    b.creating[j] = j >= vt->nparents && (pdls[j]->state & PDLGB300_NOMYDIMS);
    if (j < vt->nparents && (pdls[j]->state & PDLGB300_NOMYDIMS))
      return err(PDLGB300_EUSERERROR, "Error in %s%s: input parameter '%s' is null",
                 op_package(vt->name), vt->name, vt->par_names[j]);
    if (b.creating[j]) continue;
    if (pdls[j]->ndims < 0 || pdls[j]->ndims > PDLGB300_MAXDIMS)
      return err(PDLGB300_EUSERERROR, "%s: parameter '%s' has %d dims (max %d)", vt->name,
                 vt->par_names[j], pdls[j]->ndims, PDLGB300_MAXDIMS);
    nimpl = std::max(nimpl, pdls[j]->ndims - (int)vt->par_realdims[j]);
  }
  b.nimpl = nimpl;
  b.ndims = std::max(nimpl, 2);
  for (int k = 0; k < MAXB; k++) {
    b.dims[k] = 1;
    for (int p = 0; p < MAXP; p++) b.incs[k][p] = 0;
  }
  // implicit broadcast dims: size-1 dims stretch, other sizes must agree,
  // outputs may not be stretched
  for (int nth = 0; nth < nimpl; nth++) {
    for (int j = 0; j < np; j++) {
      if (b.creating[j]) continue;
      const pdlgb300_ndarray *p = pdls[j];
      const bool out = j >= vt->nparents;
      const int rd = vt->par_realdims[j];
      if (nth >= p->ndims - rd) {
        if (out && b.dims[nth] != 1)
          return param_error(vt, nth, pdls, nimpl, b.creating,
                             "implicit dim %d size %lld, can't broadcast over output ndarray with size > 1",
                             nth, (long long)b.dims[nth]);
        continue;
      }
      const int64_t cur = p->dims[nth + rd];
      if (out && cur == 1 && cur != b.dims[nth])
        return param_error(vt, nth, pdls, nimpl, b.creating,
                           "implicit dim %d size %lld, but dim has size %lld", nth,
                           (long long)b.dims[nth], (long long)cur);
      if (out && cur != 1 && dummy_dim(p, nth + rd))
        return param_error(vt, nth, pdls, nimpl, b.creating,
                           "implicit dim %d size %lld, but dim is dummy", nth,
                           (long long)b.dims[nth]);
      if (cur == 1) continue;
      if (b.dims[nth] == 1) b.dims[nth] = cur;
      else if (b.dims[nth] != cur)
        return param_error(vt, j, pdls, nimpl, b.creating,
                           "Mismatched implicit broadcast dimension %d: size %lld vs. %lld", nth,
                           (long long)b.dims[nth], (long long)cur);
      b.incs[nth][j] = p->incs[nth + rd];
    }
  }
  // real (named) dims
  for (int k = 0; k < 4; k++) b.ind_sizes[k] = -1;
  for (int i = 0; i < np; i++) {
    if (b.creating[i]) continue;
    const pdlgb300_ndarray *p = pdls[i];
    const bool out = i >= vt->nparents;
    for (int j = 0; j < vt->par_realdims[i]; j++) {
      const int id = ind_id(vt, i, j);
      int64_t sz = b.ind_sizes[id];
      const bool has = j < p->ndims;
      if (!has && sz == -1) sz = b.ind_sizes[id] = 1;
      if (sz == -1 || (has && sz == 1)) {
        b.ind_sizes[id] = has ? p->dims[j] : 1;
        continue;
      }
      if (!has && out && sz != 1)
        return param_error(vt, i, pdls, nimpl, b.creating,
                           "index '%s' size %lld, can't broadcast over output ndarray with size > 1",
                           vt->ind_names[id], (long long)sz);
      if (out && sz != 1 && dummy_dim(p, j))
        return param_error(vt, i, pdls, nimpl, b.creating,
                           "index '%s' size %lld, can't broadcast over dummy dim with size > 1",
                           vt->ind_names[id], (long long)sz);
      if (has && sz != p->dims[j] && (out || p->dims[j] != 1))
        return param_error(vt, i, pdls, nimpl, b.creating,
                           "index '%s' size %lld, but ndarray dim has size %lld", vt->ind_names[id],
                           (long long)sz, (long long)p->dims[j]);
    }
  }
  for (int k = 0; k < 4; k++)
    if (b.ind_sizes[k] < 0) b.ind_sizes[k] = 1;
  // null outputs: real dims then the broadcast dims
  for (int j = 0; j < np; j++) {
    if (!b.creating[j]) continue;
    pdlgb300_ndarray *p = pdls[j];
    const int rd = vt->par_realdims[j];
    if (rd + nimpl > PDLGB300_MAXDIMS)
      return err(PDLGB300_EUSERERROR, "%s: output would have more than %d dims", vt->name,
                 PDLGB300_MAXDIMS);
    p->ndims = rd + nimpl;
    for (int i = 0; i < rd; i++) p->dims[i] = b.ind_sizes[ind_id(vt, j, i)];
    for (int i = 0; i < nimpl; i++) p->dims[rd + i] = b.dims[i];
    default_incs(p);
    p->offs = 0;
    for (int i = 0; i < nimpl; i++) b.incs[i][j] = p->incs[rd + i];
  }
  for (int i = 0; i < np; i++) {
    const pdlgb300_ndarray *p = pdls[i];
    for (int j = 0; j < vt->par_realdims[i] && j < 2; j++)
      b.inc_sizes[i][j] = (p->ndims <= j || p->dims[j] <= 1) ? 0 : p->incs[j];
  }
  return ok();
}

// Collapse broadcast dims into a kernel Loop over the given ndarrays.
Loop collapse(const Brc &b, int np_loop, const int *which) {
  Loop L;
  memset(&L, 0, sizeof L);
  L.np = np_loop;
  int nd = 0;
  int64_t total = 1;
  for (int k = 0; k < b.ndims; k++) {
    const int64_t s = b.dims[k];
    total *= s;
    if (s == 1) continue;
    if (nd > 0) {
      bool merge = true;
      for (int p = 0; p < np_loop; p++)
        if (b.incs[k][which[p]] != L.inc[p][nd - 1] * L.size[nd - 1]) merge = false;
      if (merge) {
        L.size[nd - 1] *= s;
        continue;
      }
    }
    L.size[nd] = s;
    for (int p = 0; p < np_loop; p++) L.inc[p][nd] = b.incs[k][which[p]];
    nd++;
  }
  if (nd == 0) {
    L.size[0] = 1;
    nd = 1;
  }
  L.nd = nd;
  L.total = total;
  return L;
}

// --------------------------------------------------------------- staging

struct Operand {
  char *dev = nullptr;    // device address of element offs (the view origin)
  void *owned = nullptr;  // device allocation to release
  bool to_host = false;   // copy the span back to host memory after the op
  char *host_lo = nullptr;
  char *dev_lo = nullptr;
  size_t span_bytes = 0;
};

void span_of(const pdlgb300_ndarray *x, int64_t &lo, int64_t &hi) {
  lo = hi = x->offs;
  for (int i = 0; i < x->ndims; i++) {
    if (x->dims[i] == 0) { lo = 0; hi = -1; return; }
    int64_t ext = (x->dims[i] - 1) * x->incs[i];
    if (ext < 0) lo += ext; else hi += ext;
  }
}

// Keep freed stream-ordered memory cached in the device's default pool
// (its default release threshold of 0 returns memory to the driver at every
// synchronisation, which makes per-call temporaries expensive).
std::mutex g_pool_mu;
bool g_pool_set[64] = {false};
void keep_pool_cached() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (g_pool_set[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  g_pool_set[dev] = true;
}

pdlgb300_error dalloc(size_t nbytes, void **p) {
  *p = nullptr;
  keep_pool_cached();
  if (nbytes == 0) nbytes = 16;
  cudaError_t e = cudaMallocAsync(p, nbytes, g_stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return err(PDLGB300_EFATAL, "device allocation of %zu bytes failed: %s", nbytes,
               cudaGetErrorString(e));
  }
  return ok();
}

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  bool on = false;
  void start() {
    if (!g_timing) return;
    on = true;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, g_stream);
  }
  double stop() {
    if (!on) return 0;
    cudaEventRecord(b, g_stream);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    on = false;
    return ms;
  }
};

// Make x addressable on the device.  input: copy host data in.
pdlgb300_error stage(pdlgb300_ndarray *x, bool is_out, Operand &op) {
  const size_t ts = TSIZES[x->datatype];
  if (x->ddata) {
    op.dev = (char *)x->ddata + x->offs * (int64_t)ts;
    return ok();
  }
  if (!x->data) {
    if (nvals(x) == 0) {
      op.dev = nullptr;
      return ok();
    }
    return err(PDLGB300_EUSERERROR, "ndarray has neither host nor device data");
  }
  int64_t lo, hi;
  span_of(x, lo, hi);
  if (hi < lo) {
    op.dev = nullptr;
    return ok();
  }
  size_t bytes = (size_t)(hi - lo + 1) * ts;
  RET_IF(dalloc(bytes, &op.owned));
  op.dev_lo = (char *)op.owned;
  op.host_lo = (char *)x->data + lo * (int64_t)ts;
  op.span_bytes = bytes;
  op.dev = op.dev_lo + (x->offs - lo) * (int64_t)ts;
  // outputs too: elements outside the view keep their host values
  Timer t;
  t.start();
  cudaError_t e = cudaMemcpyAsync(op.dev_lo, op.host_lo, bytes, cudaMemcpyHostToDevice, g_stream);
  tl_info.h2d_ms += t.stop();
  tl_info.h2d_bytes += (double)bytes;
  if (e != cudaSuccess) return err(PDLGB300_EFATAL, "H2D copy: %s", cudaGetErrorString(e));
  op.to_host = is_out;
  return ok();
}

pdlgb300_error unstage(Operand &op) {
  if (op.to_host && op.owned) {
    Timer t;
    t.start();
    cudaError_t e =
        cudaMemcpyAsync(op.host_lo, op.dev_lo, op.span_bytes, cudaMemcpyDeviceToHost, g_stream);
    tl_info.d2h_ms += t.stop();
    tl_info.d2h_bytes += (double)op.span_bytes;
    if (e != cudaSuccess) return err(PDLGB300_EFATAL, "D2H copy: %s", cudaGetErrorString(e));
  }
  return ok();
}

uint64_t bits_of(pdlgb300_value v) {
  uint64_t b;
  memcpy(&b, &v, 8);
  return b;
}

pdlgb300_value badval_of(const pdlgb300_ndarray *x) {
  if (x->has_badvalue && x->badvalue.type == x->datatype) return x->badvalue.value;
  return defbad(x->datatype);
}

uint64_t bad_bits(const pdlgb300_ndarray *x) {
  pdlgb300_value v = badval_of(x);
  uint64_t b = 0;
  memcpy(&b, &v, TSIZES[x->datatype]);
  return b;
}
int bad_isnan(const pdlgb300_ndarray *x) {
  pdlgb300_value v = badval_of(x);
  if (x->datatype == PDLGB300_F) return v.F != v.F;
  if (x->datatype == PDLGB300_D) return v.D != v.D;
  return 0;
}

// Type selection, pdl__transtype_select: the highest type among the
// outputs that were supplied, else among the inputs; typed outputs (int+,
// double, indx) do not vote.
// pdl__transtype_select (lib/PDL/Core/pdlapi.c:1208-1235): the largest
// type among the untyped parameters that GenericTypes allows, outputs
// voting first; a type above the last allowed one (or none at all) gives
// the last allowed type.
int transtype_select(const pdlgb300_vtable *vt, pdlgb300_ndarray *const *pdls) {
  bool avail[PDLGB300_NTYPES] = {false};
  int last = -1, ngen = 0;
  for (int k = 0; vt->gentypes[k] >= 0; k++, ngen++) {
    avail[vt->gentypes[k]] = true;
    last = vt->gentypes[k];
  }
  if (ngen == 1) return last;
  int ret = -1;
  bool use_last = false;
  for (int i = vt->npdls - 1; i >= 0; i--) {
    const pdlgb300_ndarray *p = pdls[i];
    if (!(p->state & PDLGB300_NOMYDIMS) && !(vt->par_flags[i] & PDLGB300_PARAM_ISTYPED)) {
      const int t = p->datatype;
      const bool ok = t >= 0 && t < PDLGB300_NTYPES && avail[t];
      if (!ok && t > last) use_last = true;
      if (ok && ret < t) ret = t;
    }
    if (i == vt->nparents && ret != -1) return ret;
  }
  if (use_last || ret < 0 || !avail[ret]) ret = last;
  return ret;
}

int out_type(const pdlgb300_vtable *vt, int i, int ttype) {
  int f = vt->par_flags[i];
  if (!(f & PDLGB300_PARAM_ISTYPED)) return ttype;
  if (f & PDLGB300_PARAM_ISTPLUS) return std::max((int)vt->par_types[i], ttype);
  return vt->par_types[i];
}

// Convert x (device view) into a fresh contiguous device buffer of type `to`.
pdlgb300_error convert_view(const pdlgb300_ndarray &x, const char *src, int to, int bad,
                            void **dst) {
  RET_IF(dalloc((size_t)std::max<int64_t>(nvals(&x), 1) * TSIZES[to], dst));
  ConvArgs g;
  memset(&g, 0, sizeof g);
  g.src = src;
  g.dst = (char *)*dst;
  // loop over x's dims: src increments, dst default increments
  Brc b;
  b.np = 2;
  b.ndims = std::max(x.ndims, 1);
  int64_t s = 1;
  for (int k = 0; k < b.ndims; k++) {
    b.dims[k] = k < x.ndims ? x.dims[k] : 1;
    b.incs[k][0] = k < x.ndims ? x.incs[k] : 0;
    b.incs[k][1] = s;
    s *= b.dims[k];
  }
  const int which[2] = {0, 1};
  g.L = collapse(b, 2, which);
  g.bad = bad;
  g.sbad = bad_bits(&x);
  g.sbad_isnan = bad_isnan(&x);
  pdlgb300_value tb = defbad(to);
  g.dbad = bits_of(tb);
  return launch_convert(x.datatype, to, g, g_stream);
}

// ================================================================ run

struct RunCtx {
  const pdlgb300_vtable *vt;
  int op;
  int ttype;
  int bvalflag;
  pdlgb300_ndarray v[MAXP];    // working (device) views
  pdlgb300_ndarray *user[MAXP];
  Operand opd[MAXP];
  void *conv[MAXP] = {nullptr};  // converted copies
  bool out_converted[MAXP] = {false};
  char *dev[MAXP] = {nullptr};   // device origin of each working view
  Brc b;
  int *d_setbad = nullptr;
};

void release(RunCtx &c) {
  for (int i = 0; i < MAXP; i++) {
    if (c.conv[i]) cudaFreeAsync(c.conv[i], g_stream);
    if (c.opd[i].owned) cudaFreeAsync(c.opd[i].owned, g_stream);
    c.conv[i] = c.opd[i].owned = nullptr;
  }
}

// One device word per device for PDLSTATESETBAD(output) reports, allocated
// on first use and kept for the life of the process.
std::mutex g_flag_mu;
int *g_flag_word[64] = {nullptr};
pdlgb300_error setbad_word(int **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return err(PDLGB300_EFATAL, "no current CUDA device");
  std::lock_guard<std::mutex> lk(g_flag_mu);
  if (!g_flag_word[dev]) {
    cudaError_t e = cudaMalloc((void **)&g_flag_word[dev], 256);
    if (e == cudaSuccess) e = cudaMemset(g_flag_word[dev], 0, 256);
    if (e != cudaSuccess) {
      g_flag_word[dev] = nullptr;
      return err(PDLGB300_EFATAL, "device allocation failed: %s", cudaGetErrorString(e));
    }
  }
  *out = g_flag_word[dev];
  return ok();
}

// Per-row arrival counters of split reductions, per device: zeroed once;
// every launch leaves them zero again (the last block of a row resets its
// counter).
constexpr int SPLIT_CTRS = 4096;
int *g_split_ctr[64];
pdlgb300_error split_counters(int **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return err(PDLGB300_EFATAL, "no current CUDA device");
  std::lock_guard<std::mutex> lk(g_flag_mu);
  if (!g_split_ctr[dev]) {
    cudaError_t e = cudaMalloc((void **)&g_split_ctr[dev], SPLIT_CTRS * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(g_split_ctr[dev], 0, SPLIT_CTRS * sizeof(int));
    if (e != cudaSuccess) {
      g_split_ctr[dev] = nullptr;
      return err(PDLGB300_EFATAL, "device allocation failed: %s", cudaGetErrorString(e));
    }
  }
  *out = g_split_ctr[dev];
  return ok();
}

// Word 1 of the same allocation: set by kernels whose bounded waits gave up.
pdlgb300_error status_word(int **out) {
  int *w = nullptr;
  RET_IF(setbad_word(&w));
  *out = w + 1;
  return ok();
}

pdlgb300_error dispatch(RunCtx &c, const int64_t *other);

pdlgb300_error run_impl(const pdlgb300_vtable *vt, pdlgb300_ndarray *const *pdls_in,
                        const int64_t *other) {
  const int op = op_of(vt);
  if (op < 0) return err(PDLGB300_EUSERERROR, "unknown vtable");
  keep_pool_cached();
  memset(&tl_info, 0, sizeof tl_info);
  snprintf(tl_info.op, sizeof tl_info.op, "%s", vt->name);
  RunCtx c;
  c.vt = vt;
  c.op = op;
  const int np = vt->npdls;
  for (int i = 0; i < np; i++) {
    if (!pdls_in[i]) return err(PDLGB300_EUSERERROR, "%s: parameter %d is NULL", vt->name, i);
    c.user[i] = pdls_in[i];
  }
  if (is_biop(op) && other && other[0]) std::swap(c.user[0], c.user[1]);
  for (int i = 0; i < np; i++) {
    const pdlgb300_ndarray *p = c.user[i];
    if (p->state & PDLGB300_NOMYDIMS) continue;
    if (p->datatype < 0 || p->datatype >= PDLGB300_NTYPES)
      return err(PDLGB300_EUSERERROR, "%s: parameter '%s': not a known data type code=%d",
                 vt->name, vt->par_names[i], p->datatype);
    if (p->datatype > PDLGB300_D)
      return err(PDLGB300_EUSERERROR,
                 "%s: parameter '%s' has type %s, which this GPU path does not compute",
                 vt->name, vt->par_names[i], TNAMES[p->datatype]);
  }
  c.ttype = transtype_select(vt, c.user);
  if (op == O_SMP) {
    for (int i = 0; i < 3; i++)
      if (c.user[i]->datatype != c.user[0]->datatype)
        return err(PDLGB300_EUSERERROR,
                   "sumover_mult_plus: a, b and d must have one type (got %s, %s, %s)",
                   TNAMES[c.user[0]->datatype], TNAMES[c.user[1]->datatype],
                   TNAMES[c.user[2]->datatype]);
    c.ttype = c.user[0]->datatype;
  }
  c.bvalflag = 0;
  for (int i = 0; i < vt->nparents; i++)
    if (c.user[i]->state & PDLGB300_BADVAL) c.bvalflag = 1;
  // shape null outputs (on the caller's descriptors)
  for (int i = vt->nparents; i < np; i++)
    if (c.user[i]->state & PDLGB300_NOMYDIMS) {
      c.user[i]->datatype = out_type(vt, i, c.ttype);
      c.user[i]->has_badvalue = 0;
      c.user[i]->badvalue.type = -1;
    }
  RET_IF(plan_broadcast(vt, c.user, c.b));
  for (int i = vt->nparents; i < np; i++) {
    pdlgb300_ndarray *p = c.user[i];
    if (p->state & PDLGB300_NOMYDIMS) {
      p->state &= ~PDLGB300_NOMYDIMS;
      if (!p->data && !p->ddata) {
        void *d = nullptr;
        RET_IF(dalloc((size_t)std::max<int64_t>(nvals(p), 1) * TSIZES[p->datatype], &d));
        p->ddata = d;
      }
    }
  }
  // stage and convert
  pdlgb300_error e = ok();
  for (int i = 0; i < np && !e.error; i++) {
    const bool is_out = i >= vt->nparents;
    e = stage(c.user[i], is_out, c.opd[i]);
    c.v[i] = *c.user[i];
    c.dev[i] = c.opd[i].dev;
    const int want = is_out ? out_type(vt, i, c.ttype) : c.ttype;
    if (!e.error && c.v[i].datatype != want) {
      if (is_out && op == O_SMP)
        e = err(PDLGB300_EUSERERROR, "sumover_mult_plus: output type must be %s", TNAMES[want]);
      if (!e.error)
        e = convert_view(c.v[i], c.dev[i], want,
                         c.bvalflag && (c.v[i].state & PDLGB300_BADVAL), &c.conv[i]);
      if (!e.error) {
        pdlgb300_ndarray &w = c.v[i];
        pdlgb300_value nb = defbad(want);
        w.datatype = want;
        default_incs(&w);
        w.offs = 0;
        w.badvalue.type = want;
        w.badvalue.value = nb;
        w.has_badvalue = 0;
        c.dev[i] = (char *)c.conv[i];
        c.out_converted[i] = is_out;
      }
    }
  }
  pdlgb300_ndarray *vp[MAXP];
  for (int i = 0; i < np; i++) vp[i] = &c.v[i];
  if (!e.error) e = plan_broadcast(vt, vp, c.b);  // increments of the working views
  // PDLSTATESETBAD reports: min/max only when a row can be empty or all
  // bad; plus/mult/inner only in bad-value mode.  Otherwise nothing to read
  // back, so a device-resident op returns without waiting for the GPU.
  const bool minmax = op == O_MINIMUM || op == O_MAXIMUM || op == O_MINIMUM_IND ||
                      op == O_MAXIMUM_IND;
  const bool need_flag = (minmax && (c.bvalflag || c.b.ind_sizes[0] == 0)) ||
                         op == O_MINMAXIMUM ||  // an all-NaN row sets bad without bad mode
                         ((is_biop(op) || op == O_INNER) && c.bvalflag);
  if (!e.error) e = setbad_word(&c.d_setbad);
  if (!e.error && need_flag) {
    cudaError_t ce = cudaMemsetAsync(c.d_setbad, 0, sizeof(int), g_stream);
    if (ce != cudaSuccess) e = err(PDLGB300_EFATAL, "clearing the bad flag: %s", cudaGetErrorString(ce));
  }
  if (!e.error) {
    Timer t;
    t.start();
    e = dispatch(c, other);
    tl_info.kernel_ms += t.stop();
  }
  int setbad[MAXP] = {0};
  if (!e.error) {
    // converted outputs flow back into the caller's ndarray
    for (int i = vt->nparents; i < np && !e.error; i++) {
      if (!c.out_converted[i]) continue;
      const pdlgb300_ndarray &w = c.v[i];
      const pdlgb300_ndarray &u = *c.user[i];
      ConvArgs g;
      memset(&g, 0, sizeof g);
      g.src = (const char *)c.conv[i];
      g.dst = c.opd[i].dev;
      Brc b;
      b.np = 2;
      b.ndims = std::max(u.ndims, 1);
      for (int k = 0; k < b.ndims; k++) {
        b.dims[k] = k < u.ndims ? u.dims[k] : 1;
        b.incs[k][0] = k < w.ndims ? w.incs[k] : 0;
        b.incs[k][1] = k < u.ndims ? u.incs[k] : 0;
      }
      const int which[2] = {0, 1};
      g.L = collapse(b, 2, which);
      g.bad = c.bvalflag;
      g.sbad = bad_bits(&w);
      g.sbad_isnan = bad_isnan(&w);
      g.dbad = bad_bits(&u);
      e = launch_convert(w.datatype, u.datatype, g, g_stream);
    }
    if (!e.error && need_flag) {
      cudaError_t ce = cudaMemcpyAsync(setbad, c.d_setbad, sizeof(int),
                                       cudaMemcpyDeviceToHost, g_stream);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(g_stream);
      if (ce != cudaSuccess) e = err(PDLGB300_EFATAL, "reading bad flags: %s", cudaGetErrorString(ce));
    }
    for (int i = 0; i < np && !e.error; i++) e = unstage(c.opd[i]);
  }
  bool any_host = false, any_tmp = false;
  for (int i = 0; i < np; i++) {
    any_host |= c.opd[i].to_host;
    any_tmp |= c.opd[i].owned || c.conv[i];
  }
  release(c);
  if (any_host || any_tmp) {
    cudaError_t ce = cudaStreamSynchronize(g_stream);
    if (!e.error && ce != cudaSuccess) e = err(PDLGB300_EFATAL, "%s: %s", vt->name, cudaGetErrorString(ce));
  }
  if (e.error) return e;
  for (int i = vt->nparents; i < np; i++)
    if (c.bvalflag || setbad[0]) c.user[i]->state |= PDLGB300_BADVAL;
  tl_info.datatype = c.ttype;
  tl_last = tl_info;
  return ok();
}

// ------------------------------------------------------------ dispatch

pdlgb300_error dispatch_reduce(RunCtx &c, int redop) {
  const Brc &b = c.b;
  RedArgs a;
  memset(&a, 0, sizeof a);
  const int which[2] = {0, 1};
  a.L = collapse(b, 2, which);
  a.rows = a.L.total;
  a.n = b.ind_sizes[0];
  a.inc_n = b.inc_sizes[0][0];
  if (a.n <= 1) a.inc_n = 1;
  a.a = c.dev[0];
  a.b = c.dev[1];
  a.bad = c.bvalflag;
  a.abad_bits = bad_bits(&c.v[0]);
  a.abad_isnan = bad_isnan(&c.v[0]);
  a.bbad_bits = bad_bits(&c.v[1]);
  a.bbad_isnan = bad_isnan(&c.v[1]);
  a.setbad = c.d_setbad;
  a.f32_comp = (int)g_opt_comp;
  a.nsplit = 1;
  const size_t isz = TSIZES[c.v[0].datatype];
  tl_info.rows = a.rows;
  tl_info.n = a.n;
  const size_t osz = TSIZES[c.v[1].datatype];
  tl_info.bytes = (double)a.rows * a.n * isz + (double)a.rows * osz;
  if (a.rows == 0) return ok();
  const int nsm = pgh::num_sms();
  RedLaunch lc{0, 0, 0};
  const bool contiguous = a.inc_n == 1;
  if (!contiguous && a.rows >= (int64_t)nsm * 256 && a.L.inc[0][0] == 1) {
    lc.kind = 1;  // thread per row, coalesced across rows
    lc.block = 128;
    lc.grid = (int)std::min<int64_t>((a.rows + 127) / 128, (int64_t)nsm * 64);
  } else if (a.n * (int64_t)isz <= 32768) {
    // rows up to 32 KiB: a warp per row (a block per row with 128 bytes per
    // thread measured slower on the float64 (4096, 2048) family: its
    // 256-thread row merges cost more than the occupancy gained).  Up to 8
    // rows per block, fewer when rows are few, so the blocks spread evenly:
    // with 2048 rows, 8-row blocks leave the busiest SMs 16 rows against an
    // average of 13.5; 1-row blocks, 14.
    a.group = 32;
    const int64_t rpb = std::max<int64_t>(1, std::min<int64_t>(8, a.rows / (8 * (int64_t)nsm)));
    lc.block = (int)(32 * rpb);
    lc.grid = (int)std::min<int64_t>((a.rows + rpb - 1) / rpb, (int64_t)1 << 30);
  } else {
    a.group = a.n >= 16384 ? 256 : 128;
    lc.block = a.group;
    int64_t units = a.rows;
    // few long rows: split each row over several blocks, as many splits as
    // fill whole waves of resident blocks
    if (a.rows < 2 * (int64_t)nsm && a.n >= 65536) {
      const int dt0 = c.v[0].datatype;
      int occ = (redop == R_SUM || redop == R_DSUM || redop == R_AVG || redop == R_DAVG)
                    ? red_occ_sum(redop, dt0, a.f32_comp, a.bad, lc.block)
                : (redop == R_PROD || redop == R_DPROD) ? red_occ_prod(redop, dt0, a.bad, lc.block)
                : red_is_logic(redop) ? red_occ_logic(redop, dt0, a.bad, lc.block)
                                      : red_occ_minmax(redop, dt0, a.bad, lc.block);
      const int64_t slots = (int64_t)nsm * occ;
      int64_t want = std::max<int64_t>(1, slots / a.rows);
      int64_t maxs = a.n / 8192;
      a.nsplit = (int)std::max<int64_t>(1, std::min(want, maxs));
      units = a.rows * a.nsplit;
    }
    lc.grid = (int)std::min<int64_t>(units, (int64_t)1 << 30);
  }
  void *scratch = nullptr;
  const int dtin = c.v[0].datatype;
  // floating products: the reference's sequential product with its early
  // exit, by the prefix/suffix kernel (rows up to 2^20 elements)
  if (lc.kind == 0 && a.n <= PROD_SEQ_MAXN &&
      (redop == R_DPROD || (redop == R_PROD && (dtin == PDLGB300_F || dtin == PDLGB300_D)))) {
    const int64_t S = std::min<int64_t>(a.n, redop == R_PROD && dtin == PDLGB300_F ? 4096 : 2048);
    tl_info.grid = (a.rows + 31) / 32;
    return launch_prod_seq(redop, dtin, a, S, g_stream);
  }
  // floating products of longer rows (row kernel): per row, the first good
  // exact zero
  const bool zfix = lc.kind == 0 && (redop == R_DPROD ||
                                     (redop == R_PROD && (dtin == PDLGB300_F || dtin == PDLGB300_D)));
  if (a.nsplit > 1 || zfix) {
    size_t accsz = red_is_logic(redop) ? red_acc_size_logic(redop, dtin)
                                       : red_acc_size(redop, dtin, a.f32_comp);
    size_t npart = a.nsplit > 1 ? (size_t)a.rows * a.nsplit : 0;
    size_t off = (npart * accsz + 15) & ~(size_t)15;
    size_t offz = off + ((npart * sizeof(int64_t) + 15) & ~(size_t)15);
    size_t need = offz + (zfix ? (size_t)a.rows * sizeof(int64_t) : 0) + 256;
    RET_IF(dalloc(need, &scratch));
    if (npart) {
      a.partials = scratch;
      a.pcounts = (int64_t *)((char *)scratch + off);
    }
    if (zfix) a.zidx = (int64_t *)((char *)scratch + offz);
  }
  // split rows: the last block of a row merges its partials (rows split
  // only when there are fewer than 2 per SM, and a group is then a block)
  if (a.nsplit > 1 && a.group == lc.block && a.rows <= SPLIT_CTRS) RET_IF(split_counters(&a.split_ctr));
  pdlgb300_error e;
  const int dt = c.v[0].datatype;
  if (redop == R_SUM || redop == R_DSUM || redop == R_AVG || redop == R_DAVG)
    e = launch_red_sum(redop, dt, a, lc, g_stream);
  else if (redop == R_PROD || redop == R_DPROD)
    e = launch_red_prod(redop, dt, a, lc, g_stream);
  else if (red_is_logic(redop))
    e = launch_red_logic(redop, dt, a, lc, g_stream);
  else
    e = launch_red_minmax(redop, dt, a, lc, g_stream);
  if (scratch) cudaFreeAsync(scratch, g_stream);
  if (g_opt_debug)
    fprintf(stderr, "[pdlgb300] %s: rows=%lld n=%lld inc_n=%lld group=%d nsplit=%d grid=%d block=%d kind=%d\n",
            c.vt->name, (long long)a.rows, (long long)a.n, (long long)a.inc_n, a.group, a.nsplit,
            lc.grid, lc.block, lc.kind);
  return e;
}

// Rows start on 16-byte boundaries in both ndarrays (base and every
// broadcast increment).
bool chain_aligned(const Loop &L, const void *a, const void *b, size_t asz, size_t bsz) {
  if ((uintptr_t)a % 16 || (uintptr_t)b % 16) return false;
  for (int d = 0; d < L.nd; d++) {
    if (L.size[d] <= 1) continue;
    if ((L.inc[0][d] * (int64_t)asz) % 16 || (L.inc[1][d] * (int64_t)bsz) % 16) return false;
  }
  return true;
}

// Look-back slots of the chained scan, per device: a power-of-two ring at
// least as large as one launch's chunk count, tagged by a 64-bit unit id
// that only grows, so slots never need clearing between launches.
struct ChainRing {
  ChainSlot *slots = nullptr;
  uint64_t cap = 0;
  uint64_t next = 1;  // unit id 0 never used: zeroed memory reads as empty
};
ChainRing g_chain[64];
std::mutex g_chain_mu;

pdlgb300_error chain_slots(uint64_t units, ScanArgs *g) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return err(PDLGB300_EFATAL, "no current CUDA device");
  std::lock_guard<std::mutex> lk(g_chain_mu);
  ChainRing &r = g_chain[dev];
  if (r.cap < units) {
    uint64_t cap = 1024;
    while (cap < units) cap <<= 1;
    if (r.slots) {
      cudaStreamSynchronize(g_stream);
      cudaFree(r.slots);
      r.slots = nullptr;
      r.cap = 0;
    }
    cudaError_t e = cudaMalloc((void **)&r.slots, cap * sizeof(ChainSlot));
    if (e == cudaSuccess) e = cudaMemset(r.slots, 0, cap * sizeof(ChainSlot));
    if (e != cudaSuccess) {
      r.slots = nullptr;
      return err(PDLGB300_EFATAL, "device allocation failed: %s", cudaGetErrorString(e));
    }
    r.cap = cap;
  }
  g->status = r.slots;
  g->status_mask = r.cap - 1;
  g->gid_base = r.next;
  r.next += units;
  return ok();
}

pdlgb300_error dispatch_cumusum(RunCtx &c, int dop) {
  const Brc &b = c.b;
  ScanArgs g;
  memset(&g, 0, sizeof g);
  const int which[2] = {0, 1};
  g.L = collapse(b, 2, which);
  g.rows = g.L.total;
  g.n = b.ind_sizes[0];
  g.inc_a = g.n <= 1 ? 1 : b.inc_sizes[0][0];
  g.inc_b = g.n <= 1 ? 1 : b.inc_sizes[1][0];
  g.a = c.dev[0];
  g.b = c.dev[1];
  g.bad = c.bvalflag;
  g.abad = bad_bits(&c.v[0]);
  g.abad_isnan = bad_isnan(&c.v[0]);
  g.bbad = bad_bits(&c.v[1]);
  g.f32_comp = (int)g_opt_comp;
  g.nchunk = 1;
  g.chunk = g.n;
  tl_info.rows = g.rows;
  tl_info.n = g.n;
  tl_info.bytes = (double)g.rows * g.n * (TSIZES[c.v[0].datatype] + TSIZES[c.v[1].datatype]);
  if (g.rows == 0 || g.n == 0) return ok();
  const int nsm = pgh::num_sms();
  if (g.inc_a != 1 || g.inc_b != 1) {
    g.mode = -1;
    return launch_cumusum(dop, c.v[0].datatype, g, g_stream);
  }
  RET_IF(status_word(&g.err));
  // Many rows of several chunks, equally wide types: a block per row walks
  // its chunks in order (three blocks per SM; taken when the rows fill the
  // resident blocks eight times or more, so that the last partial round of
  // rows costs little)
  const int64_t rch = scan_rowblk_chunk(dop, c.v[0].datatype);
  if (rch > 0 && g.n >= 2 * rch && g.rows >= 8LL * 3 * nsm &&
      chain_aligned(g.L, c.dev[0], c.dev[1], TSIZES[c.v[0].datatype], TSIZES[c.v[1].datatype])) {
    g.mode = 4;
    g.chunk = rch;
    g.nchunk = (int)((g.n + rch - 1) / rch);
    return launch_cumusum(dop, c.v[0].datatype, g, g_stream);
  }
  // 16-byte aligned rows of 4- and 8-byte types, not too short: the chained
  // single-pass scan (one block per chunk, look-back across a row's chunks)
  const int64_t cch = scan_chain_chunk(dop, c.v[0].datatype, g.f32_comp);
  if (cch > 0 && g.n >= cch / 4 && chain_aligned(g.L, c.dev[0], c.dev[1],
                                                  TSIZES[c.v[0].datatype],
                                                  TSIZES[c.v[1].datatype])) {
    g.mode = 3;
    g.chunk = cch;
    g.nchunk = (int)((g.n + cch - 1) / cch);
    if (g.nchunk > 1) RET_IF(chain_slots((uint64_t)g.rows * g.nchunk, &g));
    return launch_cumusum(dop, c.v[0].datatype, g, g_stream);
  }
  void *scratch = nullptr;
  // few rows: cut them into chunks so that ~24 warps per SM have work
  const int64_t target = 24LL * nsm;
  if (g.rows < target && g.n >= 32768) {
    int64_t nch = std::max<int64_t>(1, std::min<int64_t>((target + g.rows - 1) / g.rows,
                                                          g.n / 8192));
    g.chunk = (g.n + nch - 1) / nch;
    g.chunk = (g.chunk + 4095) / 4096 * 4096;  // chunk starts stay 16-byte aligned
    g.nchunk = (int)((g.n + g.chunk - 1) / g.chunk);
    if (g.nchunk > 1) {
      size_t accsz = scan_acc_size(dop, c.v[0].datatype, g.f32_comp);
      RET_IF(dalloc((size_t)g.rows * g.nchunk * accsz + 16, &scratch));
      g.partials = scratch;
    }
  }
  pdlgb300_error e = launch_cumusum(dop, c.v[0].datatype, g, g_stream);
  if (scratch) cudaFreeAsync(scratch, g_stream);
  return e;
}

pdlgb300_error dispatch_minmaximum(RunCtx &c) {
  MM4Args g;
  memset(&g, 0, sizeof g);
  const int which[5] = {0, 1, 2, 3, 4};
  g.L = collapse(c.b, 5, which);
  g.rows = g.L.total;
  g.n = c.b.ind_sizes[0];
  g.inc_n = g.n <= 1 ? 1 : c.b.inc_sizes[0][0];
  g.a = c.dev[0];
  for (int i = 0; i < 4; i++) {
    g.out[i] = c.dev[1 + i];
    g.obad[i] = bad_bits(&c.v[1 + i]);
  }
  g.bad = c.bvalflag;
  g.abad = bad_bits(&c.v[0]);
  g.abad_isnan = bad_isnan(&c.v[0]);
  g.setbad = c.d_setbad;
  tl_info.rows = g.rows;
  tl_info.n = g.n;
  tl_info.bytes = (double)g.rows * g.n * TSIZES[c.v[0].datatype];
  return launch_minmaximum(c.v[0].datatype, g, g_stream);
}

pdlgb300_error dispatch_sortred(RunCtx &c, int kind) {
  const Brc &b = c.b;
  SortArgs g;
  memset(&g, 0, sizeof g);
  const bool pct = kind == SR_PCT || kind == SR_ODDPCT;
  const int np = pct ? 3 : 2;
  const int which[3] = {0, 1, 2};
  g.L = collapse(b, np, which);
  g.out_pdl = np - 1;
  g.rows = g.L.total;
  g.n = b.ind_sizes[0];
  g.inc_a = g.n <= 1 ? 1 : b.inc_sizes[0][0];
  g.inc_b = (kind == SR_QSORT || kind == SR_QSORTI) && g.n > 1 ? b.inc_sizes[1][0] : 1;
  g.a = c.dev[0];
  g.p = pct ? c.dev[1] : nullptr;
  g.b = c.dev[np - 1];
  g.bad = c.bvalflag;
  g.abad = bad_bits(&c.v[0]);
  g.abad_isnan = bad_isnan(&c.v[0]);
  g.obad = bad_bits(&c.v[np - 1]);
  const int dt = c.v[0].datatype;
  tl_info.rows = g.rows;
  tl_info.n = g.n;
  tl_info.bytes = (double)g.rows * g.n * TSIZES[dt] +
                  (double)g.rows * (kind <= SR_QSORTI ? g.n : 1) * TSIZES[c.v[np - 1].datatype];
  if (kind != SR_QSORT && kind != SR_QSORTI && kind != SR_MODE && nvals(&c.v[0]) == 0)
    return err(PDLGB300_EUSERERROR, "Error in %s:cannot process empty ndarray", c.vt->name);
  if (g.rows == 0 || g.n == 0) return ok();
  void *scratch = nullptr;
  if (g.n > SORT_SHARED_MAXN) {  // (shorter rows sort in shared memory)
    RET_IF(dalloc(sortred_long_scratch(kind, g.rows, g.n, TSIZES[dt]), &scratch));
    g.scratch = scratch;
  }
  int *w = nullptr;
  pdlgb300_error e = status_word(&w);
  g.err = w;
  int hs = 0;
  if (!e.error) {
    cudaError_t ce = cudaMemsetAsync(w, 0, sizeof(int), g_stream);
    if (ce != cudaSuccess) e = err(PDLGB300_EFATAL, "clearing the status word: %s", cudaGetErrorString(ce));
  }
  if (!e.error) e = launch_sortred(kind, dt, g, g_stream);
  if (!e.error) {
    cudaError_t ce = cudaMemcpyAsync(&hs, w, sizeof(int), cudaMemcpyDeviceToHost, g_stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(g_stream);
    if (ce != cudaSuccess) e = err(PDLGB300_EFATAL, "%s: %s", c.vt->name, cudaGetErrorString(ce));
  }
  if (scratch) cudaFreeAsync(scratch, g_stream);
  if (!e.error && hs) e = err(PDLGB300_EFATAL, "%s: a sort scan left its range", c.vt->name);
  return e;
}

pdlgb300_error dispatch_qsortvec(RunCtx &c, bool ind) {
  const Brc &b = c.b;
  VecSortArgs g;
  memset(&g, 0, sizeof g);
  const int which[2] = {0, 1};
  g.L = collapse(b, 2, which);
  g.rows = g.L.total;
  g.n = b.ind_sizes[0];
  g.m = b.ind_sizes[1];
  g.inc_an = b.inc_sizes[0][0];
  g.inc_am = b.inc_sizes[0][1];
  g.inc_bn = ind ? 0 : b.inc_sizes[1][0];
  g.inc_bm = ind ? b.inc_sizes[1][0] : b.inc_sizes[1][1];
  g.a = c.dev[0];
  g.b = c.dev[1];
  g.bad = c.bvalflag;
  g.abad = bad_bits(&c.v[0]);
  g.abad_isnan = bad_isnan(&c.v[0]);
  g.obad = bad_bits(&c.v[1]);
  const int dt = c.v[0].datatype;
  tl_info.rows = g.rows;
  tl_info.n = g.n * g.m;
  tl_info.bytes = (double)g.rows * g.n * g.m * TSIZES[dt] +
                  (double)g.rows * (ind ? g.m * 8 : g.n * g.m * TSIZES[dt]);
  // qsort_returnempty (Ufunc.pd:1038): nothing to do for an empty a
  if (g.rows == 0 || g.n == 0 || g.m == 0) return ok();
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t limit = (size_t)std::max(0, optin - 1024);  // (the block's static shared words)
  void *scratch = nullptr;
  if (qsortvec_smem_bytes(g.n, g.m, (int)TSIZES[dt]) > limit) {
    const size_t vbytes = ((size_t)g.rows * g.n * g.m * TSIZES[dt] + 15) & ~(size_t)15;
    RET_IF(dalloc(vbytes + (size_t)g.rows * g.m * sizeof(int64_t), &scratch));
    g.scratch = scratch;
    g.iscratch = (int64_t *)((char *)scratch + vbytes);
  }
  int *w = nullptr;
  pdlgb300_error e = status_word(&w);
  g.err = w;
  int hs = 0;
  if (!e.error) {
    cudaError_t ce = cudaMemsetAsync(w, 0, sizeof(int), g_stream);
    if (ce != cudaSuccess) e = err(PDLGB300_EFATAL, "clearing the status word: %s", cudaGetErrorString(ce));
  }
  if (!e.error) e = launch_qsortvec(ind, dt, g, limit, g_stream);
  if (!e.error) {
    cudaError_t ce = cudaMemcpyAsync(&hs, w, sizeof(int), cudaMemcpyDeviceToHost, g_stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(g_stream);
    if (ce != cudaSuccess) e = err(PDLGB300_EFATAL, "%s: %s", c.vt->name, cudaGetErrorString(ce));
  }
  if (scratch) cudaFreeAsync(scratch, g_stream);
  if (!e.error && hs) e = err(PDLGB300_EFATAL, "%s: a sort scan left its range", c.vt->name);
  return e;
}

pdlgb300_error dispatch_biop(RunCtx &c, int which_op) {
  BiopArgs g;
  memset(&g, 0, sizeof g);
  const int which[3] = {0, 1, 2};
  g.L = collapse(c.b, 3, which);
  g.a = c.dev[0];
  g.b = c.dev[1];
  g.c = c.dev[2];
  g.bad = c.bvalflag;
  g.statebad_a = !!(c.v[0].state & PDLGB300_BADVAL);
  g.statebad_b = !!(c.v[1].state & PDLGB300_BADVAL);
  g.abad = bad_bits(&c.v[0]);
  g.bbad = bad_bits(&c.v[1]);
  g.cbad = bad_bits(&c.v[2]);
  g.abad_isnan = bad_isnan(&c.v[0]);
  g.bbad_isnan = bad_isnan(&c.v[1]);
  g.setbad = c.d_setbad;
  const size_t ts = TSIZES[c.ttype];
  tl_info.rows = g.L.total;
  tl_info.bytes = (double)g.L.total * ts * 3;
  return launch_biop(which_op, c.ttype, g, g_stream);
}

pdlgb300_error dispatch_inner(RunCtx &c) {
  InnerArgs g;
  memset(&g, 0, sizeof g);
  const int which[3] = {0, 1, 2};
  g.L = collapse(c.b, 3, which);
  g.rows = g.L.total;
  g.n = c.b.ind_sizes[0];
  g.inc_a = g.n <= 1 ? 1 : c.b.inc_sizes[0][0];
  g.inc_b = g.n <= 1 ? 1 : c.b.inc_sizes[1][0];
  // a size-1 n dim broadcasts against the other's n (increment 0)
  if (c.v[0].ndims < 1 || c.v[0].dims[0] <= 1) g.inc_a = 0;
  if (c.v[1].ndims < 1 || c.v[1].dims[0] <= 1) g.inc_b = 0;
  g.a = c.dev[0];
  g.b = c.dev[1];
  g.c = c.dev[2];
  g.bad = c.bvalflag;
  g.abad = bad_bits(&c.v[0]);
  g.bbad = bad_bits(&c.v[1]);
  g.cbad = bad_bits(&c.v[2]);
  g.abad_isnan = bad_isnan(&c.v[0]);
  g.bbad_isnan = bad_isnan(&c.v[1]);
  g.setbad = c.d_setbad;
  const size_t ts = TSIZES[c.ttype];
  tl_info.rows = g.rows;
  tl_info.n = g.n;
  tl_info.bytes = (double)g.rows * g.n * 2 * ts + (double)g.rows * ts;
  tl_info.flops = 2.0 * g.rows * g.n;
  const bool contig = g.inc_a == 1 && g.inc_b == 1;
  if (!contig && g.rows >= 256LL * pgh::num_sms()) g.group = 0;
  else g.group = g.n * (int64_t)TSIZES[c.v[0].datatype] <= 32768 ? 32 : (g.n >= 16384 ? 256 : 128);
  return launch_inner(c.ttype, g, g_stream);
}

pdlgb300_error dispatch_matmult(RunCtx &c) {
  MMArgs g;
  memset(&g, 0, sizeof g);
  const int which[3] = {0, 1, 2};
  g.L = collapse(c.b, 3, which);
  g.batch = g.L.total;
  g.K = c.b.ind_sizes[0];
  g.M = c.b.ind_sizes[1];
  g.N = c.b.ind_sizes[2];
  // increments: a(t,h) b(w,t) c(w,h); a size-1 dim contributes increment 0
  g.a_k = c.b.inc_sizes[0][0];
  g.a_m = c.b.inc_sizes[0][1];
  g.b_n = c.b.inc_sizes[1][0];
  g.b_k = c.b.inc_sizes[1][1];
  g.c_n = c.b.inc_sizes[2][0];
  g.c_m = c.b.inc_sizes[2][1];
  g.a = c.dev[0];
  g.b = c.dev[1];
  g.c = c.dev[2];
  g.bad = c.bvalflag;
  g.abad = bad_bits(&c.v[0]);
  g.bbad = bad_bits(&c.v[1]);
  g.cbad = bad_bits(&c.v[2]);
  g.abad_isnan = bad_isnan(&c.v[0]);
  g.bbad_isnan = bad_isnan(&c.v[1]);
  g.cbad_isnan = bad_isnan(&c.v[2]);
  const size_t ts = TSIZES[c.ttype];
  tl_info.rows = g.batch;
  tl_info.n = g.K;
  tl_info.flops = 2.0 * g.batch * g.M * g.N * g.K;
  tl_info.bytes = (double)ts * (g.batch * (g.M * g.K + g.K * g.N + g.M * g.N));
  if (g.batch == 0 || g.M == 0 || g.N == 0) return ok();
  if (g.K == 0) {
    // nothing to accumulate: c = 0 (the tile loop zeroes it)
  }
  if (c.ttype == PDLGB300_F && !g.bad) {
    int mode = (int)g_opt_mm_mode;
    if ((mode == PDLGB300_MATMULT_BF16X3 || mode == PDLGB300_MATMULT_BF16X6) &&
        matmult_tc_supported(g))
      return launch_matmult_tc(mode == PDLGB300_MATMULT_BF16X3 ? 2 : 3, g, g_stream);
    if (mode == PDLGB300_MATMULT_SIMT_FP32) return launch_matmult_simt(c.ttype, 1, g, g_stream);
  }
  return launch_matmult_simt(c.ttype, 0, g, g_stream);
}

pdlgb300_error dispatch_smp(RunCtx &c) {
  FusedArgs g;
  memset(&g, 0, sizeof g);
  const int which[4] = {0, 1, 2, 3};
  g.L = collapse(c.b, 4, which);
  g.rows = g.L.total;
  g.n = c.b.ind_sizes[0];
  auto ninc = [&](int p) -> int64_t {
    if (g.n <= 1) return 0;
    if (c.v[p].ndims < 1 || c.v[p].dims[0] <= 1) return 0;
    return c.b.inc_sizes[p][0];
  };
  g.inc_a = ninc(0);
  g.inc_b = ninc(1);
  g.inc_d = ninc(2);
  g.a = c.dev[0];
  g.b = c.dev[1];
  g.d = c.dev[2];
  g.c = c.dev[3];
  g.fa = !!(c.v[0].state & PDLGB300_BADVAL);
  g.fb = !!(c.v[1].state & PDLGB300_BADVAL);
  g.fd = !!(c.v[2].state & PDLGB300_BADVAL);
  g.abad = bad_bits(&c.v[0]);
  g.bbad = bad_bits(&c.v[1]);
  g.dbad = bad_bits(&c.v[2]);
  g.abad_isnan = bad_isnan(&c.v[0]);
  g.bbad_isnan = bad_isnan(&c.v[1]);
  g.dbad_isnan = bad_isnan(&c.v[2]);
  pdlgb300_value tb = defbad(c.ttype);
  g.tbad = g.ubad = bits_of(tb);
  g.tbad_isnan = g.ubad_isnan = 0;
  g.cbad = bad_bits(&c.v[3]);
  g.f32_comp = (int)g_opt_comp;
  g.d_is_a = c.dev[2] == c.dev[0] && g.inc_d == g.inc_a;
  for (int k = 0; k < g.L.nd && g.d_is_a; k++)
    if (g.L.inc[2][k] != g.L.inc[0][k]) g.d_is_a = 0;
  // outer-product pattern over two loop dims
  if (g.L.nd == 2) {
    for (int jd = 0; jd < 2; jd++) {
      int kd = 1 - jd;
      bool a_ok = g.L.inc[0][jd] == 0 && g.L.inc[0][kd] != 0;
      bool b_ok = g.L.inc[1][kd] == 0 && g.L.inc[1][jd] != 0;
      bool d_ok = g.L.inc[2][jd] == 0;
      if (a_ok && b_ok && d_ok) {
        g.outer = 1;
        g.jdim = jd;
        g.kdim = kd;
        break;
      }
    }
  }
  const size_t ts = TSIZES[c.ttype];
  tl_info.rows = g.rows;
  tl_info.n = g.n;
  tl_info.flops = 3.0 * g.rows * g.n;
  return launch_fused_smp(c.ttype, g, g_stream);
}

pdlgb300_error dispatch(RunCtx &c, const int64_t *) {
  switch (c.op) {
    case O_SUMOVER: return dispatch_reduce(c, R_SUM);
    case O_DSUMOVER: return dispatch_reduce(c, R_DSUM);
    case O_PRODOVER: return dispatch_reduce(c, R_PROD);
    case O_DPRODOVER: return dispatch_reduce(c, R_DPROD);
    case O_AVERAGE: return dispatch_reduce(c, R_AVG);
    case O_DAVERAGE: return dispatch_reduce(c, R_DAVG);
    case O_MINIMUM: return dispatch_reduce(c, R_MIN);
    case O_MAXIMUM: return dispatch_reduce(c, R_MAX);
    case O_MINIMUM_IND: return dispatch_reduce(c, R_MIN_IND);
    case O_MAXIMUM_IND: return dispatch_reduce(c, R_MAX_IND);
    case O_CUMUSUMOVER: return dispatch_cumusum(c, 0);
    case O_DCUMUSUMOVER: return dispatch_cumusum(c, 1);
    case O_PLUS: case O_MULT: case O_MINUS: case O_DIVIDE: case O_GT: case O_LT: case O_LE:
    case O_GE: case O_EQ: case O_NE: case O_SHIFTLEFT: case O_SHIFTRIGHT: case O_OR2:
    case O_AND2: case O_XOR:
      return dispatch_biop(c, biop_code_of(c.op));
    case O_ANDOVER: return dispatch_reduce(c, R_AND);
    case O_OROVER: return dispatch_reduce(c, R_OR);
    case O_XOROVER: return dispatch_reduce(c, R_XOR);
    case O_ZCOVER: return dispatch_reduce(c, R_ZC);
    case O_BANDOVER: return dispatch_reduce(c, R_BAND);
    case O_BOROVER: return dispatch_reduce(c, R_BOR);
    case O_BXOROVER: return dispatch_reduce(c, R_BXOR);
    case O_FIRSTNONZEROOVER: return dispatch_reduce(c, R_FIRSTNZ);
    case O_MINMAXIMUM: return dispatch_minmaximum(c);
    case O_QSORT: return dispatch_sortred(c, SR_QSORT);
    case O_QSORTI: return dispatch_sortred(c, SR_QSORTI);
    case O_MEDOVER: return dispatch_sortred(c, SR_MED);
    case O_ODDMEDOVER: return dispatch_sortred(c, SR_ODDMED);
    case O_PCTOVER: return dispatch_sortred(c, SR_PCT);
    case O_ODDPCTOVER: return dispatch_sortred(c, SR_ODDPCT);
    case O_MODEOVER: return dispatch_sortred(c, SR_MODE);
    case O_QSORTVEC: return dispatch_qsortvec(c, false);
    case O_QSORTVECI: return dispatch_qsortvec(c, true);
    case O_CUMUPRODOVER: return dispatch_cumusum(c, 2);
    case O_DCUMUPRODOVER: return dispatch_cumusum(c, 3);
    case O_INNER: return dispatch_inner(c);
    case O_MATMULT: return dispatch_matmult(c);
    case O_SMP: return dispatch_smp(c);
  }
  return err(PDLGB300_EFATAL, "no dispatch for op %d", c.op);
}

pdlgb300_error guard_run(int op, pdlgb300_ndarray *const *pdls, const int64_t *other) {
  try {
    return run_impl(&VT[op], pdls, other);
  } catch (...) {
    return err(PDLGB300_EFATAL, "%s: internal error", VT[op].name);
  }
}

// ------------------------------------------------------ fused expressions

int redop_of(int op) {
  switch (op) {
    case O_SUMOVER: return R_SUM;
    case O_DSUMOVER: return R_DSUM;
    case O_PRODOVER: return R_PROD;
    case O_DPRODOVER: return R_DPROD;
    case O_AVERAGE: return R_AVG;
    case O_DAVERAGE: return R_DAVG;
    case O_MINIMUM: return R_MIN;
    case O_MAXIMUM: return R_MAX;
    case O_MINIMUM_IND: return R_MIN_IND;
    case O_MAXIMUM_IND: return R_MAX_IND;
    case O_ANDOVER: return R_AND;
    case O_OROVER: return R_OR;
    case O_XOROVER: return R_XOR;
    case O_ZCOVER: return R_ZC;
    case O_BANDOVER: return R_BAND;
    case O_BOROVER: return R_BOR;
    case O_BXOROVER: return R_BXOR;
    case O_FIRSTNONZEROOVER: return R_FIRSTNZ;
    default: return -1;
  }
}

// The expression's value is what the ops would materialise one by one; its
// dims are the broadcast of the leaves' dims (size-1 dims stretch), its bad
// flag the OR of the leaves' flags.  The reduction then runs on it as on a
// materialised ndarray: same type selection, output shape and bad rules.
pdlgb300_error run_expr_impl(const pdlgb300_vtable *rvt, int nleaf,
                             pdlgb300_ndarray *const *leaves, int nnode,
                             const pdlgb300_expr_node *nodes, pdlgb300_ndarray *out) {
  const int rop = op_of(rvt);
  const int redop = rop < 0 ? -1 : redop_of(rop);
  if (redop < 0) return err(PDLGB300_EUSERERROR, "expression reduction: not a reduction over dim 0");
  if (nleaf < 1 || nleaf > EXPR_MAXL || nnode < 1 || nnode > EXPR_MAXN)
    return err(PDLGB300_EUSERERROR, "expression reduction: %d leaves and %d ops (at most %d and %d)",
               nleaf, nnode, EXPR_MAXL, EXPR_MAXN);
  if (!out) return err(PDLGB300_EUSERERROR, "%s: output is NULL", rvt->name);
  keep_pool_cached();
  memset(&tl_info, 0, sizeof tl_info);
  snprintf(tl_info.op, sizeof tl_info.op, "%s(expr)", rvt->name);
  const int T = leaves[0] ? leaves[0]->datatype : -1;
  int lflag[EXPR_MAXL] = {0}, nflag[EXPR_MAXN] = {0};
  int nd = 0;
  for (int l = 0; l < nleaf; l++) {
    const pdlgb300_ndarray *x = leaves[l];
    if (!x || (x->state & PDLGB300_NOMYDIMS))
      return err(PDLGB300_EUSERERROR, "expression reduction: leaf %d is null", l);
    if (x->datatype != T)
      return err(PDLGB300_EUSERERROR, "expression reduction: leaves of types %s and %s", TNAMES[T],
                 TNAMES[x->datatype]);
    if (x->ndims < 0 || x->ndims > PDLGB300_MAXDIMS)
      return err(PDLGB300_EUSERERROR, "expression reduction: leaf %d has %d dims", l, x->ndims);
    lflag[l] = !!(x->state & PDLGB300_BADVAL);
    nd = std::max(nd, x->ndims);
  }
  if (!expr_fusable(redop, T))
    return err(PDLGB300_EUSERERROR, "expression reduction: %s over %s is not fused", rvt->name,
               T >= 0 && T < PDLGB300_NTYPES ? TNAMES[T] : "?");
  const bool is_int = T < PDLGB300_F;
  ExprArgs g;
  memset(&g, 0, sizeof g);
  std::vector<bool> used(nleaf + nnode, false);
  for (int k = 0; k < nnode; k++) {
    const pdlgb300_expr_node &q = nodes[k];
    const int op = q.op ? op_of(q.op) : -1;
    if (op < 0 || !is_biop(op))
      return err(PDLGB300_EUSERERROR, "expression reduction: op %d is not a binary op of PDL::Ops", k);
    const int code = biop_code_of(op);
    if (!is_int && code >= B_SHL)
      return err(PDLGB300_EUSERERROR, "expression reduction: %s works in an integer type", q.op->name);
    int ab[2] = {q.a, q.b};
    for (int i = 0; i < 2; i++) {
      if (ab[i] < 0 || ab[i] >= nleaf + k)
        return err(PDLGB300_EUSERERROR, "expression reduction: op %d operand %d refers to %d", k, i, ab[i]);
      used[ab[i]] = true;
      nflag[k] |= ab[i] < nleaf ? lflag[ab[i]] : nflag[ab[i] - nleaf];
      ab[i] = ab[i] < nleaf ? ab[i] : EXPR_MAXL + (ab[i] - nleaf);
    }
    g.node[k] = ExprNode{code, ab[0], ab[1]};
  }
  for (int i = 0; i < nleaf + nnode - 1; i++)
    if (!used[i])
      return err(PDLGB300_EUSERERROR, "expression reduction: %s %d does not reach the result",
                 i < nleaf ? "leaf" : "op", i < nleaf ? i : i - nleaf);
  // the expression's dims
  int64_t E[PDLGB300_MAXDIMS];
  for (int k = 0; k < nd; k++) {
    E[k] = 1;
    for (int l = 0; l < nleaf; l++) {
      const int64_t d = k < leaves[l]->ndims ? leaves[l]->dims[k] : 1;
      if (d == 1) continue;
      if (E[k] == 1) E[k] = d;
      else if (E[k] != d)
        return err(PDLGB300_EUSERERROR,
                   "expression reduction: mismatched broadcast dimension %d: size %lld vs. %lld", k,
                   (long long)E[k], (long long)d);
    }
  }
  const int rootflag = nflag[nnode - 1];
  pdlgb300_ndarray root;
  memset(&root, 0, sizeof root);
  root.datatype = T;
  root.ndims = nd;
  for (int k = 0; k < nd; k++) root.dims[k] = E[k];
  default_incs(&root);
  root.state = rootflag ? PDLGB300_BADVAL : 0;
  root.badvalue.type = -1;
  pdlgb300_ndarray *rp[2] = {&root, out};
  const int tt = transtype_select(rvt, rp);
  const int otype = out_type(rvt, 1, tt);
  if (tt != T)
    return err(PDLGB300_EUSERERROR, "expression reduction: %s would convert %s to %s", rvt->name,
               TNAMES[T], TNAMES[tt]);
  const bool creating = out->state & PDLGB300_NOMYDIMS;
  if (creating) {
    out->datatype = otype;
    out->has_badvalue = 0;
    out->badvalue.type = -1;
  } else if (out->datatype != otype) {
    return err(PDLGB300_EUSERERROR, "expression reduction: output type %s, %s gives %s",
               TNAMES[out->datatype], rvt->name, TNAMES[otype]);
  }
  Brc rb;
  RET_IF(plan_broadcast(rvt, rp, rb));
  if (creating) {
    out->state &= ~PDLGB300_NOMYDIMS;
    if (!out->data && !out->ddata) {
      void *d = nullptr;
      RET_IF(dalloc((size_t)std::max<int64_t>(nvals(out), 1) * TSIZES[out->datatype], &d));
      out->ddata = d;
    }
  }
  // the kernel's loop: broadcast dims 1.. of the expression, leaves 0..3,
  // the output at EXPR_MAXL
  const int64_t n = nd > 0 ? E[0] : 1;
  Brc b;
  b.np = EXPR_MAXL + 1;
  b.ndims = std::max(nd - 1, 1);
  for (int k = 0; k < MAXB; k++) {
    b.dims[k] = 1;
    for (int p = 0; p < MAXP; p++) b.incs[k][p] = 0;
  }
  for (int k = 0; k + 1 < nd; k++) {
    b.dims[k] = E[k + 1];
    for (int l = 0; l < nleaf; l++)
      if (k + 1 < leaves[l]->ndims && leaves[l]->dims[k + 1] == E[k + 1])
        b.incs[k][l] = leaves[l]->incs[k + 1];
    b.incs[k][EXPR_MAXL] = k < out->ndims ? out->incs[k] : 0;
  }
  Operand opd[EXPR_MAXL + 1];
  pdlgb300_error e = ok();
  for (int l = 0; l < nleaf && !e.error; l++) e = stage(leaves[l], false, opd[l]);
  if (!e.error) e = stage(out, true, opd[EXPR_MAXL]);
  const int which[EXPR_MAXL + 1] = {0, 1, 2, 3, EXPR_MAXL};
  g.L = collapse(b, EXPR_MAXL + 1, which);
  g.nleaf = nleaf;
  g.nnode = nnode;
  for (int l = 0; l < nleaf; l++) {
    const pdlgb300_ndarray *x = leaves[l];
    g.leaf[l] = opd[l].dev;
    g.inc_n[l] = (n > 1 && x->ndims > 0 && x->dims[0] == n) ? x->incs[0] : 0;
    g.lbad[l] = bad_bits(x);
    g.lbad_isnan[l] = bad_isnan(x);
    g.lflag[l] = lflag[l];
  }
  for (int k = 0; k < nnode; k++) g.nflag[k] = nflag[k];
  g.tbad = bad_bits(&root);
  g.tbad_isnan = bad_isnan(&root);
  g.bad = rootflag;
  g.out = opd[EXPR_MAXL].dev;
  g.obad = bad_bits(out);
  g.n = n;
  g.rows = g.L.total;
  g.f32_comp = (int)g_opt_comp;
  g.nsplit = 1;
  // 16-byte loads: every leaf contiguous along dim 0 with each row start
  // 16-byte aligned (its base and all its broadcast increments), or constant
  // along dim 0
  {
    const int64_t vec = 16 / (int64_t)TSIZES[T];
    bool ok = n >= 2 * vec;
    for (int l = 0; l < nleaf && ok; l++) {
      if (g.inc_n[l] == 0) continue;
      if (g.inc_n[l] != 1 || ((uintptr_t)g.leaf[l] & 15)) ok = false;
      for (int k = 0; k < g.L.nd && ok; k++)
        if (g.L.size[k] > 1 && g.L.inc[l][k] % vec) ok = false;
    }
    g.vec = ok;
  }
  const int nsm = pgh::num_sms();
  int grid = 0, block = 256;
  if (n * (int64_t)TSIZES[T] <= 32768) {
    g.group = 32;
    grid = (int)std::min<int64_t>((g.rows + 7) / 8, (int64_t)1 << 30);
  } else {
    g.group = 256;
    int64_t units = g.rows;
    if (g.rows < 2 * (int64_t)nsm && n >= 65536) {
      const int64_t want = std::max<int64_t>(1, (int64_t)nsm * 4 / g.rows);
      g.nsplit = (int)std::max<int64_t>(1, std::min<int64_t>(want, n / 8192));
      units = g.rows * g.nsplit;
    }
    grid = (int)std::min<int64_t>(units, (int64_t)1 << 30);
  }
  tl_info.rows = g.rows;
  tl_info.n = n;
  tl_info.datatype = T;
  tl_info.bytes = (double)g.rows * n * TSIZES[T] * nleaf + (double)g.rows * TSIZES[out->datatype];
  const bool minmax = redop == R_MIN || redop == R_MAX || redop == R_MIN_IND || redop == R_MAX_IND;
  const bool need_flag = minmax && (rootflag || n == 0);
  int *d_setbad = nullptr;
  if (!e.error) e = setbad_word(&d_setbad);
  g.setbad = d_setbad;
  if (!e.error && need_flag) {
    cudaError_t ce = cudaMemsetAsync(d_setbad, 0, sizeof(int), g_stream);
    if (ce != cudaSuccess) e = err(PDLGB300_EFATAL, "clearing the bad flag: %s", cudaGetErrorString(ce));
  }
  void *scratch = nullptr;
  RedArgs ra;
  memset(&ra, 0, sizeof ra);
  if (!e.error && g.nsplit > 1) {
    const size_t accsz = expr_acc_size(redop, T, g.f32_comp);
    const size_t npart = (size_t)g.rows * g.nsplit;
    const size_t off = (npart * accsz + 15) & ~(size_t)15;
    e = dalloc(off + npart * sizeof(int64_t) + 256, &scratch);
    if (!e.error) {
      g.partials = scratch;
      g.pcounts = (int64_t *)((char *)scratch + off);
      const int w2[2] = {0, EXPR_MAXL};
      ra.L = collapse(b, 2, w2);
      ra.b = g.out;
      ra.rows = g.rows;
      ra.n = n;
      ra.inc_n = 1;
      ra.nsplit = g.nsplit;
      ra.partials = g.partials;
      ra.pcounts = g.pcounts;
      ra.bad = g.bad;
      ra.bbad_bits = g.obad;
      ra.setbad = d_setbad;
    }
  }
  if (!e.error && g.rows > 0) {
    Timer t;
    t.start();
    e = launch_expr_reduce(redop, T, g, ra, grid, block, g_stream);
    tl_info.kernel_ms += t.stop();
  }
  if (scratch) cudaFreeAsync(scratch, g_stream);
  int setbad = 0;
  if (!e.error) {
    if (need_flag) {
      cudaError_t ce = cudaMemcpyAsync(&setbad, d_setbad, sizeof(int), cudaMemcpyDeviceToHost, g_stream);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(g_stream);
      if (ce != cudaSuccess) e = err(PDLGB300_EFATAL, "reading bad flags: %s", cudaGetErrorString(ce));
    }
    if (!e.error) e = unstage(opd[EXPR_MAXL]);
  }
  bool sync = false;
  for (int i = 0; i <= EXPR_MAXL; i++) {
    sync |= opd[i].to_host || opd[i].owned;
    if (opd[i].owned) cudaFreeAsync(opd[i].owned, g_stream);
  }
  if (sync) {
    cudaError_t ce = cudaStreamSynchronize(g_stream);
    if (!e.error && ce != cudaSuccess) e = err(PDLGB300_EFATAL, "%s: %s", rvt->name, cudaGetErrorString(ce));
  }
  if (e.error) return e;
  if (rootflag || setbad) out->state |= PDLGB300_BADVAL;
  tl_last = tl_info;
  return ok();
}

}  // namespace

// ================================================================ C ABI
extern "C" {

int32_t pdlgb300_abi_version(void) { return PDLGB300_ABI_VERSION; }

size_t pdlgb300_type_size(int32_t t) {
  return (t >= 0 && t < PDLGB300_NTYPES) ? TSIZES[t] : 0;
}
const char *pdlgb300_type_name(int32_t t) {
  return (t >= 0 && t < PDLGB300_NTYPES) ? TNAMES[t] : "unknown";
}

pdlgb300_error pdlgb300_ndarray_init(pdlgb300_ndarray *x, int32_t datatype, int32_t ndims,
                                     const int64_t *dims, void *data, void *ddata) {
  if (!x) return err(PDLGB300_EUSERERROR, "NULL descriptor");
  if (ndims < 0 || ndims > PDLGB300_MAXDIMS)
    return err(PDLGB300_EUSERERROR, "ndims %d out of range", ndims);
  if (datatype < 0 || datatype >= PDLGB300_NTYPES)
    return err(PDLGB300_EUSERERROR, "not a known data type code=%d", datatype);
  memset(x, 0, sizeof *x);
  x->datatype = datatype;
  x->ndims = ndims;
  x->badvalue.type = -1;
  for (int i = 0; i < ndims; i++) {
    if (dims[i] < 0) return err(PDLGB300_EUSERERROR, "negative dim %lld", (long long)dims[i]);
    x->dims[i] = dims[i];
  }
  default_incs(x);
  x->data = data;
  x->ddata = ddata;
  return ok();
}

pdlgb300_error pdlgb300_ndarray_null(pdlgb300_ndarray *x) {
  if (!x) return err(PDLGB300_EUSERERROR, "NULL descriptor");
  memset(x, 0, sizeof *x);
  x->state = PDLGB300_NOMYDIMS;
  x->datatype = PDLGB300_D;
  x->badvalue.type = -1;
  return ok();
}

pdlgb300_error pdlgb300_get_default_badvalue(int32_t t, pdlgb300_anyval *out) {
  if (t < 0 || t > PDLGB300_D || !out) return err(PDLGB300_EUSERERROR, "bad type %d", t);
  out->type = t;
  out->reserved = 0;
  out->value = defbad(t);
  return ok();
}

pdlgb300_error pdlgb300_set_default_badvalue(int32_t t, pdlgb300_anyval v) {
  if (t < 0 || t > PDLGB300_D) return err(PDLGB300_EUSERERROR, "bad type %d", t);
  defbad(t);
  g_defbad[t] = v.value;
  return ok();
}

const pdlgb300_vtable *pdlgb300_get_vtable(const char *name) {
  if (!name) return nullptr;
  for (int i = 0; i < O_NOPS; i++)
    if (!strcmp(VT[i].name, name)) return &VT[i];
  return nullptr;
}

pdlgb300_error pdlgb300_redodims(const pdlgb300_vtable *vt, pdlgb300_ndarray *const *pdls,
                                 const int64_t *other) {
  int op = op_of(vt);
  if (op < 0) return err(PDLGB300_EUSERERROR, "unknown vtable");
  pdlgb300_ndarray *p[MAXP];
  for (int i = 0; i < vt->npdls; i++) {
    if (!pdls[i]) return err(PDLGB300_EUSERERROR, "%s: parameter %d is NULL", vt->name, i);
    p[i] = pdls[i];
  }
  if (is_biop(op) && other && other[0]) std::swap(p[0], p[1]);
  int tt = transtype_select(vt, p);
  Brc b;
  RET_IF(plan_broadcast(vt, p, b));
  for (int i = vt->nparents; i < vt->npdls; i++)
    if (p[i]->state & PDLGB300_NOMYDIMS) {
      p[i]->datatype = out_type(vt, i, tt);
      p[i]->state &= ~PDLGB300_NOMYDIMS;
    }
  return ok();
}

pdlgb300_error pdlgb300_run(const pdlgb300_vtable *vt, pdlgb300_ndarray *const *pdls,
                            const int64_t *other) {
  int op = op_of(vt);
  if (op < 0) return err(PDLGB300_EUSERERROR, "unknown vtable");
  return guard_run(op, pdls, other);
}

#define RUN2(NAME, OP)                                                             \
  pdlgb300_error pdlgb300_run_##NAME(pdlgb300_ndarray *a, pdlgb300_ndarray *b) {   \
    pdlgb300_ndarray *p[2] = {a, b};                                               \
    return guard_run(OP, p, nullptr);                                              \
  }
RUN2(sumover, O_SUMOVER)
RUN2(dsumover, O_DSUMOVER)
RUN2(prodover, O_PRODOVER)
RUN2(dprodover, O_DPRODOVER)
RUN2(cumusumover, O_CUMUSUMOVER)
RUN2(dcumusumover, O_DCUMUSUMOVER)
RUN2(average, O_AVERAGE)
RUN2(daverage, O_DAVERAGE)
RUN2(minimum, O_MINIMUM)
RUN2(maximum, O_MAXIMUM)
RUN2(minimum_ind, O_MINIMUM_IND)
RUN2(maximum_ind, O_MAXIMUM_IND)
RUN2(andover, O_ANDOVER)
RUN2(orover, O_OROVER)
RUN2(xorover, O_XOROVER)
RUN2(zcover, O_ZCOVER)
RUN2(bandover, O_BANDOVER)
RUN2(borover, O_BOROVER)
RUN2(bxorover, O_BXOROVER)
RUN2(firstnonzeroover, O_FIRSTNONZEROOVER)
RUN2(cumuprodover, O_CUMUPRODOVER)
RUN2(dcumuprodover, O_DCUMUPRODOVER)
RUN2(qsort, O_QSORT)
RUN2(qsorti, O_QSORTI)
RUN2(medover, O_MEDOVER)
RUN2(oddmedover, O_ODDMEDOVER)
RUN2(modeover, O_MODEOVER)
RUN2(qsortvec, O_QSORTVEC)
RUN2(qsortveci, O_QSORTVECI)

pdlgb300_error pdlgb300_run_pctover(pdlgb300_ndarray *a, pdlgb300_ndarray *p, pdlgb300_ndarray *b) {
  pdlgb300_ndarray *q[3] = {a, p, b};
  return guard_run(O_PCTOVER, q, nullptr);
}
pdlgb300_error pdlgb300_run_oddpctover(pdlgb300_ndarray *a, pdlgb300_ndarray *p,
                                       pdlgb300_ndarray *b) {
  pdlgb300_ndarray *q[3] = {a, p, b};
  return guard_run(O_ODDPCTOVER, q, nullptr);
}

pdlgb300_error pdlgb300_run_minmaximum(pdlgb300_ndarray *a, pdlgb300_ndarray *cmin,
                                       pdlgb300_ndarray *cmax, pdlgb300_ndarray *cmin_ind,
                                       pdlgb300_ndarray *cmax_ind) {
  pdlgb300_ndarray *p[5] = {a, cmin, cmax, cmin_ind, cmax_ind};
  return guard_run(O_MINMAXIMUM, p, nullptr);
}

pdlgb300_error pdlgb300_run_expr_reduce(const pdlgb300_vtable *reduction, int32_t nleaf,
                                        pdlgb300_ndarray *const *leaves, int32_t nnode,
                                        const pdlgb300_expr_node *nodes, pdlgb300_ndarray *out) {
  try {
    return run_expr_impl(reduction, nleaf, leaves, nnode, nodes, out);
  } catch (...) {
    return err(PDLGB300_EFATAL, "expression reduction: internal error");
  }
}

pdlgb300_error pdlgb300_run_plus(pdlgb300_ndarray *a, pdlgb300_ndarray *b, pdlgb300_ndarray *c,
                                 int swap) {
  pdlgb300_ndarray *p[3] = {a, b, c};
  int64_t o = swap;
  return guard_run(O_PLUS, p, &o);
}
pdlgb300_error pdlgb300_run_mult(pdlgb300_ndarray *a, pdlgb300_ndarray *b, pdlgb300_ndarray *c,
                                 int swap) {
  pdlgb300_ndarray *p[3] = {a, b, c};
  int64_t o = swap;
  return guard_run(O_MULT, p, &o);
}
#define RUNBI(NAME, OP)                                                                   \
  pdlgb300_error pdlgb300_run_##NAME(pdlgb300_ndarray *a, pdlgb300_ndarray *b,             \
                                     pdlgb300_ndarray *c, int swap) {                      \
    pdlgb300_ndarray *p[3] = {a, b, c};                                                    \
    int64_t o = swap;                                                                      \
    return guard_run(OP, p, &o);                                                           \
  }
RUNBI(minus, O_MINUS)
RUNBI(divide, O_DIVIDE)
RUNBI(gt, O_GT)
RUNBI(lt, O_LT)
RUNBI(le, O_LE)
RUNBI(ge, O_GE)
RUNBI(eq, O_EQ)
RUNBI(ne, O_NE)
RUNBI(shiftleft, O_SHIFTLEFT)
RUNBI(shiftright, O_SHIFTRIGHT)
RUNBI(or2, O_OR2)
RUNBI(and2, O_AND2)
RUNBI(xor, O_XOR)
#undef RUNBI

pdlgb300_error pdlgb300_run_inner(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                  pdlgb300_ndarray *c) {
  pdlgb300_ndarray *p[3] = {a, b, c};
  return guard_run(O_INNER, p, nullptr);
}
pdlgb300_error pdlgb300_run_matmult(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                    pdlgb300_ndarray *c) {
  pdlgb300_ndarray *p[3] = {a, b, c};
  return guard_run(O_MATMULT, p, nullptr);
}
pdlgb300_error pdlgb300_run_sumover_mult_plus(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                              pdlgb300_ndarray *d, pdlgb300_ndarray *c) {
  pdlgb300_ndarray *p[4] = {a, b, d, c};
  return guard_run(O_SMP, p, nullptr);
}

pdlgb300_error pdlgb300_convert(const pdlgb300_ndarray *src, pdlgb300_ndarray *dst) {
  if (!src || !dst) return err(PDLGB300_EUSERERROR, "convert: NULL descriptor");
  if (src->datatype > PDLGB300_D || dst->datatype > PDLGB300_D || src->datatype < 0 ||
      dst->datatype < 0)
    return err(PDLGB300_EUSERERROR, "convert: unsupported type");
  if (src->ndims != dst->ndims)
    return err(PDLGB300_EUSERERROR, "convert: dims differ");
  for (int i = 0; i < src->ndims; i++)
    if (src->dims[i] != dst->dims[i]) return err(PDLGB300_EUSERERROR, "convert: dims differ");
  memset(&tl_info, 0, sizeof tl_info);
  snprintf(tl_info.op, sizeof tl_info.op, "convert");
  pdlgb300_ndarray s = *src, d = *dst;
  Operand os, od;
  RET_IF(stage(&s, false, os));
  pdlgb300_error e = stage(&d, true, od);
  if (!e.error) {
    ConvArgs g;
    memset(&g, 0, sizeof g);
    g.src = os.dev;
    g.dst = od.dev;
    Brc b;
    b.np = 2;
    b.ndims = std::max(s.ndims, 1);
    for (int k = 0; k < b.ndims; k++) {
      b.dims[k] = k < s.ndims ? s.dims[k] : 1;
      b.incs[k][0] = k < s.ndims ? s.incs[k] : 0;
      b.incs[k][1] = k < d.ndims ? d.incs[k] : 0;
    }
    const int which[2] = {0, 1};
    g.L = collapse(b, 2, which);
    g.bad = !!(s.state & PDLGB300_BADVAL);
    g.sbad = bad_bits(&s);
    g.sbad_isnan = bad_isnan(&s);
    g.dbad = bad_bits(&d);
    e = launch_convert(s.datatype, d.datatype, g, g_stream);
  }
  if (!e.error) e = unstage(od);
  if (os.owned) cudaFreeAsync(os.owned, g_stream);
  if (od.owned) cudaFreeAsync(od.owned, g_stream);
  if (os.owned || od.owned) cudaStreamSynchronize(g_stream);
  if (!e.error && (s.state & PDLGB300_BADVAL)) dst->state |= PDLGB300_BADVAL;
  tl_last = tl_info;
  return e;
}

pdlgb300_error pdlgb300_set_option(int32_t option, int64_t value) {
  switch (option) {
    case PDLGB300_OPT_MATMULT_MODE:
      if (value < 0 || value > 3) return err(PDLGB300_EUSERERROR, "matmult mode %lld", (long long)value);
      g_opt_mm_mode = value;
      return ok();
    case PDLGB300_OPT_F32_COMPENSATED: g_opt_comp = value ? 1 : 0; return ok();
    case PDLGB300_OPT_DEBUG: g_opt_debug = value; return ok();
  }
  return err(PDLGB300_EUSERERROR, "unknown option %d", option);
}
int64_t pdlgb300_get_option(int32_t option) {
  switch (option) {
    case PDLGB300_OPT_MATMULT_MODE: return g_opt_mm_mode;
    case PDLGB300_OPT_F32_COMPENSATED: return g_opt_comp;
    case PDLGB300_OPT_DEBUG: return g_opt_debug;
  }
  return -1;
}

pdlgb300_error pdlgb300_set_stream(void *s) {
  g_stream = (cudaStream_t)s;
  return ok();
}

pdlgb300_error pdlgb300_device_alloc(size_t nbytes, void **dptr) {
  if (!dptr) return err(PDLGB300_EUSERERROR, "NULL out pointer");
  RET_IF(dalloc(nbytes, dptr));
  cudaError_t e = cudaStreamSynchronize(g_stream);
  if (e != cudaSuccess) return err(PDLGB300_EFATAL, "alloc: %s", cudaGetErrorString(e));
  return ok();
}
pdlgb300_error pdlgb300_free(void *dptr) {
  if (!dptr) return ok();
  cudaError_t e = cudaFreeAsync(dptr, g_stream);
  if (e != cudaSuccess) return err(PDLGB300_EFATAL, "free: %s", cudaGetErrorString(e));
  return ok();
}
pdlgb300_error pdlgb300_to_device(void *dptr, const void *host, size_t nbytes) {
  memset(&tl_info, 0, sizeof tl_info);
  snprintf(tl_info.op, sizeof tl_info.op, "to_device");
  Timer t;
  t.start();
  cudaError_t e = cudaMemcpyAsync(dptr, host, nbytes, cudaMemcpyHostToDevice, g_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g_stream);
  tl_info.h2d_ms = t.stop();
  tl_info.h2d_bytes = (double)nbytes;
  tl_last = tl_info;
  if (e != cudaSuccess) return err(PDLGB300_EFATAL, "to_device: %s", cudaGetErrorString(e));
  return ok();
}
pdlgb300_error pdlgb300_to_host(void *host, const void *dptr, size_t nbytes) {
  memset(&tl_info, 0, sizeof tl_info);
  snprintf(tl_info.op, sizeof tl_info.op, "to_host");
  Timer t;
  t.start();
  cudaError_t e = cudaMemcpyAsync(host, dptr, nbytes, cudaMemcpyDeviceToHost, g_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g_stream);
  tl_info.d2h_ms = t.stop();
  tl_info.d2h_bytes = (double)nbytes;
  tl_last = tl_info;
  if (e != cudaSuccess) return err(PDLGB300_EFATAL, "to_host: %s", cudaGetErrorString(e));
  return ok();
}
pdlgb300_error pdlgb300_to_device_async(void *dptr, const void *host, size_t nbytes,
                                        void *stream) {
  cudaStream_t s = stream ? (cudaStream_t)stream : g_stream;
  cudaError_t e = cudaMemcpyAsync(dptr, host, nbytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return err(PDLGB300_EFATAL, "to_device_async: %s", cudaGetErrorString(e));
  return ok();
}
pdlgb300_error pdlgb300_to_host_async(void *host, const void *dptr, size_t nbytes,
                                      void *stream) {
  cudaStream_t s = stream ? (cudaStream_t)stream : g_stream;
  cudaError_t e = cudaMemcpyAsync(host, dptr, nbytes, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return err(PDLGB300_EFATAL, "to_host_async: %s", cudaGetErrorString(e));
  return ok();
}
pdlgb300_error pdlgb300_sync(void) {
  cudaError_t e = cudaStreamSynchronize(g_stream);
  if (e != cudaSuccess) return err(PDLGB300_EFATAL, "sync: %s", cudaGetErrorString(e));
  int *w = nullptr;
  if (!setbad_word(&w).error) {
    int st = 0;
    if (cudaMemcpy(&st, w + 1, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && st) {
      cudaMemset(w + 1, 0, sizeof(int));
      return err(PDLGB300_EFATAL, "a kernel gave up waiting on its pipeline (timeout)");
    }
  }
  return ok();
}
const char *pdlgb300_op_package(const char *name) { return name ? op_package(name) : ""; }

pdlgb300_error pdlgb300_device_count(int32_t *n) {
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *n = 0;
    return ok();
  }
  *n = c;
  return ok();
}
pdlgb300_error pdlgb300_last_launch(pdlgb300_launch_info *out) {
  if (!out) return err(PDLGB300_EUSERERROR, "NULL out pointer");
  *out = tl_last;
  return ok();
}
pdlgb300_error pdlgb300_set_timing(int32_t on) {
  g_timing = on ? 1 : 0;
  return ok();
}

}  // extern "C"

// ============================================================== adjoints
namespace {

bool is_float_type(int t) { return t == PDLGB300_F || t == PDLGB300_D; }

// out = scale * unbroadcast(x [* y]) where x has the broadcast (full) shape,
// y broadcasts to it, and out has an input's shape (size-1 or missing dims
// are summed over).
pdlgb300_error unbroadcast_into(const pdlgb300_ndarray *xu, const pdlgb300_ndarray *yu,
                                pdlgb300_ndarray *ou, double scale, int64_t lead_skip) {
  if (!xu || !ou) return err(PDLGB300_EUSERERROR, "backward: NULL ndarray");
  const int dt = xu->datatype;
  if (!is_float_type(dt) || ou->datatype != dt || (yu && yu->datatype != dt))
    return err(PDLGB300_EUSERERROR, "backward: gradients must all be float or all double");
  pdlgb300_ndarray x = *xu, o = *ou, y;
  if (yu) y = *yu;
  Operand ox, oy, oo;
  RET_IF(stage(&x, false, ox));
  pdlgb300_error e = ok();
  if (yu) e = stage(&y, false, oy);
  if (!e.error) e = stage(&o, true, oo);
  UnbArgs g;
  memset(&g, 0, sizeof g);
  if (!e.error) {
    // lead_skip: leading dims of out that x lacks (sumover/average: n)
    Brc bo, br;
    bo.np = br.np = 3;
    int no = 0, nr = 0;
    const int nd = std::max(x.ndims, o.ndims - (int)lead_skip);
    for (int k = 0; k < (int)lead_skip && !e.error; k++) {
      bo.dims[no] = o.dims[k];
      bo.incs[no][0] = 0;
      bo.incs[no][1] = 0;
      bo.incs[no][2] = o.incs[k];
      no++;
    }
    for (int k = 0; k < nd && !e.error; k++) {
      const int ko = k + (int)lead_skip;
      int64_t xs = k < x.ndims ? x.dims[k] : 1;
      int64_t os = ko < o.ndims ? o.dims[ko] : 1;
      int64_t xi = k < x.ndims ? x.incs[k] : 0;
      int64_t yi = 0;
      if (yu && k < y.ndims) {
        if (y.dims[k] == xs) yi = y.incs[k];
        else if (y.dims[k] != 1) e = err(PDLGB300_EUSERERROR, "backward: operand dims do not broadcast");
      }
      if (os == xs) {
        bo.dims[no] = xs;
        bo.incs[no][0] = xi;
        bo.incs[no][1] = yi;
        bo.incs[no][2] = ko < o.ndims ? o.incs[ko] : 0;
        no++;
      } else if (os == 1) {
        if (lead_skip) { e = err(PDLGB300_EUSERERROR, "backward: gradient dims do not match"); break; }
        br.dims[nr] = xs;
        br.incs[nr][0] = xi;
        br.incs[nr][1] = yi;
        br.incs[nr][2] = 0;
        nr++;
      } else {
        e = err(PDLGB300_EUSERERROR, "backward: gradient dim %d has size %lld, expected %lld or 1",
                ko, (long long)os, (long long)xs);
      }
    }
    if (!e.error) {
      bo.ndims = std::max(no, 1);
      if (no == 0) bo.dims[0] = 1;
      br.ndims = std::max(nr, 1);
      if (nr == 0) br.dims[0] = 1;
      const int which[3] = {0, 1, 2};
      g.Lo = collapse(bo, 3, which);
      g.Lr = collapse(br, 2, which);
      g.x = ox.dev;
      g.y = yu ? oy.dev : nullptr;
      g.out = oo.dev;
      g.scale = scale;
      e = launch_unbroadcast(dt, g, g_stream);
    }
  }
  if (!e.error) e = unstage(oo);
  for (Operand *op : {&ox, &oy, &oo})
    if (op->owned) cudaFreeAsync(op->owned, g_stream);
  if (ox.owned || oy.owned || oo.owned) cudaStreamSynchronize(g_stream);
  return e;
}

pdlgb300_ndarray xchg01(const pdlgb300_ndarray &a) {
  pdlgb300_ndarray t = a;
  if (t.ndims < 2) {
    for (int k = t.ndims; k < 2; k++) { t.dims[k] = 1; t.incs[k] = 0; }
    t.ndims = 2;
  }
  std::swap(t.dims[0], t.dims[1]);
  std::swap(t.incs[0], t.incs[1]);
  return t;
}

// Gradient of one matmult operand: full = matmult(p, q) (broadcast batch),
// then summed into `target` over the batch dims the operand was broadcast on.
pdlgb300_error mm_grad(pdlgb300_ndarray p, pdlgb300_ndarray q, pdlgb300_ndarray *target) {
  pdlgb300_ndarray full;
  pdlgb300_ndarray_null(&full);
  pdlgb300_ndarray *pp[3] = {&p, &q, &full};
  RET_IF(pdlgb300_redodims(&VT[O_MATMULT], pp, nullptr));
  bool same = full.ndims == target->ndims;
  for (int k = 0; k < full.ndims && same; k++) same = full.dims[k] == target->dims[k];
  if (same) {
    pdlgb300_ndarray out = *target;
    pdlgb300_ndarray *qq[3] = {&p, &q, &out};
    return run_impl(&VT[O_MATMULT], qq, nullptr);
  }
  // Every batch dim summed away, and in both operands each batch dim's
  // increment continues the contraction's (inc(b1) = inc(k) * K, ...): the
  // batch is part of the contraction, c(w, h) = sum over (k, b) of
  // p(k, h, b) q(w, k, b), one matmult of contraction K * B into the target.
  {
    bool fold = p.ndims >= 2 && q.ndims >= 2 && p.ndims == q.ndims && full.ndims > 2;
    for (int k = 2; k < full.ndims && fold; k++)
      fold = (k >= target->ndims || target->dims[k] == 1) && p.dims[k] == full.dims[k] &&
             q.dims[k] == full.dims[k];
    for (int k = 2; k < target->ndims && fold; k++) fold = k < full.ndims && target->dims[k] == 1;
    int64_t K = p.dims[0], ip = p.incs[0], iq = q.incs[1];
    for (int k = 2; k < full.ndims && fold; k++) {
      if (full.dims[k] == 1) continue;
      fold = p.incs[k] == ip * K && q.incs[k] == iq * K && ip != 0 && iq != 0;
      K *= full.dims[k];
    }
    if (fold && K != p.dims[0]) {
      pdlgb300_ndarray pf = p, qf = q, out = *target;
      pf.ndims = 2;
      pf.dims[0] = K;
      qf.ndims = 2;
      qf.dims[1] = K;
      out.ndims = 2;
      for (int k = target->ndims; k < 2; k++) { out.dims[k] = 1; out.incs[k] = 0; }
      pdlgb300_ndarray *qq[3] = {&pf, &qf, &out};
      return run_impl(&VT[O_MATMULT], qq, nullptr);
    }
  }
  pdlgb300_ndarray tmp;
  pdlgb300_ndarray_null(&tmp);
  pdlgb300_ndarray *qq[3] = {&p, &q, &tmp};
  RET_IF(run_impl(&VT[O_MATMULT], qq, nullptr));
  pdlgb300_error e = unbroadcast_into(&tmp, nullptr, target, 1.0, 0);
  cudaFreeAsync(tmp.ddata, g_stream);
  cudaStreamSynchronize(g_stream);
  return e;
}

}  // namespace

extern "C" {

pdlgb300_error pdlgb300_sumover_bwd(const pdlgb300_ndarray *gb, pdlgb300_ndarray *ga) {
  if (!gb || !ga) return err(PDLGB300_EUSERERROR, "sumover_bwd: NULL ndarray");
  return unbroadcast_into(gb, nullptr, ga, 1.0, 1);
}

pdlgb300_error pdlgb300_average_bwd(const pdlgb300_ndarray *gb, pdlgb300_ndarray *ga) {
  if (!gb || !ga) return err(PDLGB300_EUSERERROR, "average_bwd: NULL ndarray");
  int64_t n = ga->ndims > 0 ? ga->dims[0] : 1;
  return unbroadcast_into(gb, nullptr, ga, n ? 1.0 / (double)n : 0.0, 1);
}

pdlgb300_error pdlgb300_plus_bwd(const pdlgb300_ndarray *gc, pdlgb300_ndarray *ga,
                                 pdlgb300_ndarray *gb) {
  if (ga) RET_IF(unbroadcast_into(gc, nullptr, ga, 1.0, 0));
  if (gb) RET_IF(unbroadcast_into(gc, nullptr, gb, 1.0, 0));
  return ok();
}

pdlgb300_error pdlgb300_mult_bwd(const pdlgb300_ndarray *gc, const pdlgb300_ndarray *a,
                                 const pdlgb300_ndarray *b, pdlgb300_ndarray *ga,
                                 pdlgb300_ndarray *gb) {
  if (ga) RET_IF(unbroadcast_into(gc, b, ga, 1.0, 0));
  if (gb) RET_IF(unbroadcast_into(gc, a, gb, 1.0, 0));
  return ok();
}

// c(w,h) = sum_t a(t,h) b(w,t):  ga(t,h) = sum_w gc(w,h) b(w,t) = matmult(gc, b^T)
//                                gb(w,t) = sum_h gc(w,h) a(t,h) = matmult(a^T, gc)
pdlgb300_error pdlgb300_matmult_bwd(const pdlgb300_ndarray *gc, const pdlgb300_ndarray *a,
                                    const pdlgb300_ndarray *b, pdlgb300_ndarray *ga,
                                    pdlgb300_ndarray *gb) {
  if (!gc || !a || !b) return err(PDLGB300_EUSERERROR, "matmult_bwd: NULL ndarray");
  if (!is_float_type(gc->datatype))
    return err(PDLGB300_EUSERERROR, "matmult_bwd: float or double only");
  if (ga) RET_IF(mm_grad(*gc, xchg01(*b), ga));
  if (gb) RET_IF(mm_grad(xchg01(*a), *gc, gb));
  return ok();
}

}  // extern "C"

// ======================================================= no-allocation sumover
// pdlgb300_sumover_noalloc: the multi-block split sumover (per-split partial
// sums, then an in-order combine) with its partials in a fixed device array
// instead of memory from the allocator.  For callers that cannot allocate
// device memory: a process that hands the library a fixed device-memory
// budget up front, or code that must not trigger the device-wide
// synchronisation an allocation or free can cause.
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)1 << 20;  // 1 MiB, per device
__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[64] = {nullptr};

// Host code cannot use g_noalloc_scratch's name as a device address: look the
// address up once per device, with that device current.
pdlgb300_error noalloc_scratch(void **out) {
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess || dev < 0 || dev >= 64)
    return err(PDLGB300_EFATAL, "sumover_noalloc: no current CUDA device");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (ce != cudaSuccess || !p)
      return err(PDLGB300_EFATAL, "sumover_noalloc: cudaGetSymbolAddress failed: %s",
                 cudaGetErrorString(ce));
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return ok();
}

}  // namespace

extern "C" pdlgb300_error pdlgb300_sumover_noalloc(const pdlgb300_ndarray *a_in,
                                                   pdlgb300_ndarray *b_in) {
  if (!a_in || !b_in) return err(PDLGB300_EUSERERROR, "sumover_noalloc: NULL ndarray");
  const pdlgb300_vtable *vt = &VT[O_SUMOVER];
  if (!a_in->ddata || !b_in->ddata)
    return err(PDLGB300_EUSERERROR,
               "sumover_noalloc: a and b must both be device-resident (ddata set)");
  if (b_in->state & PDLGB300_NOMYDIMS)
    return err(PDLGB300_EUSERERROR, "sumover_noalloc: b must be shaped and allocated by the caller");
  if (a_in->datatype < 0 || a_in->datatype > PDLGB300_D)
    return err(PDLGB300_EUSERERROR, "sumover_noalloc: unsupported type %d", a_in->datatype);
  if (b_in->datatype != intplus(a_in->datatype))
    return err(PDLGB300_EUSERERROR, "sumover_noalloc: b must have type %s",
               TNAMES[intplus(a_in->datatype)]);
  pdlgb300_ndarray a = *a_in, b = *b_in;
  pdlgb300_ndarray *pp[2] = {&a, &b};
  Brc br;
  RET_IF(plan_broadcast(vt, pp, br));
  void *scratch = nullptr;
  RET_IF(noalloc_scratch(&scratch));
  RedArgs g;
  memset(&g, 0, sizeof g);
  const int which[2] = {0, 1};
  g.L = collapse(br, 2, which);
  g.rows = g.L.total;
  g.n = br.ind_sizes[0];
  g.inc_n = g.n <= 1 ? 1 : br.inc_sizes[0][0];
  const size_t isz = TSIZES[a.datatype], osz = TSIZES[b.datatype];
  g.a = (const char *)a.ddata + a.offs * (int64_t)isz;
  g.b = (char *)b.ddata + b.offs * (int64_t)osz;
  g.bad = !!(a.state & PDLGB300_BADVAL);
  g.abad_bits = bad_bits(&a);
  g.abad_isnan = bad_isnan(&a);
  g.bbad_bits = bad_bits(&b);
  g.bbad_isnan = bad_isnan(&b);
  g.setbad = nullptr;  // sumover never reports PDLSTATESETBAD
  g.f32_comp = (int)g_opt_comp;
  if (g.rows == 0) return ok();
  // always the split form: at least two partials per row, as many as the
  // planner would use for long rows, within the fixed scratch
  const size_t unit = red_acc_size(R_SUM, a.datatype, g.f32_comp) + sizeof(int64_t);
  const int nsm = pgh::num_sms();
  int64_t want = 2;
  if (g.rows < 2 * (int64_t)nsm && g.n >= 65536)
    want = std::max<int64_t>(2, std::min<int64_t>((4 * (int64_t)nsm + g.rows - 1) / g.rows,
                                                  g.n / 8192));
  const int64_t fit = (int64_t)((NOALLOC_SCRATCH_BYTES - 256) / (unit * (size_t)g.rows));
  if (fit < 2)
    return err(PDLGB300_EUSERERROR,
               "sumover_noalloc: %lld rows need %zu bytes of scratch, above the %zu-byte limit "
               "(at most %lld rows for this type)",
               (long long)g.rows, (size_t)(2 * unit * g.rows), NOALLOC_SCRATCH_BYTES,
               (long long)((NOALLOC_SCRATCH_BYTES - 256) / (2 * unit)));
  g.nsplit = (int)std::min<int64_t>(want, fit);
  const size_t accsz = unit - sizeof(int64_t);
  g.partials = scratch;
  size_t off = ((size_t)g.rows * g.nsplit * accsz + 15) & ~(size_t)15;
  g.pcounts = (int64_t *)((char *)scratch + off);
  g.group = g.n >= 16384 ? 256 : 128;
  RedLaunch lc{0, (int)std::min<int64_t>(g.rows * g.nsplit, (int64_t)1 << 30), g.group};
  memset(&tl_info, 0, sizeof tl_info);
  snprintf(tl_info.op, sizeof tl_info.op, "sumover_noalloc");
  tl_info.rows = g.rows;
  tl_info.n = g.n;
  tl_info.bytes = (double)g.rows * g.n * isz + (double)g.rows * osz;
  pdlgb300_error e = launch_red_sum(R_SUM, a.datatype, g, lc, g_stream);
  if (e.error) return e;
  if (g.bad) b_in->state |= PDLGB300_BADVAL;
  tl_last = tl_info;
  return ok();
}
