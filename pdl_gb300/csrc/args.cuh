// args.cuh -- kernel argument blocks and launcher entry points (host view).
#pragma once
#include "common.cuh"

namespace pg {

template <class T> __host__ __device__ __forceinline__ T from_bits(uint64_t b) {
  T t;
  memcpy(&t, &b, sizeof(T));
  return t;
}

// ------------------------------------------------------------ reductions
enum RedOp {
  R_SUM = 0, R_DSUM, R_PROD, R_DPROD, R_AVG, R_DAVG, R_MIN, R_MAX,
  R_MIN_IND, R_MAX_IND,
  // lib/PDL/Ufunc.pd:143-187
  R_AND, R_OR, R_XOR, R_ZC, R_BAND, R_BOR, R_BXOR, R_FIRSTNZ, R_NOPS
};
inline bool red_is_logic(int op) { return op >= R_AND && op <= R_FIRSTNZ; }

struct RedArgs {
  const char *a;      // element (0) of a (already offset)
  char *b;            // element (0) of b
  int64_t n;          // reduced length
  int64_t inc_n;      // a's increment along n (elements)
  int64_t rows;       // broadcast iterations
  Loop L;             // pdl 0 = a, pdl 1 = b
  int bad;            // trans bvalflag
  uint64_t abad_bits, bbad_bits;  // badvalues (raw bits, in a's / b's type)
  int abad_isnan, bbad_isnan;
  int *setbad;        // device flag: PDLSTATESETBAD(output)
  void *partials;     // split mode: per (row, split) accumulators
  int64_t *pcounts;   // split mode: per (row, split) good counts
  int nsplit;         // splits per row (1 = none)
  int group;          // threads per row (row kernel)
  int f32_comp;       // compensated float32 sums
  int64_t *zidx;      // floating products: per row, first good exact zero (or INT64_MAX)
  int *split_ctr;     // split mode: per-row arrival counters (zero between launches), or
                      // nullptr for a separate combine kernel
};

// A deferred expression reduced over dim 0 (expr.cu).  Operand indices:
// 0..EXPR_MAXL-1 the leaves, EXPR_MAXL + k node k; node nnode-1 is the root.
constexpr int EXPR_MAXL = 4, EXPR_MAXN = 8;
struct ExprNode {
  int op;    // BiopCode
  int a, b;  // operands
};
struct ExprArgs {
  Loop L;                          // pdls 0..EXPR_MAXL-1 leaves, EXPR_MAXL the output
  const char *leaf[EXPR_MAXL];     // element (0) of each leaf
  int64_t inc_n[EXPR_MAXL];        // each leaf's increment along dim 0 (0: broadcast)
  uint64_t lbad[EXPR_MAXL];        // leaves' badvalues (raw bits)
  int lbad_isnan[EXPR_MAXL], lflag[EXPR_MAXL];  // NaN badvalue; the leaf's bad flag
  int nleaf, nnode;
  ExprNode node[EXPR_MAXN];
  int nflag[EXPR_MAXN];            // each node's bad flag (OR of its operands')
  uint64_t tbad;                   // nodes' badvalue: the default of the type
  int tbad_isnan;
  int bad;                         // the reduction's bvalflag (the root's flag)
  char *out;                       // element (0) of the output
  uint64_t obad;
  int64_t n, rows;
  int group, nsplit, f32_comp;
  int vec;                         // leaves contiguous (16-byte aligned rows) or constant along dim 0
  void *partials;
  int64_t *pcounts;
  int *setbad;
};
bool expr_fusable(int redop, int dt);
size_t expr_acc_size(int redop, int dt, int comp);

struct RedLaunch {
  int kind;  // 0 rows, 1 thread
  int grid, block;
};

pdlgb300_error launch_expr_reduce(int redop, int dt, const ExprArgs &g, const RedArgs &ra,
                                  int grid, int block, cudaStream_t s);
pdlgb300_error launch_red_sum(int op, int in_dt, RedArgs args, const RedLaunch &lc,
                              cudaStream_t s);
// Floating prodover/dprodover with the reference's early exit (prod_seq.cu):
// the first S elements of each row sequentially, then the rest.
constexpr int64_t PROD_SEQ_MAXN = (int64_t)1 << 20;
pdlgb300_error launch_prod_seq(int op, int in_dt, const RedArgs &a, int64_t S, cudaStream_t s);
pdlgb300_error launch_red_prod(int op, int in_dt, RedArgs args, const RedLaunch &lc,
                               cudaStream_t s);
pdlgb300_error launch_red_minmax(int op, int in_dt, RedArgs args, const RedLaunch &lc,
                                 cudaStream_t s);
pdlgb300_error launch_red_logic(int op, int in_dt, RedArgs args, const RedLaunch &lc,
                                cudaStream_t s);
int red_occ_logic(int op, int in_dt, bool bad, int block);
size_t red_acc_size_logic(int op, int in_dt);
size_t red_acc_size(int op, int in_dt, int f32_comp);
int red_occ_sum(int op, int in_dt, int comp, bool bad, int block);
int red_occ_prod(int op, int in_dt, bool bad, int block);
int red_occ_minmax(int op, int in_dt, bool bad, int block);

// ------------------------------------------------------------ plus/mult
struct BiopArgs {
  const char *a, *b;
  char *c;
  Loop L;  // pdl 0 a, 1 b, 2 c
  int bad, statebad_a, statebad_b;
  uint64_t abad, bbad, cbad;
  int abad_isnan, bbad_isnan;
  int *setbad;
};
pdlgb300_error launch_biop(int op, int dt, const BiopArgs &g, cudaStream_t s);

// minmaximum: a(n) -> cmin, cmax, cmin_ind, cmax_ind (pdls 1..4 of L)
struct MM4Args {
  const char *a;
  char *out[4];
  int64_t n, inc_n, rows;
  Loop L;  // pdl 0 a, 1 cmin, 2 cmax, 3 cmin_ind, 4 cmax_ind
  int bad;
  uint64_t abad;
  int abad_isnan;
  uint64_t obad[4];
  int *setbad;
};
pdlgb300_error launch_minmaximum(int dt, const MM4Args &g, cudaStream_t s);

// The sort-based functions of PDL::Ufunc (sortred.cu).
enum SortKind { SR_QSORT, SR_QSORTI, SR_MED, SR_ODDMED, SR_PCT, SR_ODDPCT, SR_MODE };
struct SortArgs {
  const char *a;      // element (0) of a
  const char *p;      // element (0) of p (pctover, oddpctover)
  char *b;            // element (0) of the output
  int out_pdl;        // the output's index in L
  int64_t n, inc_a, inc_b, rows;
  Loop L;             // pdl 0 a, [1 p], then the output
  int bad;
  uint64_t abad, obad;
  int abad_isnan;
  void *scratch;      // long rows: the merge sort's buffers
  int *err;           // bit 0: a scan left its range (never expected)
};
pdlgb300_error launch_sortred(int kind, int dt, const SortArgs &g, cudaStream_t s);
// scratch bytes of the merge sort of rows longer than SORT_SHARED_MAXN
size_t sortred_long_scratch(int kind, int64_t rows, int64_t n, int tsize);
// rows up to this length sort in shared memory (warp or block kernels); the
// scratch copies serve longer rows only
constexpr int64_t SORT_SHARED_MAXN = 8192;

// qsortvec / qsortveci: a(n,m) -> b(n,m) or indx(m)
struct VecSortArgs {
  const char *a;      // element (0,0) of a
  char *b;            // element (0) of the output
  int64_t n, m, rows;
  int64_t inc_an, inc_am, inc_bn, inc_bm;
  Loop L;             // pdl 0 a, 1 the output
  int bad;
  uint64_t abad, obad;
  int abad_isnan;
  void *scratch;      // rows x n x m values (the one-thread-per-row kernel)
  int64_t *iscratch;  // rows x m positions (the same)
  int *err;           // bit 0: a scan left its range (never expected)
};
size_t qsortvec_smem_bytes(int64_t n, int64_t m, int tsize);
pdlgb300_error launch_qsortvec(bool ind, int dt, const VecSortArgs &g, size_t smem_limit,
                               cudaStream_t s);

struct ConvArgs {
  const char *src;
  char *dst;
  Loop L;  // pdl 0 src, 1 dst
  int bad;
  uint64_t sbad, dbad;
  int sbad_isnan;
};
pdlgb300_error launch_convert(int from, int to, const ConvArgs &g, cudaStream_t s);

// ----------------------------------------------------------- cumusumover
struct ScanArgs {
  const char *a;
  char *b;
  int64_t n, inc_a, inc_b, rows;
  Loop L;  // pdl 0 a, 1 b
  int bad;
  uint64_t abad, bbad;
  int abad_isnan;
  int f32_comp;
  int nchunk;        // chunks per row (> 1: three-pass long-row scan)
  int64_t chunk;     // elements per chunk
  void *partials;    // per (row, chunk) totals, then exclusive carries
  int mode;          // 0 full row, 1 chunk totals only, 2 chunk scan with carry, 3 chained,
                     // 4 a block per row
  int *err;          // device status word: set when a bounded wait gives up
  void *status;      // chained scan: look-back slots (ChainSlot), a power of two
  uint64_t status_mask;
  uint64_t gid_base;  // unit id of this launch's first chunk
};
// One look-back slot of the chained scan: flag = (unit id << 2) | state
// (1 aggregate, 2 inclusive prefix); values are the accumulator's bits.
struct alignas(32) ChainSlot {
  unsigned long long flag, agg, incl, pad;
};
// elements per chunk of the chained scan for an input type (0: not used)
int64_t scan_chain_chunk(int dop, int in_dt, int f32_comp);
// elements per chunk of the row-block scan of many rows (0: not used)
int64_t scan_rowblk_chunk(int dop, int in_dt);
pdlgb300_error launch_cumusum(int dop, int in_dt, ScanArgs g, cudaStream_t s);
size_t scan_acc_size(int dop, int in_dt, int f32_comp);

}  // namespace pg

namespace pg {
// ----------------------------------------------------------------- inner
struct InnerArgs {
  const char *a, *b;
  char *c;
  int64_t n, inc_a, inc_b, rows;
  Loop L;  // pdl 0 a, 1 b, 2 c
  int bad;
  uint64_t abad, bbad, cbad;
  int abad_isnan, bbad_isnan;
  int *setbad;
  int group;
};
pdlgb300_error launch_inner(int dt, const InnerArgs &g, cudaStream_t s);

// --------------------------------------------------------------- matmult
struct MMArgs {
  const char *a, *b;
  char *c;
  int64_t K, M, N;                 // t, h, w
  int64_t a_k, a_m, b_n, b_k, c_n, c_m;  // element increments
  int64_t batch;
  Loop L;  // batch dims: pdl 0 a, 1 b, 2 c
  int bad;
  uint64_t abad, bbad, cbad;
  int abad_isnan, bbad_isnan, cbad_isnan;
};
// mode: PDLGB300_MATMULT_* (float32 only; other types use the exact kernel)
pdlgb300_error launch_matmult_simt(int dt, int fused, const MMArgs &g, cudaStream_t s);
pdlgb300_error launch_matmult_tc(int limbs, const MMArgs &g, cudaStream_t s);
bool matmult_tc_supported(const MMArgs &g);

// ------------------------------------------- fused sumover(mult+plus)
struct FusedArgs {
  const char *a, *b, *d;
  char *c;
  int64_t n, inc_a, inc_b, inc_d, rows;
  Loop L;  // pdl 0 a, 1 b, 2 d, 3 c
  int fa, fb, fd;                  // input badflag states
  uint64_t abad, bbad, dbad, tbad, ubad, cbad;
  int abad_isnan, bbad_isnan, dbad_isnan, tbad_isnan, ubad_isnan;
  int f32_comp;
  int outer;                       // 1: a/d vary with dim ky only, b with dim jx only
  int d_is_a;                      // d aliases a (same data and increments)
  int jdim, kdim;                  // loop dims of the outer pattern
};
pdlgb300_error launch_fused_smp(int dt, const FusedArgs &g, cudaStream_t s);

// ------------------------------------------------------------ adjoints
struct UnbArgs {  // out(o) = sum over r of f(in(o, r))
  const char *x, *y;               // y optional (mult_bwd multiplies by y)
  char *out;
  Loop Lo;                         // output index space: pdl 0 x, 1 y, 2 out
  Loop Lr;                         // reduced index space: pdl 0 x, 1 y
  double scale;
  int nsplit;                      // r splits (column kernel), set by the launcher
  void *partials;                  // per (split, output) partial sums when nsplit > 1
};
pdlgb300_error launch_unbroadcast(int dt, const UnbArgs &g, cudaStream_t s);
}  // namespace pg
