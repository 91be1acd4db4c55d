/*
 * pdlgb300.h -- C ABI of libpdlgb300, the GB300 (sm_103a) implementation of
 * PDL's broadcast-loop hot path: the PDL::Ufunc reductions over dim 0, the
 * PDL::Ops binary ops plus/mult under broadcasting, and the PDL::Primitive
 * contractions inner/matmult.
 *
 * Plain C: no torch, Perl or CUDA types appear in any signature.  Every entry
 * point returns a pdlgb300_error by value, the same convention as PDL's
 * pdl_error (lib/PDL/Core/pdl.h.PL:370-379): error == 0 means success, a
 * non-zero error carries a message that a Perl XS caller turns into barf()
 * exactly as PDL->barf_if_error does (lib/PDL/Core/pdlutil.c:507).
 *
 * Array descriptors (pdlgb300_ndarray) carry what a PDL readdata body reads
 * from a pdl: datatype, dims, per-dim element increments and offset (the
 * vaffine view PDL_REPRINCS/PDL_REPROFFS of lib/PDL/Core/pdl.h.PL:511-517),
 * the data pointer, the PDL_BADVAL state bit and the per-ndarray badvalue.
 */
#ifndef PDLGB300_H
#define PDLGB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PDLGB300_ABI_VERSION 1
#define PDLGB300_MAXDIMS 16

/* Element types, in PDL's own enum order (lib/PDL/Types.pm:29-230):
 * sbyte byte short ushort long ulong indx ulonglong longlong float double
 * ldouble cfloat cdouble cldouble.  The GPU path computes every real type
 * except ldouble; complex and ldouble return PDLGB300_EUSERERROR. */
typedef enum pdlgb300_datatype {
  PDLGB300_SB = 0, PDLGB300_B, PDLGB300_S, PDLGB300_US, PDLGB300_L,
  PDLGB300_UL, PDLGB300_IND, PDLGB300_ULL, PDLGB300_LL, PDLGB300_F,
  PDLGB300_D, PDLGB300_LD, PDLGB300_CF, PDLGB300_CD, PDLGB300_CLD,
  PDLGB300_NTYPES
} pdlgb300_datatype;

/* Error kinds, mirroring PDL_ENONE / PDL_EUSERERROR / PDL_EFATAL. */
enum { PDLGB300_ENONE = 0, PDLGB300_EUSERERROR = 1, PDLGB300_EFATAL = 2 };

/* Replaces pdl_error (lib/PDL/Core/pdl.h.PL:370-379).  PDL's needs_free
 * says whether the caller frees the message; here the library always owns
 * it (a per-thread buffer), so there is nothing to free.  The XS glue
 * copies the text into croak() before the next library call. */
typedef struct pdlgb300_error {
  int32_t error;       /* PDLGB300_ENONE on success */
  int32_t reserved;
  const char *message; /* NUL-terminated; owned by the library, valid until the
                          next call on the same host thread; NULL on success */
} pdlgb300_error;

/* One value of any real type (PDL_Anyval, lib/PDL/Core/pdl.h.PL). */
typedef union pdlgb300_value {
  int8_t A; uint8_t B; int16_t S; uint16_t U; int32_t L; uint32_t K;
  int64_t N; uint64_t P; int64_t Q; float F; double D;
} pdlgb300_value;

typedef struct pdlgb300_anyval {
  int32_t type;        /* pdlgb300_datatype, or -1 for "none" */
  int32_t reserved;
  pdlgb300_value value;
} pdlgb300_anyval;

/* pdl->state bits that matter on this path. */
#define PDLGB300_BADVAL   0x1u /* PDL_BADVAL: the ndarray may contain bad values */
#define PDLGB300_NOMYDIMS 0x2u /* PDL_NOMYDIMS: a null output, shaped by the op */

typedef struct pdlgb300_ndarray {
  int32_t datatype;      /* pdlgb300_datatype */
  int32_t ndims;         /* 0..PDLGB300_MAXDIMS */
  uint32_t state;        /* PDLGB300_BADVAL | PDLGB300_NOMYDIMS */
  int32_t has_badvalue;  /* 1: use badvalue below; 0: the per-type default */
  pdlgb300_anyval badvalue;
  int64_t offs;          /* element offset of element (0,0,..) from data */
  void *data;            /* host memory of the physical data, or NULL */
  void *ddata;           /* device memory of the same data, or NULL */
  int64_t dims[PDLGB300_MAXDIMS];
  int64_t incs[PDLGB300_MAXDIMS]; /* element increments (may be 0 or < 0) */
} pdlgb300_ndarray;

/* Where an op finds its data: ddata when non-NULL (device-resident, no
 * copies), else data (host memory: the call copies inputs to the device and
 * outputs back, timed separately in pdlgb300_launch_info).  A null output
 * (PDLGB300_NOMYDIMS) with both pointers NULL is shaped, typed and allocated
 * on the device by the call (ddata set; release it with pdlgb300_free). */

/* ---- descriptor helpers ------------------------------------------------ */

/* Fill a descriptor for a contiguous ndarray (PDL's default increments:
 * dim 0 fastest, pdl_resize_defaultincs). */
pdlgb300_error pdlgb300_ndarray_init(pdlgb300_ndarray *x, int32_t datatype,
                                     int32_t ndims, const int64_t *dims,
                                     void *data, void *ddata);
/* A null output (PDL->null). */
pdlgb300_error pdlgb300_ndarray_null(pdlgb300_ndarray *x);
size_t pdlgb300_type_size(int32_t datatype);
const char *pdlgb300_type_name(int32_t datatype);

/* Default badvalue per type (PDL->bvals; defaults Types.pm defbval) and the
 * setter behind `byte->badvalue(23)` (lib/PDL/Bad.pd:83-256). */
pdlgb300_error pdlgb300_get_default_badvalue(int32_t datatype, pdlgb300_anyval *out);
pdlgb300_error pdlgb300_set_default_badvalue(int32_t datatype, pdlgb300_anyval val);

/* ---- vtables: the op signatures (pdl_transvtable, pdl.h.PL:381-403) ---- */

typedef struct pdlgb300_vtable {
  const char *name;
  int32_t npdls, nparents, ninds, nother;
  const char *const *par_names;      /* [npdls] */
  const int32_t *par_realdims;       /* [npdls] */
  const int32_t *par_flags;          /* [npdls] PDLGB300_PARAM_* */
  const int32_t *par_types;          /* [npdls] fixed type or -1 */
  const int32_t *ind_ids;            /* [sum realdims] index id of each real dim */
  const char *const *ind_names;      /* [ninds] */
  const int32_t *gentypes;           /* GenericTypes, terminated by -1 */
} pdlgb300_vtable;

#define PDLGB300_PARAM_ISOUT    0x01
#define PDLGB300_PARAM_ISCREAT  0x02
#define PDLGB300_PARAM_ISTYPED  0x04
#define PDLGB300_PARAM_ISTPLUS  0x08 /* "int+": max(typed, trans type) */

/* Look up an op by its PDL name ("sumover", "plus", "matmult", ...).
 * Returns NULL for an unknown name. */
const pdlgb300_vtable *pdlgb300_get_vtable(const char *name);

/* The Perl package that defines an op ("PDL::Ufunc::", "PDL::Ops::",
 * "PDL::Primitive::"; "" for an op PDL does not have): PDL names an op in
 * its error messages by the package-qualified pp_def name
 * (lib/PDL/PP.pm vtable names), so a caller forming PDL's text prefixes it. */
const char *pdlgb300_op_package(const char *name);

/* Host-only shaping: the type selection, dim checks and output creation of
 * pdl_type_coerce + pdl_redodims_default (lib/PDL/Core/pdlapi.c:829-869,
 * 1169-1327; lib/PDL/Core/pdlbroadcast.c:211-523).  Null outputs get their
 * datatype, ndims, dims and default incs; nothing is allocated or launched.
 * other_pars: the op's OtherPars (swap for plus/mult), may be NULL. */
pdlgb300_error pdlgb300_redodims(const pdlgb300_vtable *vt,
                                 pdlgb300_ndarray *const *pdls,
                                 const int64_t *other_pars);

/* Generic run: redodims + type conversion + bad-value flag propagation +
 * the GPU kernels (the readdata of the op), synchronised before return. */
pdlgb300_error pdlgb300_run(const pdlgb300_vtable *vt,
                            pdlgb300_ndarray *const *pdls,
                            const int64_t *other_pars);

/* ---- the ops: one entry per pdl_run_<op> (PP.pm:1836-1852) ------------ */
/* lib/PDL/Ufunc.pd:94-118   sumover/dsumover: a(n); int+ [o]b()           */
pdlgb300_error pdlgb300_run_sumover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_dsumover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
/* lib/PDL/Ufunc.pd:91-118   prodover/dprodover (stops at a zero product)  */
pdlgb300_error pdlgb300_run_prodover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_dprodover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
/* lib/PDL/Ufunc.pd:120-140  cumusumover/dcumusumover: a(n); [o]b(n)      */
pdlgb300_error pdlgb300_run_cumusumover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_dcumusumover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
/* lib/PDL/Ufunc.pd:413-444  average/daverage                              */
pdlgb300_error pdlgb300_run_average(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_daverage(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
/* lib/PDL/Ufunc.pd:446-500  minimum/maximum: a(n); [o]c();
 *                           minimum_ind/maximum_ind: a(n); indx [o]c()     */
pdlgb300_error pdlgb300_run_minimum(pdlgb300_ndarray *a, pdlgb300_ndarray *c);
pdlgb300_error pdlgb300_run_maximum(pdlgb300_ndarray *a, pdlgb300_ndarray *c);
pdlgb300_error pdlgb300_run_minimum_ind(pdlgb300_ndarray *a, pdlgb300_ndarray *c);
pdlgb300_error pdlgb300_run_maximum_ind(pdlgb300_ndarray *a, pdlgb300_ndarray *c);
/* lib/PDL/Ufunc.pd:143-187  a(n); [o]b() in a's type: andover (all good
 * elements nonzero), orover, xorover (an odd count nonzero), zcover (all
 * zero), bandover/borover/bxorover (bitwise, integer types; float inputs
 * work in longlong), firstnonzeroover (the first nonzero good element, else
 * the last good one).  All bad in bad-value mode gives BAD.               */
pdlgb300_error pdlgb300_run_andover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_orover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_xorover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_zcover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_bandover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_borover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_bxorover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_firstnonzeroover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
/* lib/PDL/Ufunc.pd:120-140  cumuprodover: a(n); int+ [o]b(n), the running
 * product (a bad element gives a bad output and leaves the product as it
 * is); dcumuprodover: double [o]b(n).                                     */
pdlgb300_error pdlgb300_run_cumuprodover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_dcumuprodover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
/* lib/PDL/Ufunc.pd:563-613  minmaximum: a(n); [o]cmin(); [o]cmax();
 * indx [o]cmin_ind(); indx [o]cmax_ind() -- bad and NaN elements skipped,
 * first index on ties; nothing left: all four BAD with their bad state.   */
pdlgb300_error pdlgb300_run_minmaximum(pdlgb300_ndarray *a, pdlgb300_ndarray *cmin,
                                       pdlgb300_ndarray *cmax, pdlgb300_ndarray *cmin_ind,
                                       pdlgb300_ndarray *cmax_ind);
/* lib/PDL/Ufunc.pd:744-1112, the sort-based functions, each with the
 * reference's quicksort (lib/PDL/Core/pdl.h.PL:618-640) so that equal keys,
 * NaN and signed zeros land where the reference puts them:
 *   qsort a(n); [o]b(n)           -- bad values moved to the end (:1040-1077)
 *   qsorti a(n); indx [o]indx(n)  -- bad indices from the end backwards (:1079-1112)
 *   medover / oddmedover a(n); [o]b()  (:878-903)
 *   pctover / oddpctover a(n); p(); [o]b()  (:975-1007)
 *   modeover data(n); [o]out(), integer types (:905-939)
 * medover .. oddpctover fail on an empty ndarray as the reference does.   */
pdlgb300_error pdlgb300_run_qsort(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_qsorti(pdlgb300_ndarray *a, pdlgb300_ndarray *indx);
pdlgb300_error pdlgb300_run_medover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_oddmedover(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_pctover(pdlgb300_ndarray *a, pdlgb300_ndarray *p,
                                    pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_oddpctover(pdlgb300_ndarray *a, pdlgb300_ndarray *p,
                                       pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_modeover(pdlgb300_ndarray *data, pdlgb300_ndarray *out);
/* lib/PDL/Ufunc.pd:1115-1231, the vector sorts, with the reference's vector
 * quicksort (lexicographic pdl_cmpvec, middle vector as pivot) so that
 * vectors comparing equal keep the reference's order:
 *   qsortvec a(n,m); [o]b(n,m)         -- vectors with a bad component to
 *                                          the end, the first of them last
 *   qsortveci a(n,m); indx [o]indx(m)  -- the same order as positions
 * An empty a leaves the outputs unwritten, as the reference does.       */
pdlgb300_error pdlgb300_run_qsortvec(pdlgb300_ndarray *a, pdlgb300_ndarray *b);
pdlgb300_error pdlgb300_run_qsortveci(pdlgb300_ndarray *a, pdlgb300_ndarray *indx);
/* lib/PDL/IO/FastRaw.pm:202-323: FastRaw files.  The header ("<name>.hdr"
 * unless `header` names one) holds "<type id>\n<ndims>\n<dim0> <dim1> ...\n".
 *   pdlgb300_fraw_header  -- shape and type x from the header (_read_frawhdr)
 *   pdlgb300_readfraw_into -- the file's bytes into x's memory: host `data`,
 *     or device `ddata` copied from a mapping of the file (a file that
 *     cannot be mapped, a pipe for one, streams through pinned staging
 *     buffers with the reads overlapping the copies); a short file leaves
 *     the rest zero, as readfraw's zeroes() does
 *   pdlgb300_writefraw    -- header and data of a contiguous x (writefraw)
 * Device-memory transfers of one device share its two pinned staging
 * buffers: concurrent calls from several host threads are safe but take
 * turns (each holds the buffers for its whole transfer).  */
pdlgb300_error pdlgb300_fraw_header(const char *name, const char *header, pdlgb300_ndarray *x);
pdlgb300_error pdlgb300_readfraw_into(const char *name, pdlgb300_ndarray *x);
pdlgb300_error pdlgb300_writefraw(const pdlgb300_ndarray *x, const char *name, const char *header);
/* A deferred expression of PDL::Ops binary ops (lib/PDL/Ops.pd:104-153,
 * 288-307) reduced over dim 0 by a PDL::Ufunc reduction in one pass, with
 * the result the ops and the reduction give one after the other
 * (lib/PDL/Ufunc.pd:94-187, 413-500).  No reference function is replaced:
 * the reference always materialises each op (the broadcast loop of
 * lib/PDL/Core/pdlbroadcast.c runs once per op).  Node k applies `op` (a
 * binary-op vtable) to operands a, b: 0..nleaf-1 the leaves, nleaf+j node
 * j < k; the last node is the expression.  Leaves share one type (int32,
 * int64, float or double); `out` null or of the reduction's output type.  */
typedef struct {
  const pdlgb300_vtable *op;
  int32_t a, b;
} pdlgb300_expr_node;
pdlgb300_error pdlgb300_run_expr_reduce(const pdlgb300_vtable *reduction, int32_t nleaf,
                                        pdlgb300_ndarray *const *leaves, int32_t nnode,
                                        const pdlgb300_expr_node *nodes, pdlgb300_ndarray *out);
/* lib/PDL/Ops.pd:104-153,288-289  plus/mult: a(); b(); [o]c(); int swap   */
pdlgb300_error pdlgb300_run_plus(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                 pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_mult(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                 pdlgb300_ndarray *c, int swap);
/* The other binary ops of lib/PDL/Ops.pd:290-307, same convention as
 * plus/mult (pdl_run_minus, pdl_run_divide, pdl_run_gt ... pdl_run_xor):
 * c = a op b in the working type (comparisons give 0 or 1; shiftleft,
 * shiftright, or2, and2, xor have the integer types as GenericTypes, so
 * float inputs work in longlong).  Integer division by zero and shifts by a
 * negative or too large count have no defined result in the reference's C. */
pdlgb300_error pdlgb300_run_minus(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                  pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_divide(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                   pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_gt(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                               pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_lt(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                               pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_le(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                               pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_ge(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                               pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_eq(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                               pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_ne(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                               pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_shiftleft(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                      pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_shiftright(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                       pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_or2(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_and2(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                 pdlgb300_ndarray *c, int swap);
pdlgb300_error pdlgb300_run_xor(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                pdlgb300_ndarray *c, int swap);
/* lib/PDL/Primitive.pd:48-76  inner: a(n); b(n); [o]c()                   */
pdlgb300_error pdlgb300_run_inner(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                  pdlgb300_ndarray *c);
/* lib/PDL/Primitive.pd:191-264  _matmult_int: a(t,h); b(w,t); [o]c(w,h).
 * The PMCode wrapper (dummy-padding, scalar shortcut, the "Dim mismatch in
 * matmult" check, Primitive.pd:196-210) is host logic above this call. */
pdlgb300_error pdlgb300_run_matmult(pdlgb300_ndarray *a, pdlgb300_ndarray *b,
                                    pdlgb300_ndarray *c);

/* Fused sumover(plus(mult(a,b),d)): a(n); b(n); d(n); int+ [o]c().
 * Exactly the composition of the three reference ops (each element's
 * product and sum rounded as PDL rounds them, bad values propagated as
 * Ops.pd:142-148 then skipped as Ufunc.pd:104-108), without materialising
 * the broadcast intermediates.  No single reference function: it replaces
 * the eager chain `sumover($a*$b+$d)`. */
pdlgb300_error pdlgb300_run_sumover_mult_plus(pdlgb300_ndarray *a,
                                              pdlgb300_ndarray *b,
                                              pdlgb300_ndarray *d,
                                              pdlgb300_ndarray *c);

/* Type conversion of one ndarray into another of the same dims
 * (pdlconv.c's converttypei; C conversion rules). */
pdlgb300_error pdlgb300_convert(const pdlgb300_ndarray *src, pdlgb300_ndarray *dst);

/* ---- adjoints (backward calls), float32/float64 ----------------------- */
/* Given the upstream gradient of an op's output, write the gradient of its
 * inputs.  Gradients of broadcast inputs are summed over the broadcast dims
 * they were expanded along (recomputed, never stored). ga/gb may be NULL to
 * skip that input.  Shapes: each gradient has its input's dims. */
pdlgb300_error pdlgb300_sumover_bwd(const pdlgb300_ndarray *gb, pdlgb300_ndarray *ga);
pdlgb300_error pdlgb300_average_bwd(const pdlgb300_ndarray *gb, pdlgb300_ndarray *ga);
pdlgb300_error pdlgb300_plus_bwd(const pdlgb300_ndarray *gc, pdlgb300_ndarray *ga,
                                 pdlgb300_ndarray *gb);
pdlgb300_error pdlgb300_mult_bwd(const pdlgb300_ndarray *gc, const pdlgb300_ndarray *a,
                                 const pdlgb300_ndarray *b, pdlgb300_ndarray *ga,
                                 pdlgb300_ndarray *gb);
pdlgb300_error pdlgb300_matmult_bwd(const pdlgb300_ndarray *gc, const pdlgb300_ndarray *a,
                                    const pdlgb300_ndarray *b, pdlgb300_ndarray *ga,
                                    pdlgb300_ndarray *gb);

/* ---- sumover without allocation --------------------------------------- */
/* No counterpart in the reference.  Same result as pdlgb300_run_sumover, for
 * callers that cannot let the library allocate device memory (a host that
 * hands the library a fixed device-memory budget, or code that must not
 * trigger the device-wide synchronisation an allocation or free can
 * cause).  Always runs the multi-block split form of the reduction, whose
 * per-split partial sums live in one fixed 1 MiB device array (per device,
 * held until the process exits); it calls no allocator.
 * - a and b must be device-resident (ddata set); b must already have
 *   sumover's output shape and type (no null output, no conversion).
 * - Rows are limited by the scratch: at most (1048576 - 256) / (2 * unit)
 *   rows, unit = accumulator + 8-byte count (16 bytes for float64,
 *   compensated float32 and 64-bit integers: 32760 rows; 12 bytes
 *   otherwise: 43680 rows).  More returns PDLGB300_EUSERERROR, whose text
 *   states the limit for the type.
 * - The first call on a device looks the array's device address up
 *   (cudaGetSymbolAddress); make that first call before any stream capture.
 * - Every call shares the array (it keeps the last call's partials; each
 *   call overwrites every slot it reads), so calls that overlap on the GPU
 *   (other streams, other host threads) race: serialise them. */
pdlgb300_error pdlgb300_sumover_noalloc(const pdlgb300_ndarray *a, pdlgb300_ndarray *b);

/* ---- options ------------------------------------------------------------ */
/* float32 matmult arithmetic. */
enum {
  PDLGB300_MATMULT_SIMT_FP32 = 0, /* FP32 FMA on CUDA cores, FP32 accumulate */
  PDLGB300_MATMULT_BF16X3 = 1,    /* 2 bf16 limbs, 3 tcgen05 products */
  PDLGB300_MATMULT_BF16X6 = 2,    /* 3 bf16 limbs, 6 tcgen05 products (default) */
  PDLGB300_MATMULT_SIMT_EXACT = 3 /* the reference's order and rounding: bit-identical */
};
/* float32 reductions: 1 = compensated (default), 0 = plain FP32 sums. */
#define PDLGB300_OPT_MATMULT_MODE 1
#define PDLGB300_OPT_F32_COMPENSATED 2
#define PDLGB300_OPT_DEBUG 3 /* 1: print planner decisions (PDLDEBUG_f) */
pdlgb300_error pdlgb300_set_option(int32_t option, int64_t value);
int64_t pdlgb300_get_option(int32_t option);

/* ---- device memory, mirrors and streams -------------------------------- */
/* The CUDA stream the library launches on (a cudaStream_t passed as a
 * pointer); NULL selects the legacy default stream. */
pdlgb300_error pdlgb300_set_stream(void *stream);
pdlgb300_error pdlgb300_device_alloc(size_t nbytes, void **dptr);
pdlgb300_error pdlgb300_free(void *dptr);
/* Explicit, separately timed mirror transfers (ndarray data buffer <->
 * its device mirror).  Synchronous. */
pdlgb300_error pdlgb300_to_device(void *dptr, const void *host, size_t nbytes);
pdlgb300_error pdlgb300_to_host(void *host, const void *dptr, size_t nbytes);
/* The same transfers enqueued on `stream` (a cudaStream_t passed as a
 * pointer; NULL: the library's stream) without waiting.  No counterpart in
 * the reference, which has no device: a caller that pipelines copies
 * against ops orders them with its own stream events, as with
 * cudaMemcpyAsync; `host` must stay valid (and page-locked, for the copy to
 * overlap anything) until that stream has passed the copy. */
pdlgb300_error pdlgb300_to_device_async(void *dptr, const void *host, size_t nbytes,
                                        void *stream);
pdlgb300_error pdlgb300_to_host_async(void *host, const void *dptr, size_t nbytes,
                                      void *stream);
pdlgb300_error pdlgb300_sync(void);
pdlgb300_error pdlgb300_device_count(int32_t *n);

/* What the last op did (cf. get_autopthread_actual, lib/PDL/Core.xs:564-575). */
typedef struct pdlgb300_launch_info {
  char op[32];
  char kernel[64];       /* planner's kernel choice */
  int32_t datatype;      /* trans datatype */
  int32_t nlaunches;     /* kernels launched by the op */
  int64_t grid, block;   /* of the main kernel */
  int64_t rows, n;       /* broadcast iterations and reduced/contracted length */
  double bytes;          /* algorithmic bytes (inputs once + outputs once) */
  double flops;
  double kernel_ms;      /* device time of the op's kernels (CUDA events) */
  double h2d_ms, d2h_ms; /* staging copies of host-resident operands */
  double h2d_bytes, d2h_bytes;
} pdlgb300_launch_info;
pdlgb300_error pdlgb300_last_launch(pdlgb300_launch_info *out);
/* 1: time every op with CUDA events (adds a sync); 0: no timing (default). */
pdlgb300_error pdlgb300_set_timing(int32_t on);

int32_t pdlgb300_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PDLGB300_H */
