/* PDL::GB300 -- PDL's own ndarrays on libpdlgb300's C ABI.
 *
 * The glue a PDL session uses to run this library's ops in place of
 * pdl_run_<op> (lib/PDL/PP.pm:1836-1852): a pdl* becomes a descriptor
 * (pdl_to_desc: dims, the vaffine increments and offset, the physical
 * data pointer, the bad-value state and the per-ndarray badvalue), null
 * outputs are shaped and typed by the library's redodims and then
 * allocated by PDL (PDL->setdims, PDL->allocdata), the op runs, and the
 * outputs get PDL's bad flag and a changed() notice.  Host data is staged
 * to the GPU by the library per call.  Built against PDL 2.106's
 * pdl.h/pdlcore.h; boots like any PP module (lib/PDL/API.pod:240-262). */
#include "EXTERN.h"
#include "perl.h"
#include "XSUB.h"

#include "pdl.h"
#include "pdlcore.h"

#include "pdlgb300.h"

static Core *PDL;

static void gb300_check(pdlgb300_error e) {
  if (e.error) croak("%s", e.message ? e.message : "PDL::GB300: error");
}

/* Explicit broadcast ids ($x->broadcast(...), broadcastI in
 * lib/PDL/Slices.pd:1819) regroup which dims broadcast together, and
 * pdl_initbroadcaststruct consumes them (lib/PDL/Core/pdlbroadcast.c:437-466);
 * the descriptor carries implicit broadcasting only, so a pdl with other ids
 * is refused rather than planned as implicit broadcasting. */
static void pdl_to_desc(pdl *p, pdlgb300_ndarray *d) {
  memset(d, 0, sizeof *d);
  d->datatype = p->datatype;
  d->badvalue.type = -1;
  if (p->state & PDL_NOMYDIMS) {
    d->state = PDLGB300_NOMYDIMS;
    return;
  }
  /* (dims, increments and broadcast ids are set by the view's redodims) */
  PDL->barf_if_error(PDL->make_physvaffine(p));
  if (p->nbroadcastids > 1 || (p->nbroadcastids == 1 && p->broadcastids[0] != p->ndims))
    croak("PDL::GB300: explicit broadcast ids (broadcast/broadcast1...) are not supported; "
          "use the PDL op");
  if (p->ndims > PDLGB300_MAXDIMS) croak("PDL::GB300: more than %d dims", PDLGB300_MAXDIMS);
  d->ndims = (int32_t)p->ndims;
  for (PDL_Indx i = 0; i < p->ndims; i++) {
    d->dims[i] = p->dims[i];
    d->incs[i] = PDL_REPRINCS(p)[i];  /* vaffine-aware */
  }
  d->offs = PDL_REPROFFS(p);
  d->data = PDL_REPRP(p);           /* the physical parent's data */
  if (p->state & PDL_BADVAL) d->state |= PDLGB300_BADVAL;
  d->has_badvalue = p->has_badvalue;
  if (p->has_badvalue) {
    d->badvalue.type = p->badvalue.type;
    memcpy(&d->badvalue.value, &p->badvalue.value, sizeof d->badvalue.value);
  }
}

/* The bad flag an op gives its outputs, as make_trans_mutual gives it
 * (lib/PDL/Core/pdlapi.c:806-808 calling pdl_propagate_badflag_dir,
 * :1052-1090, with newval 1): set on the pdl, forward to the children of
 * every transformation it feeds, and back to the parent of a pure vaffine
 * view (a slice that gets the flag gives it to the whole). */
static void propagate_bad(pdl *it, int is_fwd, int depth) {
  if (depth > 1000) croak("PDL::GB300: bad-flag propagation deeper than 1000");
  it->state |= PDL_BADVAL;
  pdl_trans *tp = it->trans_parent;
  int to_parents = !is_fwd ? tp != NULL
    : ((it->state & (PDL_OPT_VAFFTRANSOK | PDL_ALLOCATED)) == PDL_OPT_VAFFTRANSOK ||
       (tp && !(it->state & PDL_ALLOCATED) && (tp->flags & PDL_ITRANS_ISAFFINE)));
  if (to_parents)
    for (PDL_Indx i = 0; i < tp->vtable->nparents; i++)
      if (!(tp->pdls[i]->state & PDL_BADVAL)) propagate_bad(tp->pdls[i], 0, depth + 1);
  if (!is_fwd) return;
  for (PDL_Indx j = 0; j < it->ntrans_children_allocated; j++) {
    pdl_trans *t = it->trans_children[j];
    if (!t) continue;
    for (PDL_Indx i = t->vtable->nparents; i < t->vtable->npdls; i++)
      if (!(t->pdls[i]->state & PDL_BADVAL)) propagate_bad(t->pdls[i], 1, depth + 1);
  }
}

#define GB300_MAXP 8

/* Header propagation as an op's redodims makes it (pdl_hdr_childcopy,
 * lib/PDL/Core/pdlcore.c:872-906): the first ndarray with a header and the
 * hdrcpy flag that is not an output this call creates gives a deep copy
 * (PDL->hdr_copy) of its header to every output, with the flag. */
static void hdr_childcopy(const pdlgb300_vtable *vt, pdl **p, const int *wasnull) {
  SV *hdrp = NULL;
  for (int i = 0; i < vt->npdls; i++)
    if (!(i >= vt->nparents && wasnull[i]) && p[i]->hdrsv && (p[i]->state & PDL_HDRCPY)) {
      hdrp = (SV *)p[i]->hdrsv;
      break;
    }
  if (!hdrp) return;
  SV *copy = hdrp == &PL_sv_undef ? &PL_sv_undef : PDL->hdr_copy(hdrp);
  for (int i = vt->nparents; i < vt->npdls; i++) {
    if (p[i]->hdrsv != (void *)hdrp) {
      if (p[i]->hdrsv && p[i]->hdrsv != (void *)&PL_sv_undef) SvREFCNT_dec((SV *)p[i]->hdrsv);
      if (copy != &PL_sv_undef) SvREFCNT_inc(copy);
      p[i]->hdrsv = copy;
    }
    p[i]->state |= PDL_HDRCPY;
  }
  if (copy != &PL_sv_undef) SvREFCNT_dec(copy);
}

/* The checks PDL makes on a pdl's own state before an op, in its order:
 * a read-only output (pdl__transtype_select, lib/PDL/Core/pdlapi.c:1191-1194),
 * then an output with inward but no backward flow (pdl_trans_flow_null_checks,
 * :709, :726-729). */
static void output_checks(const pdlgb300_vtable *vt, pdl **p) {
  for (int i = vt->nparents; i < vt->npdls; i++)
    if (p[i]->state & PDL_READONLY)
      croak("%s%s error: output parameter %s is read-only", pdlgb300_op_package(vt->name),
            vt->name, vt->par_names[i]);
  for (int i = vt->nparents; i < vt->npdls; i++) {
    pdl_trans *tp = p[i]->trans_parent;
    if (tp && (tp->flags & PDL_ITRANS_DO_DATAFLOW_ANY) == PDL_ITRANS_DO_DATAFLOW_F)
      croak("%s%s: cannot output to parameter '%s' with inward but no backward flow",
            pdlgb300_op_package(vt->name), vt->name, vt->par_names[i]);
  }
}

static int get_pdls(AV *av, pdl **p, pdlgb300_ndarray *d, pdlgb300_ndarray **dp, int want) {
  const int np = (int)av_len(av) + 1;
  if (want >= 0 && np != want) croak("PDL::GB300: %d ndarrays given, %d wanted", np, want);
  if (np > GB300_MAXP) croak("PDL::GB300: too many ndarrays");
  for (int i = 0; i < np; i++) {
    SV **sv = av_fetch(av, i, 0);
    if (!sv) croak("PDL::GB300: missing ndarray %d", i);
    p[i] = PDL->SvPDLV(*sv);
    pdl_to_desc(p[i], &d[i]);
    dp[i] = &d[i];
  }
  return np;
}

MODULE = PDL::GB300  PACKAGE = PDL::GB300

PROTOTYPES: DISABLE

void
_run(name, pdls, other)
    char *name
    AV *pdls
    IV other
  CODE:
    const pdlgb300_vtable *vt = pdlgb300_get_vtable(name);
    if (!vt) croak("PDL::GB300: unknown op %s", name);
    pdl *p[GB300_MAXP];
    pdlgb300_ndarray d[GB300_MAXP], *dp[GB300_MAXP];
    get_pdls(pdls, p, d, dp, vt->npdls);
    output_checks(vt, p);
    int64_t oth[1] = {(int64_t)other};
    int inputs_bad = 0;
    for (int i = 0; i < vt->nparents; i++) inputs_bad |= !!(d[i].state & PDLGB300_BADVAL);
    int anynull = 0, wasnull[GB300_MAXP] = {0};
    for (int i = vt->nparents; i < vt->npdls; i++) {
      wasnull[i] = !!(d[i].state & PDLGB300_NOMYDIMS);
      anynull |= wasnull[i];
    }
    if (anynull) {
      /* null outputs: the library shapes and types them, PDL allocates */
      gb300_check(pdlgb300_redodims(vt, dp, oth));
      for (int i = vt->nparents; i < vt->npdls; i++) {
        if (!(p[i]->state & PDL_NOMYDIMS)) continue;
        PDL_Indx dims[PDLGB300_MAXDIMS];
        for (int k = 0; k < d[i].ndims; k++) dims[k] = d[i].dims[k];
        p[i]->datatype = d[i].datatype;
        PDL->barf_if_error(PDL->setdims(p[i], dims, d[i].ndims));
        PDL->barf_if_error(PDL->allocdata(p[i]));
        p[i]->state &= ~PDL_NOMYDIMS;
        pdl_to_desc(p[i], &d[i]);
      }
    }
    hdr_childcopy(vt, p, wasnull);
    gb300_check(pdlgb300_run(vt, dp, oth));
    for (int i = vt->nparents; i < vt->npdls; i++) {
      /* bad inputs flag the outputs and their views; an op that finds a
         bad result itself (PDLSTATESETBAD) flags the output alone */
      if (inputs_bad) propagate_bad(p[i], 1, 0);
      else if (d[i].state & PDLGB300_BADVAL) p[i]->state |= PDL_BADVAL;
      PDL->barf_if_error(PDL->changed(p[i], PDL_PARENTDATACHANGED, 0));
    }

void
_redodims(name, pdls, other)
    char *name
    AV *pdls
    IV other
  PPCODE:
    /* the shapes and types the op would give its null outputs, nothing run */
    const pdlgb300_vtable *vt = pdlgb300_get_vtable(name);
    if (!vt) croak("PDL::GB300: unknown op %s", name);
    pdl *p[GB300_MAXP];
    pdlgb300_ndarray d[GB300_MAXP], *dp[GB300_MAXP];
    get_pdls(pdls, p, d, dp, vt->npdls);
    int64_t oth[1] = {(int64_t)other};
    gb300_check(pdlgb300_redodims(vt, dp, oth));
    for (int i = vt->nparents; i < vt->npdls; i++) {
      AV *dims = newAV();
      for (int k = 0; k < d[i].ndims; k++) av_push(dims, newSViv((IV)d[i].dims[k]));
      XPUSHs(sv_2mortal(newSViv(d[i].datatype)));
      XPUSHs(sv_2mortal(newRV_noinc((SV *)dims)));
    }

void
_desc(sv)
    SV *sv
  PPCODE:
    /* the descriptor a pdl becomes: datatype, offs, state, has_badvalue,
       then [dims], [incs] */
    pdl *p = PDL->SvPDLV(sv);
    pdlgb300_ndarray d;
    pdl_to_desc(p, &d);
    AV *dims = newAV(), *incs = newAV();
    for (int k = 0; k < d.ndims; k++) {
      av_push(dims, newSViv((IV)d.dims[k]));
      av_push(incs, newSViv((IV)d.incs[k]));
    }
    XPUSHs(sv_2mortal(newSViv(d.datatype)));
    XPUSHs(sv_2mortal(newSViv((IV)d.offs)));
    XPUSHs(sv_2mortal(newSViv((IV)d.state)));
    XPUSHs(sv_2mortal(newSViv(d.has_badvalue)));
    XPUSHs(sv_2mortal(newRV_noinc((SV *)dims)));
    XPUSHs(sv_2mortal(newRV_noinc((SV *)incs)));

void
_bwd(name, pdls)
    char *name
    AV *pdls
  CODE:
    /* the backward calls; every gradient preallocated by the caller */
    pdl *p[GB300_MAXP];
    pdlgb300_ndarray d[GB300_MAXP], *dp[GB300_MAXP];
    const int np = get_pdls(pdls, p, d, dp, -1);
    int nout;
    if (!strcmp(name, "sumover_bwd") && np == 2) {
      gb300_check(pdlgb300_sumover_bwd(dp[0], dp[1]));
      nout = 1;
    } else if (!strcmp(name, "average_bwd") && np == 2) {
      gb300_check(pdlgb300_average_bwd(dp[0], dp[1]));
      nout = 1;
    } else if (!strcmp(name, "plus_bwd") && np == 3) {
      gb300_check(pdlgb300_plus_bwd(dp[0], dp[1], dp[2]));
      nout = 2;
    } else if (!strcmp(name, "mult_bwd") && np == 5) {
      gb300_check(pdlgb300_mult_bwd(dp[0], dp[1], dp[2], dp[3], dp[4]));
      nout = 2;
    } else if (!strcmp(name, "matmult_bwd") && np == 5) {
      gb300_check(pdlgb300_matmult_bwd(dp[0], dp[1], dp[2], dp[3], dp[4]));
      nout = 2;
    } else {
      croak("PDL::GB300: unknown backward call %s with %d ndarrays", name, np);
    }
    for (int i = np - nout; i < np; i++)
      PDL->barf_if_error(PDL->changed(p[i], PDL_PARENTDATACHANGED, 0));

void
_badval_warn(a, b, swap)
    SV *a
    SV *b
    IV swap
  CODE:
    /* The comparison ops' header (lib/PDL/Ops.pd:84-102, 127): after the
       swap, a and b each warn when the badvalue they would compare against
       (their own, or their type's default) is 0 or 1. */
    pdl *v[2] = {PDL->SvPDLV(swap ? b : a), PDL->SvPDLV(swap ? a : b)};
    static const char *name[2] = {"a", "b"};
    for (int i = 0; i < 2; i++) {
      pdl *x = v[i];
      if (x->has_badvalue && x->badvalue.type != x->datatype) continue;
      PDL_Anyval bv = PDL->get_pdl_badvalue(x);
      if (bv.type < 0) croak("Error getting badvalue, type=%d", bv.type);
      double bd;
      ANYVAL_TO_CTYPE(bd, double, bv);
      if (bd == 0 || bd == 1)
        warn("%s badvalue is set to 0 or 1. This will cause data loss when using badvalues "
             "for comparison operators.", name[i]);
    }

int
device_count()
  CODE:
    int32_t n = 0;
    pdlgb300_error e = pdlgb300_device_count(&n);
    RETVAL = e.error ? 0 : n;
  OUTPUT:
    RETVAL

BOOT:
  perl_require_pv("PDL/Core.pm");
  if (SvTRUE(ERRSV)) croak("%s", SvPV_nolen(ERRSV));
  {
    SV *CoreSV = perl_get_sv("PDL::SHARE", FALSE);
    if (!CoreSV) croak("PDL::GB300 needs PDL::Core ($PDL::SHARE not set)");
    if (!(PDL = INT2PTR(Core *, SvIV(CoreSV)))) croak("PDL::GB300: NULL Core pointer");
    if (PDL->Version != PDL_CORE_VERSION)
      croak("PDL::GB300 was built for PDL_CORE_VERSION %d, PDL has %d; rebuild it",
            PDL_CORE_VERSION, PDL->Version);
  }
