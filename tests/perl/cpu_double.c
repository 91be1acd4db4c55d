/* TEST DOUBLE of libpdlgb300 for the Perl glue, CPU only.
 *
 * The entry points PDL::GB300's XS calls (pdlgb300_get_vtable,
 * pdlgb300_redodims, pdlgb300_run, pdlgb300_device_count and the backward
 * calls), answered by the oracle's loops instead of the GPU, so that the
 * reference's own Perl tests can run through the glue -- descriptors of
 * PDL's views, null outputs allocated by PDL, bad flags, write-back, error
 * text -- on a machine without a GPU.  Linked only by
 * tests/test_perl_dropin.py into a scratch directory; the library's compute
 * is tested on the GPU by the -m gpu suite, never through this file. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pdlgb300.h"

int oracle_npdls(const char *opname);
int oracle_redodims(const char *opname, pdlgb300_ndarray **pdls, char *msg, size_t msglen);
int oracle_run(const char *opname, pdlgb300_ndarray **pdls_in, const int64_t *other,
               int nthreads, char *msg, size_t msglen);

const char *oracle_op_package(const char *name);
const char *oracle_par_name(const char *opname, int j);
int oracle_nparents(const char *opname);

static char msg[4096];

const char *pdlgb300_op_package(const char *name) { return oracle_op_package(name); }

static pdlgb300_error result(int rc) {
  pdlgb300_error e;
  memset(&e, 0, sizeof e);
  if (rc) {
    e.error = 1;
    e.message = msg;
  }
  return e;
}

#define NV 64
static pdlgb300_vtable vts[NV];
static int nvts;
static long nruns[NV];

/* With PDLGB300_DOUBLE_LOG set, the runs of each op are appended to that
 * file at exit: proof that the ops went through the glue. */
static void write_log(void) {
  const char *path = getenv("PDLGB300_DOUBLE_LOG");
  FILE *f = path ? fopen(path, "a") : NULL;
  if (!f) return;
  for (int i = 0; i < nvts; i++)
    if (nruns[i]) fprintf(f, "%s %ld\n", vts[i].name, nruns[i]);
  fclose(f);
}

const pdlgb300_vtable *pdlgb300_get_vtable(const char *name) {
  for (int i = 0; i < nvts; i++)
    if (!strcmp(vts[i].name, name)) return &vts[i];
  int np = oracle_npdls(name);
  if (np < 0 || nvts == NV) return NULL;
  if (nvts == 0) atexit(write_log);
  pdlgb300_vtable *v = &vts[nvts++];
  memset(v, 0, sizeof *v);
  v->name = strdup(name);
  const char **names = calloc((size_t)np, sizeof *names);
  for (int j = 0; j < np; j++) names[j] = oracle_par_name(name, j);
  v->par_names = names;
  v->npdls = np;
  v->nparents = oracle_nparents(name);
  return v;
}

pdlgb300_error pdlgb300_redodims(const pdlgb300_vtable *vt, pdlgb300_ndarray *const *pdls,
                                 const int64_t *other_pars) {
  (void)other_pars;
  msg[0] = 0;
  return result(oracle_redodims(vt->name, (pdlgb300_ndarray **)pdls, msg, sizeof msg));
}

pdlgb300_error pdlgb300_run(const pdlgb300_vtable *vt, pdlgb300_ndarray *const *pdls,
                            const int64_t *other_pars) {
  msg[0] = 0;
  nruns[vt - vts]++;
  return result(oracle_run(vt->name, (pdlgb300_ndarray **)pdls, other_pars, 1, msg, sizeof msg));
}

pdlgb300_error pdlgb300_device_count(int32_t *n) {
  *n = 0;
  return result(0);
}

static pdlgb300_error no_bwd(void) {
  snprintf(msg, sizeof msg, "PDL::GB300 test double: no backward calls");
  return result(1);
}
pdlgb300_error pdlgb300_sumover_bwd(const pdlgb300_ndarray *gb, pdlgb300_ndarray *ga) {
  (void)gb; (void)ga;
  return no_bwd();
}
pdlgb300_error pdlgb300_average_bwd(const pdlgb300_ndarray *gb, pdlgb300_ndarray *ga) {
  (void)gb; (void)ga;
  return no_bwd();
}
pdlgb300_error pdlgb300_plus_bwd(const pdlgb300_ndarray *gc, pdlgb300_ndarray *ga,
                                 pdlgb300_ndarray *gb) {
  (void)gc; (void)ga; (void)gb;
  return no_bwd();
}
pdlgb300_error pdlgb300_mult_bwd(const pdlgb300_ndarray *gc, const pdlgb300_ndarray *a,
                                 const pdlgb300_ndarray *b, pdlgb300_ndarray *ga,
                                 pdlgb300_ndarray *gb) {
  (void)gc; (void)a; (void)b; (void)ga; (void)gb;
  return no_bwd();
}
pdlgb300_error pdlgb300_matmult_bwd(const pdlgb300_ndarray *gc, const pdlgb300_ndarray *a,
                                    const pdlgb300_ndarray *b, pdlgb300_ndarray *ga,
                                    pdlgb300_ndarray *gb) {
  (void)gc; (void)a; (void)b; (void)ga; (void)gb;
  return no_bwd();
}
