/* One gauge configuration through the C ABI from plain C99, as a caller that
 * replaces the reference's create_operators + contract does: infile, engine,
 * inputs, VdaggerV, contraction, one HDF5 file per diagram.
 * Usage: abi_contract <infile> <input dir> <output dir> <precision 0|1>
 * The input directory holds V_<t>.bin (one timeslice, column-major complex
 * doubles), P_<r>.bin (perambulator, re-sorted layout) and N_<r>.bin (noise). */
#include <stdio.h>
#include <stdlib.h>

#include "slaph_gb300.h"

static int fail(const char *what) {
  fprintf(stderr, "%s: %s\n", what, slaph_last_error());
  return 1;
}

/* Reads exactly n doubles from path into a new buffer. */
static double *load(const char *dir, const char *kind, int index, size_t n) {
  char path[4096];
  double *buf = malloc(n * sizeof(double));
  FILE *fp;
  snprintf(path, sizeof path, "%s/%s_%d.bin", dir, kind, index);
  fp = fopen(path, "rb");
  if (!buf || !fp || fread(buf, sizeof(double), n, fp) != n) {
    fprintf(stderr, "cannot read %s\n", path);
    exit(4);
  }
  fclose(fp);
  return buf;
}

int main(int argc, char **argv) {
  const char *args[] = {"--start_config", "1000", "--end_config", "1000"};
  slaph_frontend *fe = NULL;
  slaph_engine *eng = NULL;
  slaph_dims d;
  const slaph_plan *plan = NULL;
  double *corr;
  size_t dim_row, n_peram;
  int precision, t, r, k, i;
  int64_t n_out;
  if (argc < 5) return 2;
  precision = atoi(argv[4]) ? SLAPH_MIXED : SLAPH_FP64;
  if (slaph_frontend_create(argv[1], 4, args, &fe) != SLAPH_OK) return fail("create");
  if (slaph_frontend_dims(fe, &d) != SLAPH_OK) return fail("dims");
  if (slaph_frontend_plan(fe, &plan) != SLAPH_OK) return fail("plan");
  if (slaph_engine_create(&d, &eng) != SLAPH_OK) return fail("engine");
  if (slaph_engine_set_operators(eng, plan->vdv_ops, plan->n_vdv_ops, plan->index_of_unity) !=
      SLAPH_OK)
    return fail("operators");
  dim_row = 3 * (size_t)d.Lx * d.Ly * d.Lz;
  n_peram = 2 * (size_t)(4 * d.nev * d.Lt) * (size_t)(d.Lt / d.dilT * d.dilE * 4);
  for (t = 0; t < d.Lt; ++t) {
    double *v = load(argv[2], "V", t, 2 * dim_row * d.nev);
    if (slaph_engine_set_eigenvectors(eng, t, v) != SLAPH_OK) return fail("eigenvectors");
    free(v);
  }
  for (r = 0; r < d.n_rnd; ++r) {
    double *p = load(argv[2], "P", r, n_peram);
    double *n = load(argv[2], "N", r, 2 * (size_t)d.Lt * 4 * d.nev);
    if (slaph_engine_set_perambulator(eng, r, p) != SLAPH_OK) return fail("perambulator");
    if (slaph_engine_set_random_vector(eng, r, n) != SLAPH_OK) return fail("noise");
    free(p);
    free(n);
  }
  if (slaph_vdaggerv_build(eng, precision) != SLAPH_OK) return fail("build");
  n_out = slaph_plan_output_doubles(plan, d.Lt);
  corr = malloc((size_t)n_out * sizeof(double));
  if (!corr) return 5;
  if (slaph_contract(eng, plan, precision, SLAPH_ACC_NATIVE, -1, corr) != SLAPH_OK)
    return fail("contract");
  /* Diagram::write: one file per diagram, one dataset per request */
  k = 0;
  for (i = 0; i < plan->n_diagrams; ++i) {
    const slaph_diagram *dg = &plan->diagrams[i];
    const char **names;
    char path[4096];
    int j;
    if (dg->n_requests == 0) continue;
    names = malloc((size_t)dg->n_requests * sizeof(char *));
    for (j = 0; j < dg->n_requests; ++j) names[j] = dg->requests[j].dataset_name;
    snprintf(path, sizeof path, "%s/%s_cnfg1000.h5", argv[3], dg->name);
    if (slaph_write_correlators_h5(path, dg->n_requests, names, d.Lt,
                                   corr + 2 * (size_t)k * d.Lt) != SLAPH_OK)
      return fail("write");
    k += dg->n_requests;
    free((void *)names);
  }
  printf("wrote %d datasets\n", k);
  free(corr);
  slaph_engine_destroy(eng);
  slaph_frontend_destroy(fe);
  return 0;
}
