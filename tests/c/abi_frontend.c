/* A plain C99 caller of the C ABI (no C++): parses an infile, reads the plan
 * and the file names a run needs, and checks an error path.  Needs no GPU.
 * Usage: abi_frontend <infile> */
#include <stdio.h>
#include <string.h>

#include "slaph_gb300.h"

static int fail(const char *what) {
  fprintf(stderr, "%s: %s\n", what, slaph_last_error());
  return 1;
}

int main(int argc, char **argv) {
  const char *args[] = {"--start_config", "1000", "--end_config", "1000"};
  slaph_frontend *fe = NULL;
  slaph_dims d;
  const slaph_plan *plan = NULL;
  char name[4096];
  int64_t start = 0;
  if (argc < 2) return 2;
  if (slaph_frontend_create(argv[1], 4, args, &fe) != SLAPH_OK) return fail("create");
  if (slaph_frontend_dims(fe, &d) != SLAPH_OK) return fail("dims");
  if (slaph_frontend_plan(fe, &plan) != SLAPH_OK) return fail("plan");
  if (slaph_frontend_get_int(fe, "start_config", &start) != SLAPH_OK) return fail("get_int");
  printf("dims %d %d %d %d nev %d dilT %d dilE %d n_rnd %d\n", d.Lt, d.Lx, d.Ly, d.Lz, d.nev,
         d.dilT, d.dilE, d.n_rnd);
  printf("ops %d diagrams %d outputs %lld start %lld\n", plan->n_vdv_ops, plan->n_diagrams,
         (long long)slaph_plan_output_doubles(plan, d.Lt), (long long)start);
  if (slaph_frontend_io_name(fe, 1000, 1, 0, name, sizeof name) != SLAPH_OK) return fail("io");
  printf("peram %s\n", name);
  if (slaph_vdaggerv_file_name("/cache", 1000, &plan->vdv_ops[1], 3, SLAPH_VDV_FILE_WRITE, name,
                               sizeof name) != SLAPH_OK)
    return fail("vdv name");
  printf("vdv %s\n", name);
  /* an unknown setting is an argument error with a message */
  if (slaph_frontend_get_int(fe, "no_such_key", &start) != SLAPH_ERR_ARG) return 3;
  printf("error %s\n", slaph_last_error());
  if (slaph_frontend_destroy(fe) != SLAPH_OK) return fail("destroy");
  return 0;
}
