/* A plain C host of libvivsim_gb300: includes the public header, links the library and
 * calls entry points that validate their arguments before any CUDA call, so it runs
 * without a GPU.  Prints one line per check; exit status 0 when all hold. */
#include <stdio.h>
#include <string.h>

#include "vivsim_gb300.h"

static int fails = 0;

static void expect(int cond, const char* what) {
  printf("%s %s\n", cond ? "ok  " : "FAIL", what);
  if (!cond) ++fails;
}

int main(void) {
  char dummy[64];
  void* p = dummy;
  expect(vs_version() >= 100, "vs_version");
  expect(strcmp(vs_status_string(VS_OK), "ok") == 0, "vs_status_string(VS_OK)");
  expect(vs_streaming(7, VS_F32, p, p, 4, 4, 1, NULL) == VS_ERR_INVALID_ARG, "vs_streaming rejects q = 7");
  expect(strlen(vs_last_error()) > 0, "vs_last_error after a failure");
  expect(vs_fine_to_coarse(VS_F32, p, 5, 12, p, 7, 5, VS_REFINE_LEFT, NULL) == VS_ERR_INVALID_ARG,
         "vs_fine_to_coarse rejects mismatched interface extents");
  expect(vs_check_finite(VS_F32, NULL, 10, (int*)p, NULL) == VS_ERR_INVALID_ARG, "vs_check_finite rejects NULL");
  {
    vs_lattice_cfg cfg;
    vs_lattice_plan* plan = NULL;
    memset(&cfg, 0, sizeof(cfg));
    cfg.q = 9;
    cfg.dtype = VS_F32;
    cfg.nx = 2; /* too small: rejected before any allocation */
    cfg.ny = 16;
    cfg.nz = 1;
    expect(vs_lattice_plan_create(&cfg, &plan) == VS_ERR_INVALID_ARG && plan == NULL,
           "vs_lattice_plan_create rejects a 2 x 16 grid");
  }
  return fails ? 1 : 0;
}
