/* A plain C caller of include/dendro_gb300.h: the header compiles as C99
 * and the library's context-free entry points answer without a GPU.
 * Driven by tests/test_abi.py. */
#include <stdio.h>
#include <string.h>

#include "dendro_gb300.h"

int main(void) {
  if (dg_version() < 1) return 2;
  if (strcmp(dg_status_string(DG_OK), "ok") != 0) return 3;
  dg_octree o = NULL;
  /* no context: rejected before any device work */
  if (dg_octree_upload(NULL, NULL, 0, 31, 0, &o) != DG_ERR_INVALID_ARG) return 4;
  size_t n = 0;
  if (dg_sort_octants(NULL, NULL, 1, 30, 0, 0, NULL, 0, &n) != DG_ERR_INVALID_ARG) return 5;
  printf("{\"version\": %d}\n", dg_version());
  return 0;
}
