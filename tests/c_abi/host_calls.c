/* A plain C caller of libstonewall.so: the entry points a C (or cgo / JNI) host would
 * bind, compiled against include/stonewall.h alone.  Host-only calls, no device work:
 * geometry, sizes, status strings, and argument checks that fail before any launch. */
#include <stdio.h>
#include <string.h>

#include "stonewall.h"

#define CHECK(cond)                                              \
  do {                                                           \
    if (!(cond)) {                                               \
      fprintf(stderr, "check failed: %s (line %d)\n", #cond, __LINE__); \
      return 1;                                                  \
    }                                                            \
  } while (0)

int main(void) {
  sw_geom g;
  CHECK(sw_geom_make(45, 7, 10, &g) == SW_OK);
  CHECK(g.nx == 45 && g.ny == 7 && g.nz == 10 && g.pitch == 64);
  CHECK(sw_cells_padded(&g) == 10 * 7 * 64);
  CHECK(sw_lattice_elems(&g) == 19LL * 10 * 7 * 64);
  CHECK(sw_tile_count(&g) == 10 * 7 * 2);
  CHECK(sw_dtype_size(SW_F32) == 4 && sw_dtype_size(SW_F16_SHIFT) == 2 && sw_dtype_size(SW_F64) == 8);
  CHECK(sw_geom_make(0, 4, 4, &g) == SW_ERR_BAD_ARG);
  CHECK(strstr(sw_version(), "sm_103a") != NULL);
  CHECK(strcmp(sw_status_string(SW_ERR_BAD_ARG), "bad argument") == 0);
  CHECK(sw_step_config_count() >= 4);
  /* argument checks happen on the host, before anything is launched */
  sw_geom h;
  CHECK(sw_geom_make(32, 4, 4, &h) == SW_OK);
  CHECK(sw_step(&h, SW_F32, NULL, NULL, NULL, NULL, NULL, 1e-3, 0.1, 20, 0.05, NULL, 0, NULL) == SW_ERR_BAD_ARG);
  CHECK(sw_step(&h, 9, (void *)16, (void *)32, (const uint8_t *)16, (const uint8_t *)16, (const float *)16, 1e-3,
                0.1, 20, 0.05, NULL, 0, NULL) == SW_ERR_BAD_ARG);
  CHECK(sw_batch_graph_create(NULL) == SW_ERR_BAD_ARG);
  /* a status word read back from the device maps to an error code */
  CHECK(sw_status_error(0) == SW_OK);
  CHECK(sw_status_error(SW_STATUS_NONFINITE) == SW_ERR_NONFINITE);
  CHECK(sw_status_error(SW_STATUS_NONFINITE | SW_STATUS_TIMEOUT) == SW_ERR_TIMEOUT);
  CHECK(sw_step_checked(&h, SW_F32, NULL, NULL, NULL, NULL, NULL, 1e-3, 0.1, 20, 0.05, NULL, 0, NULL, -1, NULL,
                        NULL) == SW_ERR_BAD_ARG);
  printf("c abi ok: %s\n", sw_version());
  return 0;
}
