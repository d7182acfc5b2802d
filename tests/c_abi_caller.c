/* A plain C99 caller of the C ABI: include/crg.h compiles as C, the shared
 * library links, and the entry points that need no GPU answer through it
 * (the ABI version, status strings, and argument refusals made before any
 * device work).  Built and run by tests/test_abi.py. */
#include <stdio.h>
#include <string.h>

#include "crg.h"

static int fails = 0;
#define EXPECT(cond)                                              \
    do {                                                          \
        if (!(cond)) {                                            \
            fprintf(stderr, "%s:%d: %s\n", __FILE__, __LINE__, #cond); \
            fails++;                                              \
        }                                                         \
    } while (0)

int main(void) {
    EXPECT(crg_abi_version() == CRG_ABI_VERSION);
    EXPECT(strcmp(crg_status_string(CRG_OK), "ok") == 0);
    EXPECT(strcmp(crg_status_string(CRG_ERR_DIMENSION_MISMATCH), "dimension mismatch") == 0);

    crg_regridder* r = (crg_regridder*)1;
    EXPECT(crg_build(NULL, NULL, NULL, &r) == CRG_ERR_INVALID_ARGUMENT);
    EXPECT(r == NULL);

    /* a 2 x 2 curvilinear grid whose ncells disagrees with its block */
    int64_t nx = 2, ny = 2;
    double pts[3 * 3 * 3] = {0};
    crg_grid_desc g;
    memset(&g, 0, sizeof g);
    g.kind = CRG_GRID_CURVILINEAR;
    g.manifold = CRG_SPHERICAL;
    g.nblocks = 1;
    g.ncells = 5;
    g.block_nx = &nx;
    g.block_ny = &ny;
    g.points = pts;
    crg_grid_desc ok = g;
    ok.ncells = 4;
    EXPECT(crg_build(&g, &ok, NULL, &r) == CRG_ERR_DIMENSION_MISMATCH);
    EXPECT(strstr(crg_last_error(), "destination grid: ncells = 5") != NULL);
    crg_build_opts opts = {1, 7, NULL};
    EXPECT(crg_build(&ok, &ok, &opts, &r) == CRG_ERR_INVALID_ARGUMENT); /* flags must be 0 */
    EXPECT(crg_regridder_release(NULL) == CRG_OK);
    EXPECT(crg_apply(NULL, 0, CRG_F32, NULL, 0, 0, NULL, 0, 0, 1, 1, NULL) == CRG_ERR_INVALID_ARGUMENT);

    if (fails) return 1;
    printf("c abi ok\n");
    return 0;
}
