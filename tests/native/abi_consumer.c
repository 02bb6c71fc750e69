/*
 * A plain C99 consumer of the harmonica_gb300 C ABI: it includes the public
 * headers in a C translation unit, links against libharmonica_gb300.so and
 * calls the entry points that validate their arguments before touching CUDA
 * (version, error text, workspace queries, argument checks), so it runs on
 * a machine without a GPU.  Exit status 0 means every check passed; a
 * failing check prints its line and returns 1.
 */
#include <stdio.h>
#include <string.h>

#include "harmonica_gb300.h"

static int failures = 0;

#define CHECK(cond)                                                    \
    do {                                                               \
        if (!(cond)) {                                                 \
            fprintf(stderr, "check failed at line %d: %s\n", __LINE__, \
                    #cond);                                            \
            failures++;                                                \
        }                                                              \
    } while (0)

int main(void) {
    size_t bytes = 0;
    const char *msg;

    CHECK(hg_version() >= 100);

    /* negative sizes are rejected before any CUDA call */
    CHECK(hg_prism_forward_workspace(-1, 10, HG_FIELD_MASK_ALL, &bytes) == HG_ERR_INVALID);
    msg = hg_last_error();
    CHECK(msg != NULL && strstr(msg, "bad sizes") != NULL);

    /* an empty field mask is rejected */
    CHECK(hg_prism_forward_workspace(10, 10, 0u, &bytes) == HG_ERR_INVALID);

    /* a valid query succeeds and reports the chunk partial sums */
    bytes = 0;
    CHECK(hg_prism_forward_workspace(2500, 10000, 1u << 3, &bytes) == HG_OK);

    /* tesseroid workspace holds the prepared records: 52 doubles per tesseroid */
    bytes = 0;
    CHECK(hg_tesseroid_forward_workspace(100, 1000, &bytes) == HG_OK);
    CHECK(bytes >= (size_t)52 * 1000 * sizeof(double));
    CHECK(hg_tesseroid_forward_workspace(-5, 1000, &bytes) == HG_ERR_INVALID);

    /* null device pointers with work to do are rejected */
    CHECK(hg_eqs_jacobian(NULL, NULL, NULL, 2, NULL, NULL, NULL, 3, 0, NULL, NULL) ==
          HG_ERR_INVALID);
    msg = hg_last_error();
    CHECK(msg != NULL && strstr(msg, "null pointer") != NULL);

    if (failures == 0) printf("abi consumer: all checks passed\n");
    return failures == 0 ? 0 : 1;
}
