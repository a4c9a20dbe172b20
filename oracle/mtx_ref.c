/* mtx_ref.c -- test harness around the reference's own Matrix Market readers.
 *
 * Test infrastructure only: built into oracle/_ref/ (never shipped) from the reference's
 * spmv_cuda/mmio.h, found through -I when the reference tree is present.  It runs the
 * reference's mm_read_banner (mmio.h:249) and mm_read_mtx_crd_size (mmio.h:334) on a file so
 * that the tests can pin the banner and size parsing of the Python restatement
 * (oracle/mtx_oracle.py) and of the library's loader to the reference itself.  Call it only on
 * files whose size line holds three integers: the reference's size reader does not return on
 * some malformed size lines. */
#include "mmio.h"

/* typecode: the reference's 4-character type code; returns the reference driver's status
 * (main.cu:582-604): 0, -1 fopen, -2 banner, -3 complex, -4 size. */
int ref_mtx_header(const char* path, char* typecode, int* m, int* n, int* nz) {
    FILE* f = fopen(path, "r");
    if (f == NULL) return -1;
    MM_typecode mc;
    if (mm_read_banner(f, &mc) != 0) {
        fclose(f);
        return -2;
    }
    memcpy(typecode, mc, 4);
    if (mm_is_complex(mc)) {
        fclose(f);
        return -3;
    }
    const int rc = mm_read_mtx_crd_size(f, m, n, nz);
    fclose(f);
    return rc != 0 ? -4 : 0;
}
