// A caller written against the reference's host class, compiled unchanged against
// include/bhsparse_spmv_cuda.h and linked with libspmv_gb300.so.  It follows the two flows
// of spmv_cuda/main.cu: the 6x6 known-answer mode `./spmv 0` (call_bhsparse_small,
// main.cu:431-545, here with the missing get_y() call added) and the benchmark flow
// (call_bhsparse, main.cu:547-835) on a seeded integer-valued random matrix, with the
// exact check against the serial loop (main.cu:748-767, 789-806) and the NUM_RUN timing
// loop and its print-out (main.cu:811-821).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bhsparse_spmv_cuda.h"

static unsigned long long lcg(unsigned long long &s) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return s >> 33;
}

static int small_case() {
    int m = 6, n = 6, nnzA = 15;
    int row_ptr[7] = {0, 3, 9, 11, 11, 12, 15};
    int col_idx[15] = {0, 2, 5, 0, 1, 2, 3, 4, 5, 2, 4, 4, 2, 3, 4};
    value_type val[15];
    for (int i = 0; i < 15; i++) val[i] = (value_type)(i + 1);
    value_type x[6], y[6], y_ref[6];
    for (int i = 0; i < n; i++) x[i] = 1.0;
    for (int i = 0; i < m; i++) {
        value_type sum = 0;
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; j++) sum += x[col_idx[j]] * val[j];
        y_ref[i] = sum;
    }
    memset(y, 0, sizeof(y));
    bhsparse_spmv_cuda *bhsparse = new bhsparse_spmv_cuda();
    int err = bhsparse->init_platform();
    if (!err) err = bhsparse->prepare_mem(m, n, nnzA, row_ptr, col_idx, val, x, y);
    if (!err) err = bhsparse->run_benchmark();
    bhsparse->get_y();
    int errors = 0;
    for (int i = 0; i < m; i++) errors += (y_ref[i] != y[i]);
    printf("(GPU) y = ");
    for (int i = 0; i < m; i++) printf("%g, ", (double)y[i]);
    printf("\n%s\n", (!err && !errors) ? "PASS!" : "NO PASS.");
    bhsparse->free_platform();
    bhsparse->free_mem();
    delete bhsparse;
    return (err || errors) ? 1 : 0;
}

static int random_case(int m, unsigned long long seed) {
    unsigned long long s = seed;
    int n = m;
    std::vector<int> row_ptr(m + 1, 0);
    for (int i = 0; i < m; i++) {
        int len = (int)(lcg(s) % 40);
        if (lcg(s) % 20 == 0) len = 0;  // empty rows
        if (lcg(s) % 5000 == 0) len = 3000;  // a few long rows
        row_ptr[i + 1] = row_ptr[i] + len;
    }
    int nnzA = row_ptr[m];
    std::vector<int> col(nnzA);
    std::vector<value_type> val(nnzA), x(n), y(m), y_ref(m);
    for (int i = 0; i < m; i++) {
        int c = (int)(lcg(s) % 7);
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; j++) {
            c += 1 + (int)(lcg(s) % 3);
            col[j] = c % n;
        }
    }
    for (int i = 0; i < nnzA; i++) val[i] = (value_type)(lcg(s) % 10);  // main.cu:736-739
    for (int i = 0; i < n; i++) x[i] = (value_type)(lcg(s) % 10);       // main.cu:741-743
    for (int i = 0; i < m; i++) {
        value_type sum = 0;
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; j++) sum += x[col[j]] * val[j];
        y_ref[i] = sum;
    }
    double gb = (double)((m + 1 + nnzA) * sizeof(int) + (2 * nnzA + m) * sizeof(value_type));
    double gflop = (double)(2 * nnzA);
    bhsparse_spmv_cuda *bhsparse = new bhsparse_spmv_cuda();
    int err = bhsparse->init_platform();
    if (!err) err = bhsparse->prepare_mem(m, n, nnzA, row_ptr.data(), col.data(), val.data(),
                                          x.data(), y.data());
    if (!err) err = bhsparse->run_benchmark();
    bhsparse->get_y();
    int errors = 0;
    for (int i = 0; i < m; i++) errors += (y_ref[i] != y[i]);
    if (err || errors) {
        printf("NO PASS. err = %d (%s), error count = %d out of %d\n", err, bhsparse->last_error(),
               errors, m);
    } else {
        printf("PASS!\n");
        bhsparse_timer t;
        t.start();
        for (int i = 0; i < NUM_RUN; i++) err |= bhsparse->run_benchmark();
        double time = t.stop() / (double)NUM_RUN;
        printf("bhSPARSE time = %g ms. Bandwidth = %g GB/s. GFlops = %g GFlops.\n", time,
               gb / (1.0e+6 * time), gflop / (1.0e+6 * time));
    }
    bhsparse->free_platform();
    bhsparse->free_mem();
    delete bhsparse;
    return (err || errors) ? 1 : 0;
}

int main(int argc, char **argv) {
    if (argc > 1 && strcmp(argv[1], "0") == 0) return small_case();
    int m = argc > 2 ? atoi(argv[2]) : 200000;
    unsigned long long seed = argc > 3 ? strtoull(argv[3], NULL, 10) : 1;
    return random_case(m, seed);
}
