// spmv_main.cpp -- the benchmark driver of the reference (spmv_cuda/main.cu) on this library.
//
//   spmv 0                         the 6x6 known-answer mode (call_bhsparse_small, main.cu:431-545)
//   spmv <file.mtx> [options]      the file mode (call_bhsparse, main.cu:547-835)
//   options: --runs N (timed calls per method, default NUM_RUN = 200), --seed S (values),
//            --no-compare (skip the CSR-vector, cuSPARSE and OpenMP comparisons)
//
// As in the reference: the matrix is loaded from a Matrix Market file (include/spmv_mtx.h), its
// values and x are replaced by integers 0..9 (main.cu:735-743; here seeded instead of taken from
// the clock, bhsp_gen_uniform_int), y is computed by the serial CSR loop (main.cu:748-767), the
// comparators run (CSR-vector with the CUSP schedule, call_cusp_ref main.cu:186-335; cuSPARSE,
// call_cusparse_ref main.cu:49-183; OpenMP at the reference's 4 threads and at every host
// thread, call_omp_ref main.cu:337-429), then the drop-in class (include/bhsparse_spmv_cuda.h)
// runs y = A.x, is checked for exact equality (main.cu:789-806) and timed over NUM_RUN calls
// (main.cu:811-821), each printed in the reference's format with its bytes formula
// (main.cu:688).  Differences: get_y()
// is called before the check (the reference checks y without it), and every method's result is
// checked, not only the first.
#include <cuda_runtime.h>
#include <omp.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "bhsparse_spmv_cuda.h"
#include "spmv_compare.h"
#include "spmv_gen.h"
#include "spmv_mtx.h"

namespace {

int g_runs = NUM_RUN;
unsigned long long g_seed = 1;
bool g_compare = true;

struct Csr {
    int m = 0, n = 0, nnz = 0;
    std::vector<int> row_ptr, col;
    std::vector<value_type> val;
};

double g_gb = 0.0, g_gflop = 0.0;

void print_rate(const char* what, double ms) {
    printf("%s time = %g ms. Bandwidth = %g GB/s. GFlops = %g GFlops.\n", what, ms,
           g_gb / (1.0e+6 * ms), g_gflop / (1.0e+6 * ms));
}

int count_errors(const std::vector<value_type>& y, const std::vector<value_type>& y_ref) {
    int e = 0;
    for (size_t i = 0; i < y_ref.size(); i++) e += (y[i] != y_ref[i]);
    return e;
}

void report_check(const char* what, int errors, int m) {
    printf("\nChecking %s SpMV Correctness ... ", what);
    if (errors)
        printf("NO PASS. Error count = %d out of %d entries.\n", errors, m);
    else
        printf("PASS!\n");
}

void serial(const Csr& a, const std::vector<value_type>& x, std::vector<value_type>& y) {
    for (int i = 0; i < a.m; i++) {
        value_type sum = 0;
        for (int j = a.row_ptr[i]; j < a.row_ptr[i + 1]; j++) sum += x[a.col[j]] * a.val[j];
        y[i] = sum;
    }
}

void omp_spmv(const Csr& a, const std::vector<value_type>& x, std::vector<value_type>& y,
              int threads) {
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int i = 0; i < a.m; i++) {
        value_type sum = 0;
        for (int j = a.row_ptr[i]; j < a.row_ptr[i + 1]; j++) sum += x[a.col[j]] * a.val[j];
        y[i] = sum;
    }
}

int value_tag() { return BHSPARSE_VALUE_TYPE_TAG == BHSP_VALUE_F32 ? BHSP_VALUE_F32 : BHSP_VALUE_F64; }

// CSR-vector and cuSPARSE on device copies of A and x (main.cu:49-183, 186-335)
int gpu_comparators(const Csr& a, const std::vector<value_type>& x,
                    const std::vector<value_type>& y_ref) {
    if (BHSPARSE_VALUE_TYPE_TAG != BHSP_VALUE_F64 && BHSPARSE_VALUE_TYPE_TAG != BHSP_VALUE_F32)
        return 0;  // the mixed forms have no comparator in this precision
    int *d_rp = nullptr, *d_col = nullptr;
    value_type *d_val = nullptr, *d_x = nullptr, *d_y = nullptr;
    const size_t vs = sizeof(value_type);
    if (cudaMalloc(&d_rp, (a.m + 1) * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&d_col, (a.nnz > 0 ? a.nnz : 1) * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&d_val, (a.nnz > 0 ? a.nnz : 1) * vs) != cudaSuccess ||
        cudaMalloc(&d_x, (a.n > 0 ? a.n : 1) * vs) != cudaSuccess ||
        cudaMalloc(&d_y, (a.m > 0 ? a.m : 1) * vs) != cudaSuccess) {
        printf("comparators: cudaMalloc failed\n");
        return 1;
    }
    cudaMemcpy(d_rp, a.row_ptr.data(), (a.m + 1) * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(d_col, a.col.data(), a.nnz * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(d_val, a.val.data(), a.nnz * vs, cudaMemcpyHostToDevice);
    cudaMemcpy(d_x, x.data(), a.n * vs, cudaMemcpyHostToDevice);
    std::vector<value_type> y(a.m);
    int failures = 0;

    // CSR-vector with the CUSP schedule (width from nnz / m)
    const int tpv = bhsp_csr_vector_width(a.m, a.nnz);
    printf("\nCSR-vector is using dedicated GPU memory, %d threads per row.", tpv);
    cudaMemset(d_y, 0, a.m * vs);
    int rc = bhsp_csr_vector(value_tag(), a.m, d_rp, d_col, d_val, d_x, d_y, tpv, nullptr);
    cudaDeviceSynchronize();
    cudaMemcpy(y.data(), d_y, a.m * vs, cudaMemcpyDeviceToHost);
    int errors = rc ? a.m : count_errors(y, y_ref);
    report_check("CSR-vector", errors, a.m);
    failures += errors != 0;
    if (!errors) {
        bhsparse_timer t;
        t.start();
        for (int i = 0; i < g_runs; i++)
            bhsp_csr_vector(value_tag(), a.m, d_rp, d_col, d_val, d_x, d_y, tpv, nullptr);
        cudaDeviceSynchronize();
        print_rate("CSR-vector", t.stop() / g_runs);
    }

    // cuSPARSE generic SpMV
    printf("\ncuSPARSE (cusparseSpMV, CSR_ALG1) is using dedicated GPU memory.");
    bhsp_cusparse* cs = nullptr;
    rc = bhsp_cusparse_create(&cs, value_tag(), a.m, a.n, a.nnz, d_rp, d_col, d_val, d_x, d_y,
                              nullptr);
    if (rc == BHSP_CMP_UNAVAILABLE) {
        printf("\ncuSPARSE is not available on this host (status %d).\n", rc);
    } else if (rc != 0) {
        printf("\ncuSPARSE set-up failed (status %d).\n", rc);
        failures++;
    } else {
        cudaMemset(d_y, 0, a.m * vs);
        rc = bhsp_cusparse_run(cs);
        cudaDeviceSynchronize();
        cudaMemcpy(y.data(), d_y, a.m * vs, cudaMemcpyDeviceToHost);
        errors = rc ? a.m : count_errors(y, y_ref);
        report_check("cuSPARSE", errors, a.m);
        failures += errors != 0;
        if (!errors) {
            bhsparse_timer t;
            t.start();
            for (int i = 0; i < g_runs; i++) bhsp_cusparse_run(cs);
            cudaDeviceSynchronize();
            print_rate("cuSPARSE", t.stop() / g_runs);
        }
        bhsp_cusparse_destroy(cs);
    }
    cudaFree(d_rp);
    cudaFree(d_col);
    cudaFree(d_val);
    cudaFree(d_x);
    cudaFree(d_y);
    return failures;
}

// OpenMP CSR loop at the reference's 4 threads (main.cu:370) and at every host thread
int omp_comparators(const Csr& a, const std::vector<value_type>& x,
                    const std::vector<value_type>& y_ref) {
    int failures = 0;
    const int all = omp_get_max_threads();
    for (int threads : {4, all}) {
        std::vector<value_type> y(a.m);
        printf("\nOpenMP is using dedicated HOST memory, %d threads.", threads);
        omp_spmv(a, x, y, threads);
        const int errors = count_errors(y, y_ref);
        report_check("OpenMP", errors, a.m);
        failures += errors != 0;
        if (!errors) {
            const int runs = g_runs < 20 ? g_runs : 20;
            bhsparse_timer t;
            t.start();
            for (int i = 0; i < runs; i++) omp_spmv(a, x, y, threads);
            print_rate("OpenMP", t.stop() / runs);
        }
        if (all == 4) break;
    }
    return failures;
}

int run_matrix(Csr& a, const std::vector<value_type>& x, bool print_vectors) {
    g_gb = (double)((a.m + 1 + (double)a.nnz) * sizeof(int) + (2.0 * a.nnz + a.m) * sizeof(value_type));
    g_gflop = 2.0 * a.nnz;

    std::vector<value_type> y_ref(a.m), y(a.m, 0);
    bhsparse_timer ref_timer;
    ref_timer.start();
    serial(a, x, y_ref);
    print_rate("cpu sequential", ref_timer.stop());

    bhsparse_spmv_cuda* bhsparse = new bhsparse_spmv_cuda();
    int err = bhsparse->init_platform();
    printf("Initializing CUDA platform ... %s\n", err ? "Failed." : "Done.");
    if (err) {
        printf("Error code = %d (%s)\n", err, bhsparse->last_error());
        delete bhsparse;
        return 1;
    }
    int failures = 0;
    if (g_compare) {
        failures += gpu_comparators(a, x, y_ref);
        failures += omp_comparators(a, x, y_ref);
    }

    err = bhsparse->prepare_mem(a.m, a.n, a.nnz, a.row_ptr.data(), a.col.data(), a.val.data(),
                                const_cast<value_type*>(x.data()), y.data());
    if (!err) err = bhsparse->run_benchmark();
    if (!err) bhsparse->get_y();
    if (print_vectors) {
        printf("\n(CPU) y = ");
        for (int i = 0; i < a.m; i++) printf("%g, ", (double)y_ref[i]);
        printf("\n(GPU) y = ");
        for (int i = 0; i < a.m; i++) printf("%g, ", (double)y[i]);
        printf("\n");
    }
    const int errors = err ? a.m : count_errors(y, y_ref);
    report_check("bhSPARSE", errors, a.m);
    if (err) printf("status %d: %s\n", err, bhsparse->last_error());
    failures += errors != 0;
    if (!errors) {
        bhsparse_timer t;
        t.start();
        for (int i = 0; i < g_runs; i++) err |= bhsparse->run_benchmark();
        const double ms = t.stop() / g_runs;
        printf("\n");
        print_rate("bhSPARSE", ms);
        failures += err != 0;
    }
    bhsparse->free_platform();
    bhsparse->free_mem();
    delete bhsparse;
    return failures ? 1 : 0;
}

int small_case() {
    Csr a;
    a.m = 6;
    a.n = 6;
    a.nnz = 15;
    a.row_ptr = {0, 3, 9, 11, 11, 12, 15};
    a.col = {0, 2, 5, 0, 1, 2, 3, 4, 5, 2, 4, 4, 2, 3, 4};
    for (int i = 0; i < 15; i++) a.val.push_back((value_type)(i + 1));
    printf("row_ptr = [ ");
    for (int v : a.row_ptr) printf("%d, ", v);
    printf(" ]\ncol_idx = [ ");
    for (int v : a.col) printf("%d, ", v);
    printf(" ]\nvalue   = [ ");
    for (value_type v : a.val) printf("%g, ", (double)v);
    printf(" ]\n\n");
    std::vector<double> xr(a.n);
    bhsp_gen_uniform_int(a.n, g_seed, 10, xr.data());  // main.cu:474-476: x = rand() % 10
    std::vector<value_type> x(xr.begin(), xr.end());
    return run_matrix(a, x, true);
}

int file_case(const char* path) {
    printf("PRECISION = %s\n", sizeof(value_type) == 8 ? "64-bit Double Precision"
                                                       : "32-bit Single Precision");
    printf("RUN SpMV %d times\n", g_runs);
    bhsp_mtx* h = nullptr;
    const int rc = bhsp_mtx_load(path, &h);
    if (rc != BHSP_MTX_OK) {
        switch (rc) {
            case BHSP_MTX_BAD_BANNER: printf("Could not process Matrix Market banner.\n"); break;
            case BHSP_MTX_COMPLEX: printf("Sorry, data type 'COMPLEX' is not supported. \n"); break;
            default: printf("Could not load %s (status %d).\n", path, rc); break;
        }
        return rc;
    }
    bhsp_mtx_info info;
    bhsp_mtx_get_info(h, &info);
    Csr a;
    a.m = info.m;
    a.n = info.n;
    a.nnz = info.nnz;
    a.row_ptr.assign(bhsp_mtx_row_ptr(h), bhsp_mtx_row_ptr(h) + a.m + 1);
    a.col.assign(bhsp_mtx_col_idx(h), bhsp_mtx_col_idx(h) + a.nnz);
    bhsp_mtx_free(h);
    printf(" ( %d, %d ) nnz = %d\n", a.m, a.n, a.nnz);
    // main.cu:735-743: values and x replaced by integers 0..9
    std::vector<double> vr(a.nnz), xr(a.n);
    bhsp_gen_uniform_int(a.nnz, g_seed, 10, vr.data());
    bhsp_gen_uniform_int(a.n, g_seed + 1, 10, xr.data());
    a.val.assign(vr.begin(), vr.end());
    std::vector<value_type> x(xr.begin(), xr.end());
    return run_matrix(a, x, false);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        printf("usage: %s 0 | <file.mtx> [--runs N] [--seed S] [--no-compare]\n", argv[0]);
        return 2;
    }
    for (int i = 2; i < argc; i++) {
        if (!strcmp(argv[i], "--runs") && i + 1 < argc)
            g_runs = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--seed") && i + 1 < argc)
            g_seed = strtoull(argv[++i], nullptr, 10);
        else if (!strcmp(argv[i], "--no-compare"))
            g_compare = false;
    }
    if (g_runs < 1) g_runs = 1;
    int err;
    if (strcmp(argv[1], "0") == 0) {
        err = small_case();
    } else {
        printf("--------------%s--------------\n", argv[1]);
        err = file_case(argv[1]);
    }
    printf("------------------------------------------------------\n");
    return err;
}
