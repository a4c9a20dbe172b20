// ref_harness.cpp -- compiles the reference's own host loops (test infrastructure).
//
// The three .inc files are regions of the reference's sources cut out at build time by
// oracle/extract_ref.py into oracle/_ref/ (see that script for the anchors):
//   calib.inc  -- spmv_cuda/bhsparse_spmv_cuda.h, run_benchmark's host calibration
//                 (inter-warp += of the synchronizer, speculative fix-up of dirty tiles);
//   serial.inc -- spmv_cuda/main.cu, the serial CSR loop (y_ref);
//   omp.inc    -- spmv_cuda/main.cu, the OpenMP CSR loop.
// Each is included inside a function whose parameters carry the names the block uses, so
// what runs is the reference's code.  value_type is the reference's USE_DOUBLE typedef
// (spmv_cuda/common.h:27-31); USE_SVM_ALWAYS = 0 selects the host-array branch of the OpenMP
// loop, as the reference's Makefile builds it.  Only the oracle's tests and bench.py's CPU
// legs load the result (oracle/_ref/libref.so).
#include <omp.h>

#include <cstring>

#define USE_SVM_ALWAYS 0

namespace {

template <typename value_type>
void calibrate(int _threadbunch_num, const int* _svm_synchronizer_idx,
               const value_type* _svm_synchronizer_val, value_type* _svm_y,
               const int* _svm_dirty_counter, value_type* _svm_y_temp, const int* _svm_speculator,
               const int* _svm_csrRowPtrA, int _m) {
#include "calib.inc"
}

template <typename value_type>
void serial(int m, const int* csrRowPtrA, const int* csrColIdxA, const value_type* csrValA,
            const value_type* x, value_type* y_ref) {
    int ref_iter = 1;
#include "serial.inc"
}

template <typename value_type>
void openmp(int m, const int* csrRowPtrA, const int* csrColIdxA, const value_type* csrValA,
            const value_type* x, value_type* y_omp_ref, int NUM_RUN, int threads) {
    omp_set_num_threads(threads);
#include "omp.inc"
}

}  // namespace

// Host calibration of run_benchmark.  y, y_temp and row_ptr must hold m + 1 entries: when the
// matrix's last tile is dirty the reference reads row_ptr[m + 1] and writes y[m], which the
// extra entry keeps inside the buffers (the caller pads row_ptr[m + 1] = row_ptr[m]).
extern "C" void ref_calibrate_f64(int nwarps, const int* sync_idx, const double* sync_val, double* y,
                                  int ndirty, double* y_temp, const int* spec, const int* row_ptr,
                                  int m) {
    calibrate<double>(nwarps, sync_idx, sync_val, y, &ndirty, y_temp, spec, row_ptr, m);
}
extern "C" void ref_calibrate_f32(int nwarps, const int* sync_idx, const float* sync_val, float* y,
                                  int ndirty, float* y_temp, const int* spec, const int* row_ptr,
                                  int m) {
    calibrate<float>(nwarps, sync_idx, sync_val, y, &ndirty, y_temp, spec, row_ptr, m);
}

// The serial CSR loop (one pass).
extern "C" void ref_serial_f64(int m, const int* row_ptr, const int* col, const double* val,
                               const double* x, double* y) {
    serial<double>(m, row_ptr, col, val, x, y);
}
extern "C" void ref_serial_f32(int m, const int* row_ptr, const int* col, const float* val,
                               const float* x, float* y) {
    serial<float>(m, row_ptr, col, val, x, y);
}

// The OpenMP CSR loop: `runs` passes on `threads` host threads.
extern "C" void ref_omp_f64(int m, const int* row_ptr, const int* col, const double* val,
                            const double* x, double* y, int runs, int threads) {
    openmp<double>(m, row_ptr, col, val, x, y, runs, threads);
}
extern "C" void ref_omp_f32(int m, const int* row_ptr, const int* col, const float* val,
                            const float* x, float* y, int runs, int threads) {
    openmp<float>(m, row_ptr, col, val, x, y, runs, threads);
}
