/*
 * bhsparse_spmv_cuda.h -- drop-in replacement for the reference's host class
 * (spmv_cuda/bhsparse_spmv_cuda.h:7-55 with spmv_cuda/common.h:24-66).
 *
 * A caller written against the reference (spmv_cuda/main.cu:431-545, 547-835) compiles
 * unchanged against this header and links against libspmv_gb300.so:
 *
 *   bhsparse_spmv_cuda *bhsparse = new bhsparse_spmv_cuda();
 *   bhsparse->init_platform();
 *   bhsparse->prepare_mem(m, n, nnzA, csrRowPtrA, csrColIdxA, csrValA, x, y);
 *   bhsparse->run_benchmark();
 *   bhsparse->get_y();
 *   bhsparse->free_platform();
 *   bhsparse->free_mem();
 *
 * As in the reference, value_type is double when USE_DOUBLE is non-zero and float
 * otherwise.  Defining BHSPARSE_VALUE_MODE selects a mixed form instead
 * (BHSP_VALUE_MIXED_F32 or BHSP_VALUE_MIXED_BF16; value_type is then double).
 * Every method forwards to the C ABI of spmv_gb300.h; errors come back as the int
 * status codes (the reference aborts through checkCudaErrors instead).
 */
#ifndef BHSPARSE_SPMV_CUDA_H
#define BHSPARSE_SPMV_CUDA_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include "spmv_gb300.h"

#ifndef USE_DOUBLE
#define USE_DOUBLE 1
#endif

#ifdef BHSPARSE_VALUE_MODE
typedef double value_type;
#define BHSPARSE_VALUE_TYPE_TAG BHSPARSE_VALUE_MODE
#elif USE_DOUBLE
typedef double value_type;
#define BHSPARSE_VALUE_TYPE_TAG BHSP_VALUE_F64
#else
typedef float value_type;
#define BHSPARSE_VALUE_TYPE_TAG BHSP_VALUE_F32
#endif

/* spmv_cuda/common.h:37 */
#ifndef NUM_RUN
#define NUM_RUN 200
#endif

/* Wall-clock timer with the reference's interface (spmv_cuda/common.h:51-66). */
struct bhsparse_timer {
    timeval t1, t2;
    void start() { gettimeofday(&t1, NULL); }
    double stop() {
        gettimeofday(&t2, NULL);
        return (t2.tv_sec - t1.tv_sec) * 1000.0 + (t2.tv_usec - t1.tv_usec) / 1000.0;
    }
};

class bhsparse_spmv_cuda {
public:
    bhsparse_spmv_cuda() : _h(NULL) { _status = bhsp_create(&_h, BHSPARSE_VALUE_TYPE_TAG); }
    ~bhsparse_spmv_cuda() { bhsp_destroy(_h); }

    int init_platform() { return _h ? bhsp_init_platform(_h) : _status; }
    int prepare_mem(int m, int n, int nnzA, int *csrRowPtrA, int *csrColIdxA, value_type *csrValA,
                    value_type *x, value_type *y) {
        return _h ? bhsp_prepare_mem(_h, m, n, nnzA, csrRowPtrA, csrColIdxA, csrValA, x, y) : _status;
    }
    int run_benchmark() { return _h ? bhsp_run_benchmark(_h) : _status; }
    void get_y() {
        if (_h) _status = bhsp_get_y(_h);
    }
    int free_platform() { return _h ? bhsp_free_platform(_h) : _status; }
    int free_mem() { return _h ? bhsp_free_mem(_h) : _status; }

    /* additions: the status of the last get_y(), the last error text, the handle */
    int last_status() const { return _status; }
    const char *last_error() const { return _h ? bhsp_last_error(_h) : "bhsp_create failed"; }
    bhsp_spmv *handle() { return _h; }

private:
    bhsparse_spmv_cuda(const bhsparse_spmv_cuda &);
    bhsparse_spmv_cuda &operator=(const bhsparse_spmv_cuda &);
    bhsp_spmv *_h;
    int _status;
};

#endif /* BHSPARSE_SPMV_CUDA_H */
