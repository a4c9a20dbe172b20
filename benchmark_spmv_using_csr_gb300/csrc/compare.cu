// compare.cu -- the comparators of include/spmv_compare.h: the CSR-vector kernel and
// cuSPARSE's generic SpMV (loaded at run time).
#include <cuda_runtime.h>
#include <cusparse.h>
#include <dlfcn.h>

#include <mutex>

#include "../../include/spmv_compare.h"
#include "../../include/spmv_gb300.h"
#include "internal.h"

namespace {

// One vector of TPV lanes per row, grid-stride over rows (the CSR-vector schedule of
// spmv_cuda/kernels_cuda.h:273-342): lane j of a vector accumulates entries row_start + j,
// + TPV, ..., serially in its lane, then the vector reduces its TPV partial sums by shuffles
// (a tree: lanes j and j + d for d = TPV/2, ..., 1, as the reference's shared-memory
// reduction).  Rows longer than 32 entries with TPV = 32 start at the 32-aligned entry below
// row_start, as the reference does for coalescing.
template <typename VT, int TPV>
__global__ void __launch_bounds__(256) k_csr_vector(int m, const int* __restrict__ row_ptr,
                                                    const int* __restrict__ col,
                                                    const VT* __restrict__ val,
                                                    const VT* __restrict__ x, VT* __restrict__ y) {
    const int lane = threadIdx.x & (TPV - 1);
    const long long vec = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / TPV;
    const long long nvec = (long long)gridDim.x * blockDim.x / TPV;  // 64-bit: m may be near 2^31
    const unsigned mask = TPV == 32 ? 0xffffffffu
                                    : (((1u << TPV) - 1u) << ((threadIdx.x & 31) & ~(TPV - 1)));
    for (long long row = vec; row < m; row += nvec) {
        const int rs = __ldg(row_ptr + row);
        const int re = __ldg(row_ptr + row + 1);
        VT sum = VT(0);
        if (TPV == 32 && re - rs > 32) {
            int jj = rs - (rs & (TPV - 1)) + lane;
            if (jj >= rs && jj < re) sum += __ldg(val + jj) * __ldg(x + __ldg(col + jj));
            for (jj += TPV; jj < re; jj += TPV) sum += __ldg(val + jj) * __ldg(x + __ldg(col + jj));
        } else {
            for (int jj = rs + lane; jj < re; jj += TPV)
                sum += __ldg(val + jj) * __ldg(x + __ldg(col + jj));
        }
#pragma unroll
        for (int d = TPV / 2; d > 0; d >>= 1) sum += __shfl_down_sync(mask, sum, d, TPV);
        if (lane == 0) y[row] = sum;
    }
}

template <typename VT>
cudaError_t launch_vector(int m, const int* rp, const int* col, const VT* val, const VT* x, VT* y,
                          int tpv, cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    const int threads = 256;
    const long long blocks = spmv::grid_for((long long)m * tpv, threads, 16);  // grid-stride beyond 16 blocks per SM
    switch (tpv) {
        case 2: k_csr_vector<VT, 2><<<(int)blocks, threads, 0, st>>>(m, rp, col, val, x, y); break;
        case 4: k_csr_vector<VT, 4><<<(int)blocks, threads, 0, st>>>(m, rp, col, val, x, y); break;
        case 8: k_csr_vector<VT, 8><<<(int)blocks, threads, 0, st>>>(m, rp, col, val, x, y); break;
        case 16: k_csr_vector<VT, 16><<<(int)blocks, threads, 0, st>>>(m, rp, col, val, x, y); break;
        case 32: k_csr_vector<VT, 32><<<(int)blocks, threads, 0, st>>>(m, rp, col, val, x, y); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// ---- cuSPARSE, resolved with dlopen ----
struct CusparseApi {
    decltype(&cusparseCreate) create = nullptr;
    decltype(&cusparseDestroy) destroy = nullptr;
    decltype(&cusparseSetStream) set_stream = nullptr;
    decltype(&cusparseCreateCsr) create_csr = nullptr;
    decltype(&cusparseCreateDnVec) create_dnvec = nullptr;
    decltype(&cusparseDestroySpMat) destroy_spmat = nullptr;
    decltype(&cusparseDestroyDnVec) destroy_dnvec = nullptr;
    decltype(&cusparseSpMV_bufferSize) spmv_buffer_size = nullptr;
    decltype(&cusparseSpMV) spmv = nullptr;
    bool ok = false;
};

const CusparseApi& cusparse_api() {
    static CusparseApi api;
    static std::once_flag once;
    std::call_once(once, [] {
        void* h = dlopen("libcusparse.so.12", RTLD_NOW | RTLD_LOCAL);
        if (h == nullptr) h = dlopen("libcusparse.so", RTLD_NOW | RTLD_LOCAL);
        if (h == nullptr) return;
#define SPMV_SYM(field, name) api.field = reinterpret_cast<decltype(api.field)>(dlsym(h, name))
        SPMV_SYM(create, "cusparseCreate");
        SPMV_SYM(destroy, "cusparseDestroy");
        SPMV_SYM(set_stream, "cusparseSetStream");
        SPMV_SYM(create_csr, "cusparseCreateCsr");
        SPMV_SYM(create_dnvec, "cusparseCreateDnVec");
        SPMV_SYM(destroy_spmat, "cusparseDestroySpMat");
        SPMV_SYM(destroy_dnvec, "cusparseDestroyDnVec");
        SPMV_SYM(spmv_buffer_size, "cusparseSpMV_bufferSize");
        SPMV_SYM(spmv, "cusparseSpMV");
#undef SPMV_SYM
        api.ok = api.create && api.destroy && api.set_stream && api.create_csr &&
                 api.create_dnvec && api.destroy_spmat && api.destroy_dnvec &&
                 api.spmv_buffer_size && api.spmv;
    });
    return api;
}

}  // namespace

struct bhsp_cusparse {
    cusparseHandle_t handle = nullptr;
    cusparseSpMatDescr_t A = nullptr;
    cusparseDnVecDescr_t x = nullptr, y = nullptr;
    cudaDataType type = CUDA_R_64F;
    void* buffer = nullptr;
    double one_d = 1.0, zero_d = 0.0;
    float one_f = 1.0f, zero_f = 0.0f;
};

extern "C" int bhsp_csr_vector_width(int m, int nnz) {
    // spmv_cuda/main.cu:236-286: nnz_per_row = nnz / m (integer division)
    const int per_row = m > 0 ? nnz / m : 0;
    if (per_row <= 2) return 2;
    if (per_row <= 4) return 4;
    if (per_row <= 8) return 8;
    if (per_row <= 16) return 16;
    return 32;
}

extern "C" int bhsp_csr_vector(int value_type, int m, const int* d_row_ptr, const int* d_col_idx,
                               const void* d_val, const void* d_x, void* d_y,
                               int threads_per_vector, void* stream) {
    if (m < 0 || (m > 0 && (!d_row_ptr || !d_y)) ||
        (value_type != BHSP_VALUE_F64 && value_type != BHSP_VALUE_F32))
        return BHSP_CMP_INVALID_ARGUMENT;
    int tpv = threads_per_vector;
    if (tpv == 0) {
        int nnz = 0;
        if (m > 0 && cudaMemcpy(&nnz, d_row_ptr + m, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            return BHSP_CMP_CUDA_ERROR;
        tpv = bhsp_csr_vector_width(m, nnz);
    }
    if (tpv != 2 && tpv != 4 && tpv != 8 && tpv != 16 && tpv != 32) return BHSP_CMP_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (value_type == BHSP_VALUE_F64)
        e = launch_vector(m, d_row_ptr, d_col_idx, static_cast<const double*>(d_val),
                          static_cast<const double*>(d_x), static_cast<double*>(d_y), tpv, st);
    else
        e = launch_vector(m, d_row_ptr, d_col_idx, static_cast<const float*>(d_val),
                          static_cast<const float*>(d_x), static_cast<float*>(d_y), tpv, st);
    return e == cudaSuccess ? BHSP_CMP_OK : BHSP_CMP_CUDA_ERROR;
}

extern "C" int bhsp_cusparse_create(bhsp_cusparse** out, int value_type, int m, int n, int nnz,
                                    const int* d_row_ptr, const int* d_col_idx, const void* d_val,
                                    const void* d_x, void* d_y, void* stream) {
    if (out == nullptr) return BHSP_CMP_INVALID_ARGUMENT;
    *out = nullptr;
    if (m < 0 || n < 0 || nnz < 0 || (value_type != BHSP_VALUE_F64 && value_type != BHSP_VALUE_F32))
        return BHSP_CMP_INVALID_ARGUMENT;
    const CusparseApi& api = cusparse_api();
    if (!api.ok) return BHSP_CMP_UNAVAILABLE;
    bhsp_cusparse* c = new bhsp_cusparse();
    c->type = value_type == BHSP_VALUE_F64 ? CUDA_R_64F : CUDA_R_32F;
    auto fail = [&](int rc) {
        bhsp_cusparse_destroy(c);
        return rc;
    };
    if (api.create(&c->handle) != CUSPARSE_STATUS_SUCCESS) {
        c->handle = nullptr;
        return fail(BHSP_CMP_LIBRARY_ERROR);
    }
    if (api.set_stream(c->handle, static_cast<cudaStream_t>(stream)) != CUSPARSE_STATUS_SUCCESS ||
        api.create_csr(&c->A, m, n, nnz, const_cast<int*>(d_row_ptr), const_cast<int*>(d_col_idx),
                       const_cast<void*>(d_val), CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I,
                       CUSPARSE_INDEX_BASE_ZERO, c->type) != CUSPARSE_STATUS_SUCCESS ||
        api.create_dnvec(&c->x, n, const_cast<void*>(d_x), c->type) != CUSPARSE_STATUS_SUCCESS ||
        api.create_dnvec(&c->y, m, d_y, c->type) != CUSPARSE_STATUS_SUCCESS)
        return fail(BHSP_CMP_LIBRARY_ERROR);
    const void* one = c->type == CUDA_R_64F ? (const void*)&c->one_d : (const void*)&c->one_f;
    const void* zero = c->type == CUDA_R_64F ? (const void*)&c->zero_d : (const void*)&c->zero_f;
    size_t bytes = 0;
    if (api.spmv_buffer_size(c->handle, CUSPARSE_OPERATION_NON_TRANSPOSE, one, c->A, c->x, zero,
                             c->y, c->type, CUSPARSE_SPMV_CSR_ALG1, &bytes) != CUSPARSE_STATUS_SUCCESS)
        return fail(BHSP_CMP_LIBRARY_ERROR);
    if (bytes > 0 && cudaMalloc(&c->buffer, bytes) != cudaSuccess) {
        c->buffer = nullptr;
        return fail(BHSP_CMP_CUDA_ERROR);
    }
    *out = c;
    return BHSP_CMP_OK;
}

extern "C" int bhsp_cusparse_run(bhsp_cusparse* c) {
    if (c == nullptr) return BHSP_CMP_INVALID_ARGUMENT;
    const CusparseApi& api = cusparse_api();
    const void* one = c->type == CUDA_R_64F ? (const void*)&c->one_d : (const void*)&c->one_f;
    const void* zero = c->type == CUDA_R_64F ? (const void*)&c->zero_d : (const void*)&c->zero_f;
    return api.spmv(c->handle, CUSPARSE_OPERATION_NON_TRANSPOSE, one, c->A, c->x, zero, c->y,
                    c->type, CUSPARSE_SPMV_CSR_ALG1, c->buffer) == CUSPARSE_STATUS_SUCCESS
               ? BHSP_CMP_OK
               : BHSP_CMP_LIBRARY_ERROR;
}

extern "C" void bhsp_cusparse_destroy(bhsp_cusparse* c) {
    if (c == nullptr) return;
    const CusparseApi& api = cusparse_api();
    if (api.ok) {
        if (c->A) api.destroy_spmat(c->A);
        if (c->x) api.destroy_dnvec(c->x);
        if (c->y) api.destroy_dnvec(c->y);
        if (c->handle) api.destroy(c->handle);
    }
    if (c->buffer) cudaFree(c->buffer);
    delete c;
}
