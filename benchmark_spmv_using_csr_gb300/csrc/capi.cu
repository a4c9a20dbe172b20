// capi.cu -- the C ABI (include/spmv_gb300.h): handle API mirroring bhsparse_spmv_cuda
// (spmv_cuda/bhsparse_spmv_cuda.h:7-351) and the device-pointer plan API.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/spmv_gb300.h"
#include "internal.h"

using namespace spmv;

namespace {

constexpr int kDefaultSeg = 16;
constexpr int kDefaultTpw = 8;
constexpr int kDefaultWarps = 4;
constexpr int kDefaultStages = 0;

bool valid_vt(int vt) { return vt >= BHSP_VALUE_F64 && vt <= BHSP_VALUE_MIXED_BF16; }
bool supported_vt(int vt) { return is_supported_value_type(vt); }

// bytes of one stored matrix value / one x or y entry on the device
size_t val_bytes(int vt) {
    switch (vt) {
        case BHSP_VALUE_F64: return 8;
        case BHSP_VALUE_F32: return 4;
        case BHSP_VALUE_MIXED_F32: return 4;
        default: return 2;
    }
}
size_t vec_bytes(int vt) { return vt == BHSP_VALUE_F64 ? 8 : 4; }
// bytes of one value as the host passes it through the handle API
size_t host_bytes(int vt) { return vt == BHSP_VALUE_F32 ? 4 : 8; }

bool config_ok(const TileConfig& c, int vt) {
    if (!((c.seg == 8 || c.seg == 16 || c.seg == 32) && c.tiles_per_worker >= 1 &&
          c.tiles_per_worker <= (1 << 20) && (c.warps_per_cta == 4 || c.warps_per_cta == 8) &&
          (c.stages == 0 || c.stages == 2 || c.stages == 3 || c.stages == 4)))
        return false;
    const int smem = tile_config_smem_bytes(vt, c);
    return smem >= 0 && smem <= 227 * 1024;
}

// Default stages: direct loads, except for BF16 storage, whose 16-byte value chunks keep too few
// bytes in flight for direct loads; its TMA-staged ring is 30 % faster on the 27-point stencil
// and 6 % on the power-law matrix.
int default_stages(int vt) { return vt == BHSP_VALUE_MIXED_BF16 ? 2 : kDefaultStages; }

TileConfig make_config(int seg, int tpw, int warps, int stages, int vt) {
    TileConfig c;
    c.seg = seg > 0 ? seg : kDefaultSeg;
    c.tiles_per_worker = tpw > 0 ? tpw : kDefaultTpw;
    c.warps_per_cta = warps > 0 ? warps : kDefaultWarps;
    c.stages = stages >= 0 ? stages : default_stages(vt);
    return c;
}

}  // namespace

namespace spmv {
int tile_config_smem_bytes(int vt, const TileConfig& cfg) {
    switch (vt) {
        case BHSP_VALUE_F64: return plain_smem_bytes(true, cfg);
        case BHSP_VALUE_F32: return plain_smem_bytes(false, cfg);
        case BHSP_VALUE_MIXED_F32: return mixed_smem_bytes(false, cfg);
        default: return mixed_smem_bytes(true, cfg);
    }
}
}  // namespace spmv

namespace {

}  // namespace

// ----------------------------------------------------------------------------------------
// Plan
// ----------------------------------------------------------------------------------------
struct bhsp_plan {
    int vt = 0, m = 0, n = 0, nnz = 0;
    TileConfig cfg{};
    int ntiles = 0, nworkers = 0;
    const int* row_ptr = nullptr;
    const int* col = nullptr;
    uint32_t* tile_ptr = nullptr;
    int* rec_row = nullptr;
    void* rec_val = nullptr;
    uint32_t* err = nullptr;  // device error word
    int* ticket = nullptr;    // [2] the persistent tile kernel's work queue
    int grid_mode = -1;       // the tile kernel's grid: -1 by rule, 0 static, 1 persistent
    int short_rows = 0;     // non-empty rows shorter than one chunk of a lane's slots
    bool one_head = false;  // the tile kernels take the one-head chunk form
    int x_sampled = 0, x_near = 0;  // sampled non-zeros, those with a near column
    bool x_l2 = false;              // the tile kernels gather x from L2 only
    int device = 0;
    std::string last_error;
};

static int plan_fail(bhsp_plan* p, int code, const std::string& msg) {
    if (p) p->last_error = msg;
    return code;
}

static int cuda_fail(std::string* sink, cudaError_t e, const char* what) {
    if (sink) *sink = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? BHSPARSE_OUT_OF_MEMORY : BHSPARSE_CUDA_ERROR;
}

#define PLAN_CUDA(p, call)                                               \
    do {                                                                 \
        cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) return cuda_fail(&(p)->last_error, e_, #call); \
    } while (0)

static void plan_release(bhsp_plan* p) {
    if (!p) return;
    cudaFree(p->tile_ptr);
    cudaFree(p->rec_row);
    cudaFree(p->rec_val);
    cudaFree(p->err);
    cudaFree(p->ticket);
    p->tile_ptr = nullptr;
    p->rec_row = nullptr;
    p->rec_val = nullptr;
    p->err = nullptr;
    p->ticket = nullptr;
}

static int validate_on_device(const int* row_ptr, const int* col, int m, int n, int nnz,
                              cudaStream_t st, std::string* sink) {
    uint32_t* bad = nullptr;
    cudaError_t e = cudaMalloc(&bad, sizeof(uint32_t));
    if (e != cudaSuccess) return cuda_fail(sink, e, "cudaMalloc(validate)");
    uint32_t h = 0;
    e = cudaMemsetAsync(bad, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = launch_validate(row_ptr, col, m, n, nnz, bad, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(bad);
    if (e != cudaSuccess) return cuda_fail(sink, e, "CSR validation");
    if (h) {
        if (sink)
            *sink = (h & 1u) ? "invalid CSR: row_ptr must start at 0, be non-decreasing and end at nnz"
                             : "invalid CSR: a column index lies outside [0, n)";
        return BHSPARSE_INVALID_CSR;
    }
    return BHSPARSE_SUCCESS;
}

static int check_sizes(int m, int n, int nnz, std::string* sink) {
    if (m < 0 || n < 0 || nnz < 0 || nnz > BHSP_MAX_NNZ) {
        if (sink) *sink = "sizes must satisfy m >= 0, n >= 0, 0 <= nnz <= BHSP_MAX_NNZ";
        return BHSPARSE_INVALID_ARGUMENT;
    }
    if (nnz > 0 && n == 0) {
        if (sink) *sink = "nnz > 0 needs n > 0";
        return BHSPARSE_INVALID_ARGUMENT;
    }
    return BHSPARSE_SUCCESS;
}

static int plan_build(bhsp_plan* p, cudaStream_t st) {
    const int tile = 32 * p->cfg.seg;
    p->ntiles = num_tiles(p->nnz, tile);
    p->nworkers = (p->ntiles + p->cfg.tiles_per_worker - 1) / p->cfg.tiles_per_worker;
    PLAN_CUDA(p, cudaGetDevice(&p->device));
    PLAN_CUDA(p, cudaMalloc(&p->tile_ptr, sizeof(uint32_t) * (p->ntiles + 1)));
    PLAN_CUDA(p, cudaMalloc(&p->rec_row, sizeof(int) * (p->nworkers > 0 ? p->nworkers : 1)));
    PLAN_CUDA(p, cudaMalloc(&p->rec_val, 8 * (size_t)(p->nworkers > 0 ? p->nworkers : 1)));
    PLAN_CUDA(p, cudaMalloc(&p->err, sizeof(uint32_t)));
    PLAN_CUDA(p, cudaMemsetAsync(p->err, 0, sizeof(uint32_t), st));
    PLAN_CUDA(p, cudaMalloc(&p->ticket, 2 * sizeof(int)));
    PLAN_CUDA(p, cudaMemsetAsync(p->ticket, 0, 2 * sizeof(int), st));
    PLAN_CUDA(p, launch_partition(p->row_ptr, p->m, p->nnz, tile, p->tile_ptr, st));
    // The kernel variant, from two counts made on the device and read back once:
    //  - the chunk form: rows shorter than the plain / mixed kernels' chunk width (scalar x
    //    entries: 4 slots at S = 8, else 8);
    //  - the x gather path: the locality of the columns on about 2^20 sampled non-zeros.
    const int cw = p->cfg.seg == 8 ? 4 : 8;
    const int step = p->nnz > (1 << 20) ? p->nnz / (1 << 20) : 1;
    uint32_t* counts = nullptr;
    uint32_t h[3] = {0u, 0u, 0u};
    PLAN_CUDA(p, cudaMalloc(&counts, 3 * sizeof(uint32_t)));
    cudaError_t e = launch_short_rows(p->row_ptr, p->m, cw, counts, st);
    if (e == cudaSuccess)
        e = launch_x_locality(p->row_ptr, p->col, p->m, p->nnz, step, counts + 1, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, counts, sizeof h, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(counts);
    if (e != cudaSuccess) return cuda_fail(&p->last_error, e, "plan counts");
    p->short_rows = (int)h[0];
    p->one_head = one_head_pays(h[0], p->nnz, cw);
    p->x_sampled = (int)h[1];
    p->x_near = (int)h[2];
    p->x_l2 = x_l2_pays(h[1], h[2]);
    return BHSPARSE_SUCCESS;
}

static int plan_execute(bhsp_plan* p, const void* val, const void* x, void* y, cudaStream_t st,
                        int phase = 3) {
    if (p->m == 0) return BHSPARSE_SUCCESS;
    cudaError_t e = cudaSuccess;
    switch (p->vt) {
        case BHSP_VALUE_F64:
        case BHSP_VALUE_F32: {
            PlainLaunch a;
            a.row_ptr = p->row_ptr;
            a.col = p->col;
            a.val = val;
            a.x = x;
            a.y = y;
            a.tile_ptr = p->tile_ptr;
            a.rec_row = p->rec_row;
            a.rec_val = p->rec_val;
            a.err = p->err;
            a.m = p->m;
            a.n = p->n;
            a.nnz = p->nnz;
            a.phase = phase;
            a.one_head = p->one_head;
            a.x_l2 = p->x_l2;
            a.ticket = p->ticket;
            a.grid_mode = p->grid_mode;
            e = p->vt == BHSP_VALUE_F64 ? launch_plain_f64(a, p->cfg, st) : launch_plain_f32(a, p->cfg, st);
            break;
        }
        default: {
            MixedLaunch a;
            a.row_ptr = p->row_ptr;
            a.col = p->col;
            a.val = val;
            a.x = static_cast<const float*>(x);
            a.y = static_cast<float*>(y);
            a.tile_ptr = p->tile_ptr;
            a.rec_row = p->rec_row;
            a.rec_val = static_cast<double*>(p->rec_val);
            a.err = p->err;
            a.m = p->m;
            a.n = p->n;
            a.nnz = p->nnz;
            a.bf16 = p->vt == BHSP_VALUE_MIXED_BF16;
            a.phase = phase;
            a.one_head = p->one_head;
            a.x_l2 = p->x_l2;
            a.ticket = p->ticket;
            a.grid_mode = p->grid_mode;
            e = launch_mixed(a, p->cfg, st);
            break;
        }
    }
    if (e != cudaSuccess) return cuda_fail(&p->last_error, e, "SpMV launch");
    return BHSPARSE_SUCCESS;
}

static int plan_check(bhsp_plan* p, cudaStream_t st) {
    uint32_t h = 0;
    PLAN_CUDA(p, cudaMemcpyAsync(&h, p->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    PLAN_CUDA(p, cudaStreamSynchronize(st));
    if (h) {
        PLAN_CUDA(p, cudaMemsetAsync(p->err, 0, sizeof(uint32_t), st));
        PLAN_CUDA(p, cudaStreamSynchronize(st));
        char buf[96];
        snprintf(buf, sizeof buf, "device-side check failed (error word 0x%x)", h);
        return plan_fail(p, BHSPARSE_DEVICE_CHECK_FAILED, buf);
    }
    return BHSPARSE_SUCCESS;
}

namespace spmv {
int plan_create_impl(bhsp_plan** out, int value_type, int m, int n, int nnz, const int* d_row_ptr,
                     const int* d_col_idx, int seg, int tiles_per_worker, int warps_per_cta,
                     int stages, void* stream, bool validate);
}

extern "C" int bhsp_plan_create(bhsp_plan** out, int value_type, int m, int n, int nnz,
                                const int* d_row_ptr, const int* d_col_idx, int seg,
                                int tiles_per_worker, int warps_per_cta, int stages,
                                void* stream) {
    return spmv::plan_create_impl(out, value_type, m, n, nnz, d_row_ptr, d_col_idx, seg,
                                  tiles_per_worker, warps_per_cta, stages, stream, true);
}

int spmv::plan_create_impl(bhsp_plan** out, int value_type, int m, int n, int nnz,
                           const int* d_row_ptr, const int* d_col_idx, int seg,
                           int tiles_per_worker, int warps_per_cta, int stages, void* stream,
                           bool validate) {
    if (!out) return BHSPARSE_INVALID_ARGUMENT;
    *out = nullptr;
    if (!valid_vt(value_type) || !supported_vt(value_type)) return BHSPARSE_UNSUPPORTED_VALUE_TYPE;
    std::string msg;
    int rc = check_sizes(m, n, nnz, &msg);
    if (rc) return rc;
    if (!d_row_ptr || (nnz > 0 && !d_col_idx)) return BHSPARSE_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(d_col_idx) % 32 != 0) return BHSPARSE_INVALID_ARGUMENT;
    TileConfig cfg = make_config(seg, tiles_per_worker, warps_per_cta, stages, value_type);
    if (!config_ok(cfg, value_type)) return BHSPARSE_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (validate) {
        rc = validate_on_device(d_row_ptr, d_col_idx, m, n, nnz, st, &msg);
        if (rc) return rc;
    }
    bhsp_plan* p = new bhsp_plan;
    p->vt = value_type;
    p->m = m;
    p->n = n;
    p->nnz = nnz;
    p->cfg = cfg;
    p->row_ptr = d_row_ptr;
    p->col = d_col_idx;
    rc = plan_build(p, st);
    if (rc) {
        plan_release(p);
        delete p;
        return rc;
    }
    *out = p;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_plan_execute(bhsp_plan* p, const void* d_val, const void* d_x, void* d_y,
                                 void* stream) {
    if (!p) return BHSPARSE_INVALID_ARGUMENT;
    if (p->m > 0 && (!d_y || (p->nnz > 0 && (!d_val || !d_x))))
        return plan_fail(p, BHSPARSE_INVALID_ARGUMENT, "null device buffer");
    if (reinterpret_cast<uintptr_t>(d_val) % 32 != 0)
        return plan_fail(p, BHSPARSE_INVALID_ARGUMENT, "d_val must be 32-byte aligned");
    return plan_execute(p, d_val, d_x, d_y, static_cast<cudaStream_t>(stream));
}

extern "C" int bhsp_plan_execute_phase(bhsp_plan* p, const void* d_val, const void* d_x,
                                       void* d_y, void* stream, int phase) {
    if (!p || phase < 1 || phase > 3) return BHSPARSE_INVALID_ARGUMENT;
    if (p->m > 0 && (!d_y || (p->nnz > 0 && (!d_val || !d_x))))
        return plan_fail(p, BHSPARSE_INVALID_ARGUMENT, "null device buffer");
    if (reinterpret_cast<uintptr_t>(d_val) % 32 != 0)
        return plan_fail(p, BHSPARSE_INVALID_ARGUMENT, "d_val must be 32-byte aligned");
    return plan_execute(p, d_val, d_x, d_y, static_cast<cudaStream_t>(stream), phase);
}

extern "C" int bhsp_plan_check(bhsp_plan* p, void* stream) {
    if (!p) return BHSPARSE_INVALID_ARGUMENT;
    return plan_check(p, static_cast<cudaStream_t>(stream));
}

extern "C" int bhsp_plan_launches(const bhsp_plan* p) {
    if (!p) return 0;
    return p->m == 0 ? 0 : (p->nworkers > 0 ? 2 : 1);
}

extern "C" int bhsp_plan_tiles(const bhsp_plan* p, const uint32_t** d_tile_ptr, int* ntiles,
                               int* tile_nnz) {
    if (!p) return BHSPARSE_INVALID_ARGUMENT;
    if (d_tile_ptr) *d_tile_ptr = p->tile_ptr;
    if (ntiles) *ntiles = p->ntiles;
    if (tile_nnz) *tile_nnz = 32 * p->cfg.seg;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_plan_chunk_form(const bhsp_plan* p, int* short_rows, int* one_head) {
    if (!p) return BHSPARSE_INVALID_ARGUMENT;
    if (short_rows) *short_rows = p->short_rows;
    if (one_head) *one_head = p->one_head ? 1 : 0;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_plan_gather_path(const bhsp_plan* p, int* sampled, int* near, int* l2_only) {
    if (!p) return BHSPARSE_INVALID_ARGUMENT;
    if (sampled) *sampled = p->x_sampled;
    if (near) *near = p->x_near;
    if (l2_only) *l2_only = p->x_l2 ? 1 : 0;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_plan_set_variant(bhsp_plan* p, int one_head, int l2_only) {
    if (!p || one_head < -1 || one_head > 1 || l2_only < -1 || l2_only > 1)
        return BHSPARSE_INVALID_ARGUMENT;
    if (one_head >= 0) p->one_head = one_head == 1;
    if (l2_only >= 0) p->x_l2 = l2_only == 1;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_plan_set_grid(bhsp_plan* p, int persistent) {
    if (!p || persistent < -1 || persistent > 1) return BHSPARSE_INVALID_ARGUMENT;
    p->grid_mode = persistent;
    return BHSPARSE_SUCCESS;
}

extern "C" const char* bhsp_plan_last_error(const bhsp_plan* p) {
    return p ? p->last_error.c_str() : "null plan";
}

extern "C" void bhsp_plan_destroy(bhsp_plan* p) {
    if (!p) return;
    plan_release(p);
    delete p;
}

// ----------------------------------------------------------------------------------------
// Partition primitives
// ----------------------------------------------------------------------------------------
extern "C" int bhsp_partition(const int* d_row_ptr, int m, int nnz, int tile_nnz,
                              uint32_t* d_tile_ptr, void* stream) {
    if (check_sizes(m, 1, nnz, nullptr) || !d_row_ptr || !d_tile_ptr || tile_nnz < 1 ||
        tile_nnz > 4096)
        return BHSPARSE_INVALID_ARGUMENT;
    cudaError_t e = launch_partition(d_row_ptr, m, nnz, tile_nnz, d_tile_ptr,
                                     static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? BHSPARSE_SUCCESS : BHSPARSE_CUDA_ERROR;
}

extern "C" int bhsp_bitflags(const int* d_row_ptr, int m, int nnz, int seg,
                             const uint32_t* d_tile_ptr, uint32_t* d_words, void* stream) {
    if (check_sizes(m, 1, nnz, nullptr) || !d_row_ptr || !d_tile_ptr || (nnz > 0 && !d_words))
        return BHSPARSE_INVALID_ARGUMENT;
    if (seg != 1 && seg != 2 && seg != 4 && seg != 8 && seg != 16 && seg != 32)
        return BHSPARSE_INVALID_ARGUMENT;
    cudaError_t e = launch_bitflags(d_row_ptr, m, nnz, seg, d_tile_ptr, d_words,
                                    static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? BHSPARSE_SUCCESS : BHSPARSE_CUDA_ERROR;
}

extern "C" int bhsp_validate_csr(const int* d_row_ptr, const int* d_col_idx, int m, int n, int nnz,
                                 void* stream) {
    int rc = check_sizes(m, n, nnz, nullptr);
    if (rc) return rc;
    if (!d_row_ptr || (nnz > 0 && !d_col_idx)) return BHSPARSE_INVALID_ARGUMENT;
    return validate_on_device(d_row_ptr, d_col_idx, m, n, nnz, static_cast<cudaStream_t>(stream),
                              nullptr);
}

extern "C" const char* bhsp_version(void) { return "gb300-spmv 1.0 (sm_103a)"; }

// ----------------------------------------------------------------------------------------
// Handle: the reference class bhsparse_spmv_cuda
// ----------------------------------------------------------------------------------------
struct bhsp_spmv {
    int vt = BHSP_VALUE_F64;
    int device = 0;
    bool platform = false;
    bool prepared = false;
    TileConfig cfg = make_config(0, 0, 0, -1, BHSP_VALUE_F64);  // reset for h->vt in bhsp_create
    bool cfg_user = false;        // bhsp_set_config was called: prepare_mem keeps cfg
    bool tuner_default = true;    // bhsp_set_tuner not called (or NULL): the library's network
    std::string tuner_path;       // otherwise this network file ("" = none)
    int sched_source = BHSP_SCHEDULE_DEFAULT;
    float sched_conf = 0.f;
    int m = 0, n = 0, nnz = 0;
    int* d_row_ptr = nullptr;
    int* d_col = nullptr;
    void* d_val = nullptr;   // storage type
    void* d_x = nullptr;     // vector type
    void* d_y = nullptr;     // vector type
    double* d_stage = nullptr;  // FP64 staging for the mixed forms (max(m, n, nnz) entries)
    void* h_y = nullptr;     // caller's y (get_y target)
    bhsp_plan* plan = nullptr;
    cudaStream_t stream = nullptr;  // stream used by run_benchmark / set_x / get_y
    std::string last_error;
    std::string device_name;
    // bhsp_run_stream: two x / y buffer pairs of its own (the handle's d_x / d_y are left as they
    // were), an upload, a compute and a download stream, and per-buffer events; created on first
    // use
    void* d_xs[2] = {nullptr, nullptr};
    void* d_ys[2] = {nullptr, nullptr};
    cudaStream_t s_in = nullptr, s_comp = nullptr, s_out = nullptr;
    cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_comp[2] = {nullptr, nullptr},
                ev_out[2] = {nullptr, nullptr};
};

static int h_fail(bhsp_spmv* h, int code, const std::string& msg) {
    h->last_error = msg;
    return code;
}

#define H_CUDA(h, call)                                                   \
    do {                                                                  \
        cudaError_t e_ = (call);                                          \
        if (e_ != cudaSuccess) return cuda_fail(&(h)->last_error, e_, #call); \
    } while (0)

extern "C" int bhsp_create(bhsp_spmv** out, int value_type) {
    if (!out) return BHSPARSE_INVALID_ARGUMENT;
    *out = nullptr;
    if (!valid_vt(value_type) || !supported_vt(value_type)) return BHSPARSE_UNSUPPORTED_VALUE_TYPE;
    bhsp_spmv* h = new bhsp_spmv;
    h->vt = value_type;
    h->cfg = make_config(0, 0, 0, -1, value_type);
    *out = h;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_set_device(bhsp_spmv* h, int device) {
    if (!h || device < 0) return BHSPARSE_INVALID_ARGUMENT;
    if (h->prepared) return h_fail(h, BHSPARSE_INVALID_ARGUMENT, "set_device after prepare_mem");
    h->device = device;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_init_platform(bhsp_spmv* h) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    H_CUDA(h, cudaSetDevice(h->device));
    cudaDeviceProp prop;
    H_CUDA(h, cudaGetDeviceProperties(&prop, h->device));
    h->device_name = prop.name;
    h->platform = true;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_free_platform(bhsp_spmv* h) { return h ? BHSPARSE_SUCCESS : BHSPARSE_INVALID_ARGUMENT; }

extern "C" int bhsp_set_config(bhsp_spmv* h, int seg, int tiles_per_worker, int warps_per_cta,
                               int stages) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (h->prepared) return h_fail(h, BHSPARSE_INVALID_ARGUMENT, "set_config after prepare_mem");
    TileConfig c = make_config(seg, tiles_per_worker, warps_per_cta, stages, h->vt);
    if (!config_ok(c, h->vt)) return h_fail(h, BHSPARSE_INVALID_ARGUMENT, "unsupported tile config");
    h->cfg = c;
    h->cfg_user = true;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_set_tuner(bhsp_spmv* h, const char* path) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (h->prepared) return h_fail(h, BHSPARSE_INVALID_ARGUMENT, "set_tuner after prepare_mem");
    h->tuner_default = path == nullptr;
    h->tuner_path = path ? path : "";
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_get_schedule_source(const bhsp_spmv* h, int* source, float* confidence) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (source) *source = h->cfg_user ? BHSP_SCHEDULE_CALLER : h->sched_source;
    if (confidence) *confidence = h->cfg_user ? 0.f : h->sched_conf;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_get_config(const bhsp_spmv* h, int* seg, int* tpw, int* warps, int* stages) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (seg) *seg = h->cfg.seg;
    if (tpw) *tpw = h->cfg.tiles_per_worker;
    if (warps) *warps = h->cfg.warps_per_cta;
    if (stages) *stages = h->cfg.stages;
    return BHSPARSE_SUCCESS;
}

static void stream_release(bhsp_spmv* h) {
    for (int i = 0; i < 2; ++i) {
        cudaFree(h->d_xs[i]);
        cudaFree(h->d_ys[i]);
        h->d_xs[i] = h->d_ys[i] = nullptr;
    }
    for (int i = 0; i < 2; ++i) {
        if (h->ev_in[i]) cudaEventDestroy(h->ev_in[i]);
        if (h->ev_comp[i]) cudaEventDestroy(h->ev_comp[i]);
        if (h->ev_out[i]) cudaEventDestroy(h->ev_out[i]);
        h->ev_in[i] = h->ev_comp[i] = h->ev_out[i] = nullptr;
    }
    if (h->s_in) cudaStreamDestroy(h->s_in);
    if (h->s_comp) cudaStreamDestroy(h->s_comp);
    if (h->s_out) cudaStreamDestroy(h->s_out);
    h->s_in = h->s_comp = h->s_out = nullptr;
}

static void handle_release(bhsp_spmv* h) {
    if (h->s_comp) {
        cudaStreamSynchronize(h->s_in);
        cudaStreamSynchronize(h->s_comp);
        cudaStreamSynchronize(h->s_out);
    }
    stream_release(h);
    if (h->plan) bhsp_plan_destroy(h->plan);
    h->plan = nullptr;
    cudaFree(h->d_row_ptr);
    cudaFree(h->d_col);
    cudaFree(h->d_val);
    cudaFree(h->d_x);
    cudaFree(h->d_y);
    cudaFree(h->d_stage);
    h->d_row_ptr = nullptr;
    h->d_col = nullptr;
    h->d_val = nullptr;
    h->d_x = nullptr;
    h->d_y = nullptr;
    h->d_stage = nullptr;
    h->prepared = false;
}

// host -> device copy of a value array, converting for the mixed forms
static int upload_values(bhsp_spmv* h, void* dst, const void* src, size_t count, bool is_matrix) {
    if (count == 0) return BHSPARSE_SUCCESS;
    if (h->vt == BHSP_VALUE_F64 || h->vt == BHSP_VALUE_F32) {
        H_CUDA(h, host_copy(dst, src, count * host_bytes(h->vt), false, h->stream));
        return BHSPARSE_SUCCESS;
    }
    H_CUDA(h, host_copy(h->d_stage, src, count * 8, false, h->stream));
    const bool to_bf16 = is_matrix && h->vt == BHSP_VALUE_MIXED_BF16;
    H_CUDA(h, launch_convert_from_f64(h->d_stage, dst, count, to_bf16, h->stream));
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_prepare_mem(bhsp_spmv* h, int m, int n, int nnz, const int* row_ptr,
                                const int* col_idx, const void* val, const void* x, void* y) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    int rc = check_sizes(m, n, nnz, &h->last_error);
    if (rc) return rc;
    if (!row_ptr || (nnz > 0 && (!col_idx || !val)) || (n > 0 && !x) || (m > 0 && !y))
        return h_fail(h, BHSPARSE_INVALID_ARGUMENT, "null host array");
    if (h->prepared) handle_release(h);
    if (!h->platform) {
        rc = bhsp_init_platform(h);
        if (rc) return rc;
    }
    H_CUDA(h, cudaSetDevice(h->device));
    h->m = m;
    h->n = n;
    h->nnz = nnz;
    h->h_y = y;
    const size_t vb = vec_bytes(h->vt);
    H_CUDA(h, cudaMalloc(&h->d_row_ptr, sizeof(int) * ((size_t)m + 1)));
    H_CUDA(h, cudaMalloc(&h->d_col, sizeof(int) * (size_t)(nnz > 0 ? nnz : 1)));
    H_CUDA(h, cudaMalloc(&h->d_val, val_bytes(h->vt) * (size_t)(nnz > 0 ? nnz : 1) + 32));
    H_CUDA(h, cudaMalloc(&h->d_x, vb * (size_t)(n > 0 ? n : 1)));
    H_CUDA(h, cudaMalloc(&h->d_y, vb * (size_t)(m > 0 ? m : 1)));
    if (h->vt >= BHSP_VALUE_MIXED_F32) {
        size_t big = (size_t)m;
        if ((size_t)n > big) big = n;
        if ((size_t)nnz > big) big = nnz;
        H_CUDA(h, cudaMalloc(&h->d_stage, 8 * (big > 0 ? big : 1)));
    }
    H_CUDA(h, host_copy(h->d_row_ptr, row_ptr, sizeof(int) * ((size_t)m + 1), false, h->stream));
    if (nnz > 0) H_CUDA(h, host_copy(h->d_col, col_idx, sizeof(int) * (size_t)nnz, false, h->stream));
    rc = upload_values(h, h->d_val, val, (size_t)nnz, true);
    if (rc) return rc;
    rc = upload_values(h, h->d_x, x, (size_t)n, false);
    if (rc) return rc;
    rc = validate_on_device(h->d_row_ptr, h->d_col, m, n, nnz, h->stream, &h->last_error);
    if (rc) {
        handle_release(h);
        return rc;
    }
    if (!h->cfg_user) {
        // the schedule: the learned network's pick, or the sweep below its confidence threshold
        // (which runs SpMVs into d_y, so the caller's initial y is uploaded after it)
        int c[4];
        rc = bhsp_choose_schedule(h->vt, m, n, nnz, h->d_row_ptr, h->d_col, h->d_val, h->d_x,
                                  h->d_y, h->tuner_default ? nullptr : h->tuner_path.c_str(),
                                  &c[0], &c[1], &c[2], &c[3], &h->sched_source, &h->sched_conf,
                                  h->stream);
        if (rc) {
            handle_release(h);
            h->last_error = "schedule choice failed (tuner network file missing or malformed?)";
            return rc;
        }
        h->cfg = make_config(c[0], c[1], c[2], c[3], h->vt);
    }
    if (const char* lg = std::getenv("BHSP_LOG_SCHEDULE"); lg && *lg && *lg != '0') {
        static const char* const kSource[] = {"the caller (bhsp_set_config)", "the fixed default",
                                              "the learned network", "the autotune sweep"};
        const int src = h->cfg_user ? BHSP_SCHEDULE_CALLER : h->sched_source;
        std::fprintf(stderr,
                     "bhsp: m=%d nnz=%d schedule (%d, %d, %d, %d) from %s (confidence %.3f)\n", m,
                     nnz, h->cfg.seg, h->cfg.tiles_per_worker, h->cfg.warps_per_cta, h->cfg.stages,
                     kSource[src & 3], (double)(h->cfg_user ? 0.f : h->sched_conf));
    }
    rc = upload_values(h, h->d_y, y, (size_t)m, false);
    if (rc) return rc;
    bhsp_plan* p = nullptr;
    rc = spmv::plan_create_impl(&p, h->vt, m, n, nnz, h->d_row_ptr, h->d_col, h->cfg.seg,
                                h->cfg.tiles_per_worker, h->cfg.warps_per_cta, h->cfg.stages,
                                h->stream, false);
    if (rc) {
        handle_release(h);
        h->last_error = "plan creation failed";
        return rc;
    }
    h->plan = p;
    H_CUDA(h, cudaStreamSynchronize(h->stream));
    h->prepared = true;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_set_x(bhsp_spmv* h, const void* x) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (!h->prepared) return h_fail(h, BHSPARSE_NOT_PREPARED, "set_x before prepare_mem");
    if (h->n > 0 && !x) return h_fail(h, BHSPARSE_INVALID_ARGUMENT, "null x");
    const int rc = upload_values(h, h->d_x, x, (size_t)h->n, false);
    if (rc) return rc;
    // the caller may reuse its buffer as soon as this returns
    H_CUDA(h, cudaStreamSynchronize(h->stream));
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_run_async(bhsp_spmv* h, void* stream) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (!h->prepared) return h_fail(h, BHSPARSE_NOT_PREPARED, "run before prepare_mem");
    int rc = bhsp_plan_execute(h->plan, h->d_val, h->d_x, h->d_y, stream);
    if (rc) h->last_error = h->plan->last_error;
    return rc;
}

extern "C" int bhsp_run_phase(bhsp_spmv* h, void* stream, int phase) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (!h->prepared) return h_fail(h, BHSPARSE_NOT_PREPARED, "run before prepare_mem");
    int rc = bhsp_plan_execute_phase(h->plan, h->d_val, h->d_x, h->d_y, stream, phase);
    if (rc) h->last_error = h->plan->last_error;
    return rc;
}

extern "C" int bhsp_check(bhsp_spmv* h) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (!h->prepared) return h_fail(h, BHSPARSE_NOT_PREPARED, "check before prepare_mem");
    int rc = plan_check(h->plan, h->stream);
    if (rc) h->last_error = h->plan->last_error;
    return rc;
}

extern "C" int bhsp_run_benchmark(bhsp_spmv* h) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    int rc = bhsp_run_async(h, h->stream);
    if (rc) return rc;
    return bhsp_check(h);
}

extern "C" int bhsp_get_y(bhsp_spmv* h) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (!h->prepared) return h_fail(h, BHSPARSE_NOT_PREPARED, "get_y before prepare_mem");
    if (h->m == 0) return BHSPARSE_SUCCESS;
    if (h->vt == BHSP_VALUE_F64 || h->vt == BHSP_VALUE_F32) {
        H_CUDA(h, host_copy(h->h_y, h->d_y, (size_t)h->m * vec_bytes(h->vt), true, h->stream));
    } else {
        H_CUDA(h, launch_convert_to_f64(static_cast<const float*>(h->d_y), h->d_stage, (size_t)h->m,
                                        h->stream));
        H_CUDA(h, host_copy(h->h_y, h->d_stage, (size_t)h->m * 8, true, h->stream));
    }
    H_CUDA(h, cudaStreamSynchronize(h->stream));
    return BHSPARSE_SUCCESS;
}

// Buffers, streams and events of bhsp_run_stream, created once per prepared matrix.
static int stream_setup(bhsp_spmv* h) {
    if (h->s_comp) return BHSPARSE_SUCCESS;
    const size_t vb = vec_bytes(h->vt);
    for (int i = 0; i < 2; ++i) {
        H_CUDA(h, cudaMalloc(&h->d_xs[i], vb * (size_t)(h->n > 0 ? h->n : 1)));
        H_CUDA(h, cudaMalloc(&h->d_ys[i], vb * (size_t)(h->m > 0 ? h->m : 1)));
    }
    H_CUDA(h, cudaStreamCreateWithFlags(&h->s_in, cudaStreamNonBlocking));
    H_CUDA(h, cudaStreamCreateWithFlags(&h->s_comp, cudaStreamNonBlocking));
    H_CUDA(h, cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
        H_CUDA(h, cudaEventCreateWithFlags(&h->ev_in[i], cudaEventDisableTiming));
        H_CUDA(h, cudaEventCreateWithFlags(&h->ev_comp[i], cudaEventDisableTiming));
        H_CUDA(h, cudaEventCreateWithFlags(&h->ev_out[i], cudaEventDisableTiming));
    }
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_run_stream(bhsp_spmv* h, int count, const void* const* x_host,
                               void* const* y_host) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (!h->prepared) return h_fail(h, BHSPARSE_NOT_PREPARED, "run_stream before prepare_mem");
    if (h->vt != BHSP_VALUE_F64 && h->vt != BHSP_VALUE_F32)
        return h_fail(h, BHSPARSE_INVALID_ARGUMENT, "run_stream supports the F64 and F32 forms");
    if (count < 0 || (count > 0 && (!x_host || !y_host)))
        return h_fail(h, BHSPARSE_INVALID_ARGUMENT, "bad count or null vector list");
    for (int i = 0; i < count; ++i)
        if ((h->n > 0 && !x_host[i]) || (h->m > 0 && !y_host[i]))
            return h_fail(h, BHSPARSE_INVALID_ARGUMENT, "null host vector");
    H_CUDA(h, cudaSetDevice(h->device));
    int rc = stream_setup(h);
    if (rc) {
        stream_release(h);  // a partial set-up is not kept
        return rc;
    }
    H_CUDA(h, cudaStreamSynchronize(h->stream));  // the handle's own work comes first
    // every failure below waits for all three streams, so that no copy or kernel of this call
    // is still running when it returns
    auto drain = [&](int code) {
        cudaStreamSynchronize(h->s_in);
        cudaStreamSynchronize(h->s_comp);
        cudaStreamSynchronize(h->s_out);
        return code;
    };
#define S_CUDA(call)                                                                      \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) return drain(cuda_fail(&h->last_error, e_, #call));        \
    } while (0)
    const size_t vb = vec_bytes(h->vt);
    void* const* X = h->d_xs;
    void* const* Y = h->d_ys;
    for (int i = 0; i < count; ++i) {
        const int b = i & 1;
        // x_i into X[b] once the SpMV of i-2 has read it
        if (i >= 2) S_CUDA(cudaStreamWaitEvent(h->s_in, h->ev_comp[b], 0));
        if (h->n > 0)
            S_CUDA(cudaMemcpyAsync(X[b], x_host[i], vb * (size_t)h->n, cudaMemcpyHostToDevice,
                                   h->s_in));
        S_CUDA(cudaEventRecord(h->ev_in[b], h->s_in));
        // y_i = A x_i once x_i has landed and y_{i-2} has left Y[b]
        S_CUDA(cudaStreamWaitEvent(h->s_comp, h->ev_in[b], 0));
        if (i >= 2) S_CUDA(cudaStreamWaitEvent(h->s_comp, h->ev_out[b], 0));
        rc = bhsp_plan_execute(h->plan, h->d_val, X[b], Y[b], h->s_comp);
        if (rc) {
            h->last_error = h->plan->last_error;
            return drain(rc);
        }
        S_CUDA(cudaEventRecord(h->ev_comp[b], h->s_comp));
        // y_i to the host
        S_CUDA(cudaStreamWaitEvent(h->s_out, h->ev_comp[b], 0));
        if (h->m > 0)
            S_CUDA(cudaMemcpyAsync(y_host[i], Y[b], vb * (size_t)h->m, cudaMemcpyDeviceToHost,
                                   h->s_out));
        S_CUDA(cudaEventRecord(h->ev_out[b], h->s_out));
    }
#undef S_CUDA
    cudaError_t e = cudaStreamSynchronize(h->s_in);
    const cudaError_t e2 = cudaStreamSynchronize(h->s_comp);
    const cudaError_t e3 = cudaStreamSynchronize(h->s_out);
    if (e == cudaSuccess) e = e2 != cudaSuccess ? e2 : e3;
    if (e != cudaSuccess) return cuda_fail(&h->last_error, e, "bhsp_run_stream");
    rc = plan_check(h->plan, h->s_comp);
    if (rc) h->last_error = h->plan->last_error;
    return rc;
}

extern "C" int bhsp_free_mem(bhsp_spmv* h) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (h->prepared) H_CUDA(h, cudaStreamSynchronize(h->stream));
    handle_release(h);
    return BHSPARSE_SUCCESS;
}

extern "C" void bhsp_destroy(bhsp_spmv* h) {
    if (!h) return;
    if (h->prepared) cudaStreamSynchronize(h->stream);
    handle_release(h);
    delete h;
}

extern "C" const char* bhsp_last_error(const bhsp_spmv* h) {
    return h ? h->last_error.c_str() : "null handle";
}

extern "C" int bhsp_device_buffers(const bhsp_spmv* h, const int** row_ptr, const int** col_idx,
                                   const void** val, void** x, void** y) {
    if (!h) return BHSPARSE_INVALID_ARGUMENT;
    if (!h->prepared) return BHSPARSE_NOT_PREPARED;
    if (row_ptr) *row_ptr = h->d_row_ptr;
    if (col_idx) *col_idx = h->d_col;
    if (val) *val = h->d_val;
    if (x) *x = h->d_x;
    if (y) *y = h->d_y;
    return BHSPARSE_SUCCESS;
}

extern "C" size_t bhsp_device_bytes(const bhsp_spmv* h) {
    if (!h || !h->prepared) return 0;
    size_t b = sizeof(int) * ((size_t)h->m + 1) + sizeof(int) * (size_t)h->nnz +
               val_bytes(h->vt) * (size_t)h->nnz + vec_bytes(h->vt) * ((size_t)h->n + h->m);
    if (h->plan) b += sizeof(uint32_t) * ((size_t)h->plan->ntiles + 1) + 12 * (size_t)h->plan->nworkers;
    if (h->d_xs[0]) b += 2 * vec_bytes(h->vt) * ((size_t)h->n + h->m);  // bhsp_run_stream's pairs
    return b;
}
