// learned.cu -- the schedule a matrix runs with when its caller does not set one: the learned
// network's pick (16 row-length features -> MLP forward on the device), or the autotune sweep
// when the network is less confident than its calibrated threshold.
//
// The network file (written by the package's trainer, LearnedTuner.save) is little-endian:
//   char magic[8] = "BHSPTUN1"
//   int32 value_type, n_in, n_hidden, n_out
//   float32 threshold
//   float32 mean[n_in], std[n_in]           input standardisation
//   int32 candidates[n_out][4]              (seg, tiles_per_worker, warps_per_cta, stages) of
//                                           each output
//   int32 n_params; float32 params[n_params] W1 b1 W2 b2 W3 b3 (bhsp_mlp layout)
// optionally followed by the risk network, which decides the fallback:
//   char magic[8] = "BHSPRSK1"
//   int32 r_in (19), r_hidden, r_out (2)
//   float32 r_threshold                     the sweep runs where P(slow pick) > r_threshold
//   float32 r_mean[r_in], r_std[r_in]
//   int32 r_n_params; float32 r_params[r_n_params]
// Its inputs are the 16 features and the schedule network's largest and second-largest
// probability and the entropy of its distribution; output 1 is the probability that the pick is
// slow (below 95 % of the best time).  Without it, the sweep runs where the schedule network's
// probability of its pick is below `threshold`.
// The reference has no counterpart: its tile geometry is fixed at compile time
// (spmv_cuda/common.h:39-48, spmv_cuda/bhsparse_spmv_cuda.h:323-328).
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/spmv_gb300.h"
#include "internal.h"

namespace {

struct NetParams {
    int n_in = 0, hidden = 0, n_out = 0;
    std::vector<float> mean, stdv, params;
};

struct TunerFile {
    int vt = 0;
    float threshold = 0.f;
    NetParams net;
    std::vector<int> cands;  // n_out x 4
    bool has_risk = false;
    float risk_threshold = 1.f;
    NetParams risk;
};

size_t num_params(const NetParams& n) {
    return (size_t)n.hidden * n.n_in + n.hidden + (size_t)n.hidden * n.hidden + n.hidden +
           (size_t)n.n_out * n.hidden + n.n_out;
}

const char* vt_name(int vt) {
    switch (vt) {
        case BHSP_VALUE_F64: return "f64";
        case BHSP_VALUE_F32: return "f32";
        case BHSP_VALUE_MIXED_F32: return "mixed_f32";
        default: return "mixed_bf16";
    }
}

// <directory of this library>/tuner_data/gb300_<value type>_tuner.bin, or the same file name in
// $BHSP_TUNER_DIR when that is set
std::string default_path(int vt) {
    std::string dir;
    const char* env = std::getenv("BHSP_TUNER_DIR");
    if (env && *env) {
        dir = env;
    } else {
        Dl_info info;
        if (dladdr(reinterpret_cast<void*>(&bhsp_choose_schedule), &info) == 0 || !info.dli_fname)
            return std::string();
        dir = info.dli_fname;
        const size_t slash = dir.rfind('/');
        dir = slash == std::string::npos ? std::string(".") : dir.substr(0, slash);
        dir += "/tuner_data";
    }
    return dir + "/gb300_" + vt_name(vt) + "_tuner.bin";
}

template <typename T>
bool rd(FILE* f, T* v, size_t count) {
    return count == 0 || std::fread(v, sizeof(T), count, f) == count;
}

bool read_net_body(FILE* f, NetParams* n) {
    n->mean.resize(n->n_in);
    n->stdv.resize(n->n_in);
    return rd(f, n->mean.data(), n->mean.size()) && rd(f, n->stdv.data(), n->stdv.size());
}

bool read_params(FILE* f, NetParams* n) {
    int32_t np = 0;
    if (!rd(f, &np, 1) || np < 0 || (size_t)np != num_params(*n)) return false;
    n->params.resize((size_t)np);
    return rd(f, n->params.data(), n->params.size());
}

// 0 = loaded, 1 = no such file, -1 = malformed
int load(const std::string& path, TunerFile* t, std::string* err) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return 1;
    char magic[8];
    int32_t hdr[4];
    bool ok = rd(f, magic, 8) && std::memcmp(magic, "BHSPTUN1", 8) == 0 && rd(f, hdr, 4) &&
              rd(f, &t->threshold, 1);
    if (ok) {
        t->vt = hdr[0];
        t->net.n_in = hdr[1];
        t->net.hidden = hdr[2];
        t->net.n_out = hdr[3];
        ok = t->net.n_in == 16 && t->net.hidden > 0 && t->net.hidden <= 4096 &&
             t->net.n_out > 1 && t->net.n_out <= 4096;
    }
    if (ok) {
        t->cands.resize((size_t)t->net.n_out * 4);
        ok = read_net_body(f, &t->net) && rd(f, t->cands.data(), t->cands.size()) &&
             read_params(f, &t->net);
    }
    if (ok) {  // the optional risk network
        char m2[8];
        const size_t got = std::fread(m2, 1, 8, f);
        if (got == 8 && std::memcmp(m2, "BHSPRSK1", 8) == 0) {
            int32_t rh[3];
            ok = rd(f, rh, 3) && rd(f, &t->risk_threshold, 1);
            if (ok) {
                t->risk.n_in = rh[0];
                t->risk.hidden = rh[1];
                t->risk.n_out = rh[2];
                ok = t->risk.n_in == 19 && t->risk.hidden > 0 && t->risk.hidden <= 4096 &&
                     t->risk.n_out == 2;
            }
            ok = ok && read_net_body(f, &t->risk) && read_params(f, &t->risk);
            t->has_risk = ok;
        } else {
            ok = got == 0;  // nothing but the end of the file may follow the parameters
        }
    }
    if (ok) {
        char extra;
        ok = std::fread(&extra, 1, 1, f) == 0;
    }
    std::fclose(f);
    if (!ok && err) *err = "malformed tuner network file: " + path;
    return ok ? 0 : -1;
}

// One forward pass of a network on one input vector with the library's MLP kernels.
int forward_once(const NetParams& n, const float* input, float* out, cudaStream_t st) {
    bhsp_mlp* net = nullptr;
    int rc = bhsp_mlp_create(&net, n.n_in, n.hidden, n.n_out, 1);
    if (rc) return rc;
    float* d_in = nullptr;
    float* d_out = nullptr;
    rc = bhsp_mlp_set_params(net, n.params.data(), n.params.size());
    if (!rc) rc = bhsp_mlp_set_normalization(net, n.mean.data(), n.stdv.data());
    if (!rc && (cudaMalloc(&d_in, sizeof(float) * (size_t)n.n_in) != cudaSuccess ||
                cudaMalloc(&d_out, sizeof(float) * (size_t)n.n_out) != cudaSuccess))
        rc = BHSPARSE_OUT_OF_MEMORY;
    if (!rc && cudaMemcpyAsync(d_in, input, sizeof(float) * (size_t)n.n_in,
                               cudaMemcpyHostToDevice, st) != cudaSuccess)
        rc = BHSPARSE_CUDA_ERROR;
    if (!rc) rc = bhsp_mlp_forward(net, d_in, 1, d_out, st);
    if (!rc && (cudaMemcpyAsync(out, d_out, sizeof(float) * (size_t)n.n_out,
                                cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = BHSPARSE_CUDA_ERROR;
    cudaFree(d_in);
    cudaFree(d_out);
    bhsp_mlp_destroy(net);
    return rc;
}

int fixed_default(int vt, int* seg, int* tpw, int* warps, int* stages) {
    // the handle's defaults (bhsp_set_config with zeros / -1)
    *seg = 16;
    *tpw = 8;
    *warps = 4;
    *stages = vt == BHSP_VALUE_MIXED_BF16 ? 2 : 0;
    return BHSPARSE_SUCCESS;
}

}  // namespace

extern "C" int bhsp_choose_schedule(int value_type, int m, int n, int nnz, const int* d_row_ptr,
                                    const int* d_col_idx, const void* d_val, const void* d_x,
                                    void* d_y, const char* tuner_path, int* seg,
                                    int* tiles_per_worker, int* warps_per_cta, int* stages,
                                    int* source, float* confidence, void* stream) {
    if (!seg || !tiles_per_worker || !warps_per_cta || !stages) return BHSPARSE_INVALID_ARGUMENT;
    if (value_type < BHSP_VALUE_F64 || value_type > BHSP_VALUE_MIXED_BF16)
        return BHSPARSE_UNSUPPORTED_VALUE_TYPE;
    if (m < 0 || n < 0 || nnz < 0 || !d_row_ptr) return BHSPARSE_INVALID_ARGUMENT;
    if (source) *source = BHSP_SCHEDULE_DEFAULT;
    if (confidence) *confidence = 0.f;
    const bool explicit_path = tuner_path && *tuner_path;
    if (tuner_path && !*tuner_path)  // "" : no network
        return fixed_default(value_type, seg, tiles_per_worker, warps_per_cta, stages);
    const std::string path = explicit_path ? std::string(tuner_path) : default_path(value_type);
    TunerFile t;
    const int lr = path.empty() ? 1 : load(path, &t, nullptr);
    if (lr != 0) {
        // an explicitly named file must exist and parse; a missing default means no network
        if (explicit_path) return BHSPARSE_INVALID_ARGUMENT;
        if (lr < 0) return BHSPARSE_INVALID_ARGUMENT;
        return fixed_default(value_type, seg, tiles_per_worker, warps_per_cta, stages);
    }
    if (t.vt != value_type) return BHSPARSE_INVALID_ARGUMENT;  // trained on another form's timings

    // features on the device, then the network's forward pass (the library's MLP kernels)
    float feat[16];
    int rc = bhsp_row_features(d_row_ptr, m, n, feat, stream);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    std::vector<float> prob((size_t)t.net.n_out, 0.f);
    rc = forward_once(t.net, feat, prob.data(), st);
    if (rc) return rc;
    int pick = 0;
    for (int k = 1; k < t.net.n_out; ++k)
        if (prob[(size_t)k] > prob[(size_t)pick]) pick = k;
    const float conf = prob[(size_t)pick];
    if (confidence) *confidence = conf;
    bool slow = conf < t.threshold;
    if (t.has_risk) {  // the risk network: features, top two probabilities, entropy
        float rin[19];
        std::memcpy(rin, feat, sizeof feat);
        float second = 0.f;
        double ent = 0.0;
        for (int k = 0; k < t.net.n_out; ++k) {
            const float pk = prob[(size_t)k];
            if (k != pick && pk > second) second = pk;
            ent -= (double)pk * std::log(std::max((double)pk, 1e-30));
        }
        rin[16] = conf;
        rin[17] = second;
        rin[18] = (float)ent;
        float rout[2] = {0.f, 0.f};
        rc = forward_once(t.risk, rin, rout, st);
        if (rc) return rc;
        slow = slow || rout[1] > t.risk_threshold;
    }
    const int* c = &t.cands[(size_t)pick * 4];
    const spmv::TileConfig pc{c[0], c[1], c[2], c[3]};
    const int smem = spmv::tile_config_smem_bytes(value_type, pc);
    const bool runnable = (c[0] == 8 || c[0] == 16 || c[0] == 32) && c[1] >= 1 &&
                          (c[2] == 4 || c[2] == 8) && smem >= 0 && smem <= 227 * 1024;
    if (runnable && !slow) {
        *seg = t.cands[(size_t)pick * 4 + 0];
        *tiles_per_worker = t.cands[(size_t)pick * 4 + 1];
        *warps_per_cta = t.cands[(size_t)pick * 4 + 2];
        *stages = t.cands[(size_t)pick * 4 + 3];
        if (source) *source = BHSP_SCHEDULE_LEARNED;
        return BHSPARSE_SUCCESS;
    }
    // a likely slow pick: the full sweep decides (it needs the matrix values and x / y)
    if (nnz > 0 && (!d_col_idx || !d_val || !d_x)) return BHSPARSE_INVALID_ARGUMENT;
    if (m > 0 && !d_y) return BHSPARSE_INVALID_ARGUMENT;
    const int K = bhsp_tune_num_candidates();
    std::vector<float> ms((size_t)K, 0.f);
    int best = -1;
    rc = bhsp_autotune(value_type, m, n, nnz, d_row_ptr, d_col_idx, d_val, d_x, d_y, 1, 3,
                       ms.data(), &best, stream);
    if (rc) return rc;
    if (best < 0) return fixed_default(value_type, seg, tiles_per_worker, warps_per_cta, stages);
    rc = bhsp_tune_candidate(best, seg, tiles_per_worker, warps_per_cta, stages);
    if (rc) return rc;
    if (source) *source = BHSP_SCHEDULE_SWEEP;
    return BHSPARSE_SUCCESS;
}
