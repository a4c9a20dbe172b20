// mlp.cu -- the learned schedule tuner's network: 16 -> H -> H -> K, ReLU, softmax, trained with
// soft cross-entropy and Adam.  Hand-written CUDA forward, backward and update kernels (FP32).
// It maps a matrix's 16 row-length features to a probability over the autotuner's candidate
// schedules; it only chooses a schedule and never touches the SpMV arithmetic.
//
// Parameters live in one flat device buffer: W1[H][I] b1[H] W2[H][H] b2[H] W3[K][H] b3[K].
// Inputs are standardised on the device with a stored mean / std.  Every reduction runs in a
// fixed order (one thread per output element, sequential loop over the summed index), so
// gradients and updates are deterministic.
#include <cmath>
#include <cstdio>
#include <string>

#include "../../include/spmv_gb300.h"

namespace {

__global__ void k_normalize(const float* __restrict__ f, const float* __restrict__ mean,
                            const float* __restrict__ stdv, int B, int I, float* __restrict__ xn) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B * I) return;
    const int i = idx % I;
    xn[idx] = (f[idx] - mean[i]) / stdv[i];
}

// Z[b][o] = W[o] . X[b] + bias[o]; A = relu(Z) when A != nullptr
__global__ void k_dense(const float* __restrict__ X, int B, int I, const float* __restrict__ W,
                        const float* __restrict__ bias, int O, float* __restrict__ Z,
                        float* __restrict__ A) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B * O) return;
    const int b = idx / O, o = idx % O;
    const float* x = X + (size_t)b * I;
    const float* w = W + (size_t)o * I;
    float s = bias[o];
    for (int i = 0; i < I; ++i) s = fmaf(w[i], x[i], s);
    Z[idx] = s;
    if (A) A[idx] = s > 0.f ? s : 0.f;
}

// softmax of each row of Z into P; with targets T: dZ = (P - T) / B and the mean soft
// cross-entropy -sum(T log P) / B accumulated into *loss
__global__ void k_softmax_xent(const float* __restrict__ Z, const float* __restrict__ T, int B,
                               int O, float* __restrict__ P, float* __restrict__ dZ,
                               float* __restrict__ loss) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float* z = Z + (size_t)b * O;
    float mx = z[0];
    for (int o = 1; o < O; ++o) mx = fmaxf(mx, z[o]);
    float den = 0.f;
    for (int o = 0; o < O; ++o) den += expf(z[o] - mx);
    const float lden = logf(den);
    float l = 0.f;
    for (int o = 0; o < O; ++o) {
        const float lp = z[o] - mx - lden;
        const float p = expf(lp);
        P[(size_t)b * O + o] = p;
        if (T) {
            const float t = T[(size_t)b * O + o];
            dZ[(size_t)b * O + o] = (p - t) / (float)B;
            if (t > 0.f) l -= t * lp;
        }
    }
    if (T && loss) atomicAdd(loss, l / (float)B);
}

// dX[b][i] = sum_o dZ[b][o] W[o][i], masked by relu'(Zprev[b][i]) when Zprev != nullptr
__global__ void k_back_input(const float* __restrict__ dZ, int B, int O, const float* __restrict__ W,
                             int I, const float* __restrict__ Zprev, float* __restrict__ dX) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B * I) return;
    const int b = idx / I, i = idx % I;
    float s = 0.f;
    for (int o = 0; o < O; ++o) s = fmaf(dZ[(size_t)b * O + o], W[(size_t)o * I + i], s);
    if (Zprev && !(Zprev[idx] > 0.f)) s = 0.f;
    dX[idx] = s;
}

// dW[o][i] = sum_b dZ[b][o] A[b][i], dbias[o] = sum_b dZ[b][o]  (thread per (o, i), i == I: bias)
__global__ void k_grad_w(const float* __restrict__ dZ, const float* __restrict__ A, int B, int O,
                         int I, float* __restrict__ dW, float* __restrict__ db) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= O * (I + 1)) return;
    const int o = idx / (I + 1), i = idx % (I + 1);
    float s = 0.f;
    if (i < I) {
        for (int b = 0; b < B; ++b) s = fmaf(dZ[(size_t)b * O + o], A[(size_t)b * I + i], s);
        dW[(size_t)o * I + i] = s;
    } else {
        for (int b = 0; b < B; ++b) s += dZ[(size_t)b * O + o];
        db[o] = s;
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float beta1, float beta2, float eps,
                       float bc1, float bc2, float wd) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] + wd * p[i];
    const float mi = beta1 * m[i] + (1.f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// grid size for n threads in blocks of 256 (every launch below uses 256-thread blocks)
int blocks_for(long long n) { return (int)((n + 255) / 256); }

}  // namespace

struct bhsp_mlp {
    int I = 16, H = 64, O = 18, max_batch = 0;
    size_t nparams = 0;
    float* params = nullptr;  // W1 b1 W2 b2 W3 b3
    float* grads = nullptr;
    float* m1 = nullptr;      // Adam moments
    float* m2 = nullptr;
    float* mean = nullptr;
    float* stdv = nullptr;
    // activations [max_batch][*]
    float *xn = nullptr, *z1 = nullptr, *a1 = nullptr, *z2 = nullptr, *a2 = nullptr, *z3 = nullptr;
    float *p = nullptr, *dz3 = nullptr, *dz2 = nullptr, *dz1 = nullptr, *loss = nullptr;
    long long step = 0;
    std::string last_error;
    float* W1() { return params; }
    float* b1() { return params + H * I; }
    float* W2() { return b1() + H; }
    float* b2() { return W2() + H * H; }
    float* W3() { return b2() + H; }
    float* b3() { return W3() + O * H; }
};

static void mlp_free(bhsp_mlp* m) {
    float* ptrs[] = {m->params, m->grads, m->m1, m->m2, m->mean, m->stdv, m->xn, m->z1, m->a1,
                     m->z2, m->a2, m->z3, m->p, m->dz3, m->dz2, m->dz1, m->loss};
    for (float* q : ptrs) cudaFree(q);
}

extern "C" int bhsp_mlp_create(bhsp_mlp** out, int n_in, int n_hidden, int n_out, int max_batch) {
    if (!out || n_in < 1 || n_hidden < 1 || n_out < 2 || max_batch < 1 || n_in > 4096 ||
        n_hidden > 4096 || n_out > 4096 || max_batch > (1 << 20))
        return BHSPARSE_INVALID_ARGUMENT;
    *out = nullptr;
    bhsp_mlp* m = new bhsp_mlp;
    m->I = n_in;
    m->H = n_hidden;
    m->O = n_out;
    m->max_batch = max_batch;
    m->nparams = (size_t)n_hidden * n_in + n_hidden + (size_t)n_hidden * n_hidden + n_hidden +
                 (size_t)n_out * n_hidden + n_out;
    const size_t B = (size_t)max_batch;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](float** p, size_t n) {
        if (e == cudaSuccess) e = cudaMalloc(p, sizeof(float) * (n > 0 ? n : 1));
        if (e == cudaSuccess) e = cudaMemset(*p, 0, sizeof(float) * (n > 0 ? n : 1));
    };
    alloc(&m->params, m->nparams);
    alloc(&m->grads, m->nparams);
    alloc(&m->m1, m->nparams);
    alloc(&m->m2, m->nparams);
    alloc(&m->mean, n_in);
    alloc(&m->stdv, n_in);
    alloc(&m->xn, B * n_in);
    alloc(&m->z1, B * n_hidden);
    alloc(&m->a1, B * n_hidden);
    alloc(&m->z2, B * n_hidden);
    alloc(&m->a2, B * n_hidden);
    alloc(&m->z3, B * n_out);
    alloc(&m->p, B * n_out);
    alloc(&m->dz3, B * n_out);
    alloc(&m->dz2, B * n_hidden);
    alloc(&m->dz1, B * n_hidden);
    alloc(&m->loss, 1);
    if (e != cudaSuccess) {
        mlp_free(m);
        delete m;
        return e == cudaErrorMemoryAllocation ? BHSPARSE_OUT_OF_MEMORY : BHSPARSE_CUDA_ERROR;
    }
    // identity normalisation until set
    float* ones = new float[n_in];
    for (int i = 0; i < n_in; ++i) ones[i] = 1.f;
    e = cudaMemcpy(m->stdv, ones, sizeof(float) * n_in, cudaMemcpyHostToDevice);
    delete[] ones;
    if (e != cudaSuccess) {
        mlp_free(m);
        delete m;
        return BHSPARSE_CUDA_ERROR;
    }
    *out = m;
    return BHSPARSE_SUCCESS;
}

extern "C" size_t bhsp_mlp_num_params(const bhsp_mlp* m) { return m ? m->nparams : 0; }

extern "C" int bhsp_mlp_set_params(bhsp_mlp* m, const float* host, size_t count) {
    if (!m || !host || count != m->nparams) return BHSPARSE_INVALID_ARGUMENT;
    if (cudaMemcpy(m->params, host, sizeof(float) * count, cudaMemcpyHostToDevice) != cudaSuccess)
        return BHSPARSE_CUDA_ERROR;
    cudaMemset(m->m1, 0, sizeof(float) * m->nparams);
    cudaMemset(m->m2, 0, sizeof(float) * m->nparams);
    m->step = 0;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_mlp_get_params(const bhsp_mlp* m, float* host, size_t count) {
    if (!m || !host || count != m->nparams) return BHSPARSE_INVALID_ARGUMENT;
    return cudaMemcpy(host, m->params, sizeof(float) * count, cudaMemcpyDeviceToHost) == cudaSuccess
               ? BHSPARSE_SUCCESS
               : BHSPARSE_CUDA_ERROR;
}

extern "C" int bhsp_mlp_set_normalization(bhsp_mlp* m, const float* mean, const float* stdv) {
    if (!m || !mean || !stdv) return BHSPARSE_INVALID_ARGUMENT;
    for (int i = 0; i < m->I; ++i)
        if (!(stdv[i] > 0.f)) return BHSPARSE_INVALID_ARGUMENT;
    if (cudaMemcpy(m->mean, mean, sizeof(float) * m->I, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m->stdv, stdv, sizeof(float) * m->I, cudaMemcpyHostToDevice) != cudaSuccess)
        return BHSPARSE_CUDA_ERROR;
    return BHSPARSE_SUCCESS;
}

// forward pass on d_features[B][I] (device); probabilities into the internal buffer
static cudaError_t mlp_forward(bhsp_mlp* m, const float* d_features, int B, cudaStream_t st) {
    const int I = m->I, H = m->H, O = m->O;
    k_normalize<<<blocks_for((long long)B * I), 256, 0, st>>>(d_features, m->mean, m->stdv, B, I, m->xn);
    k_dense<<<blocks_for((long long)B * H), 256, 0, st>>>(m->xn, B, I, m->W1(), m->b1(), H, m->z1, m->a1);
    k_dense<<<blocks_for((long long)B * H), 256, 0, st>>>(m->a1, B, H, m->W2(), m->b2(), H, m->z2, m->a2);
    k_dense<<<blocks_for((long long)B * O), 256, 0, st>>>(m->a2, B, H, m->W3(), m->b3(), O, m->z3, nullptr);
    return cudaGetLastError();
}

// forward + backward into m->grads; loss in m->loss
static cudaError_t mlp_backward(bhsp_mlp* m, const float* d_features, const float* d_targets, int B,
                                cudaStream_t st) {
    const int I = m->I, H = m->H, O = m->O;
    cudaError_t e = mlp_forward(m, d_features, B, st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(m->loss, 0, sizeof(float), st);
    if (e != cudaSuccess) return e;
    k_softmax_xent<<<blocks_for(B), 256, 0, st>>>(m->z3, d_targets, B, O, m->p, m->dz3, m->loss);
    float* g = m->grads;
    float* gW1 = g;
    float* gb1 = gW1 + H * I;
    float* gW2 = gb1 + H;
    float* gb2 = gW2 + H * H;
    float* gW3 = gb2 + H;
    float* gb3 = gW3 + O * H;
    k_grad_w<<<blocks_for((long long)O * (H + 1)), 256, 0, st>>>(m->dz3, m->a2, B, O, H, gW3, gb3);
    k_back_input<<<blocks_for((long long)B * H), 256, 0, st>>>(m->dz3, B, O, m->W3(), H, m->z2, m->dz2);
    k_grad_w<<<blocks_for((long long)H * (H + 1)), 256, 0, st>>>(m->dz2, m->a1, B, H, H, gW2, gb2);
    k_back_input<<<blocks_for((long long)B * H), 256, 0, st>>>(m->dz2, B, H, m->W2(), H, m->z1, m->dz1);
    k_grad_w<<<blocks_for((long long)H * (I + 1)), 256, 0, st>>>(m->dz1, m->xn, B, H, I, gW1, gb1);
    return cudaGetLastError();
}

extern "C" int bhsp_mlp_forward(bhsp_mlp* m, const float* d_features, int batch, float* d_probs,
                                void* stream) {
    if (!m || !d_features || !d_probs || batch < 1 || batch > m->max_batch)
        return BHSPARSE_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = mlp_forward(m, d_features, batch, st);
    if (e == cudaSuccess) {
        k_softmax_xent<<<blocks_for(batch), 256, 0, st>>>(m->z3, nullptr, batch, m->O, d_probs,
                                                          nullptr, nullptr);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? BHSPARSE_SUCCESS : BHSPARSE_CUDA_ERROR;
}

extern "C" int bhsp_mlp_gradients(bhsp_mlp* m, const float* d_features, const float* d_targets,
                                  int batch, float* d_grads_out, float* loss_out, void* stream) {
    if (!m || !d_features || !d_targets || batch < 1 || batch > m->max_batch)
        return BHSPARSE_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = mlp_backward(m, d_features, d_targets, batch, st);
    if (e == cudaSuccess && d_grads_out)
        e = cudaMemcpyAsync(d_grads_out, m->grads, sizeof(float) * m->nparams, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess && loss_out)
        e = cudaMemcpyAsync(loss_out, m->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? BHSPARSE_SUCCESS : BHSPARSE_CUDA_ERROR;
}

extern "C" int bhsp_mlp_train_step(bhsp_mlp* m, const float* d_features, const float* d_targets,
                                   int batch, float lr, float weight_decay, float* loss_out,
                                   void* stream) {
    if (!m || !d_features || !d_targets || batch < 1 || batch > m->max_batch || !(lr > 0.f))
        return BHSPARSE_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = mlp_backward(m, d_features, d_targets, batch, st);
    if (e != cudaSuccess) return BHSPARSE_CUDA_ERROR;
    m->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - powf(b1, (float)m->step), bc2 = 1.f - powf(b2, (float)m->step);
    k_adam<<<blocks_for((long long)m->nparams), 256, 0, st>>>(m->params, m->grads, m->m1, m->m2,
                                                            (int)m->nparams, lr, b1, b2, 1e-8f,
                                                            bc1, bc2, weight_decay);
    e = cudaGetLastError();
    if (e == cudaSuccess && loss_out)
        e = cudaMemcpyAsync(loss_out, m->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && loss_out) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? BHSPARSE_SUCCESS : BHSPARSE_CUDA_ERROR;
}

extern "C" void bhsp_mlp_destroy(bhsp_mlp* m) {
    if (!m) return;
    mlp_free(m);
    delete m;
}
