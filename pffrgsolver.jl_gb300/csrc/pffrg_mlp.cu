// The learned parquet warm start (sm_103a): a small multilayer perceptron that maps the
// couplings of a model to the principal-component coordinates of its converged parquet
// vertex, with a fixed affine decoder (the component basis and the mean) behind it.
// Forward, backward (mean-squared error), Adam and the decoder are plain FP32 kernels: the
// network is a few thousand parameters trained on a few hundred samples, so every kernel is
// launch-bound and written for exact, deterministic sums (one thread per output, no atomics).
// It has no counterpart in the reference: the parquet iteration it starts
// (src/Launcher/parquet.jl) stays the judge of convergence.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pffrg_gpu.h"

namespace {

constexpr int kMaxLayers = 8;

__global__ void dense_forward(const float* __restrict__ X, const float* __restrict__ W, const float* __restrict__ b,
                              float* Y, int batch, int nin, int nout, int act) {
    // Y[r, j] = act(sum_i X[r, i] W[i, j] + b[j]), row-major X[batch][nin], W[nin][nout]
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)batch * nout) return;
    const int r = (int)(e / nout), j = (int)(e % nout);
    float z = b ? b[j] : 0.0f;
    for (int i = 0; i < nin; ++i) z += X[(size_t)r * nin + i] * W[(size_t)i * nout + j];
    Y[e] = act ? tanhf(z) : z;
}

__global__ void mse_grad(const float* __restrict__ Y, const float* __restrict__ T, float* dY, int n, float scale) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) dY[e] = scale * (Y[e] - T[e]);
}

__global__ void mse_loss(const float* __restrict__ Y, const float* __restrict__ T, int n, float* loss) {
    __shared__ float s[256];
    float acc = 0.0f;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const float d = Y[e] - T[e];
        acc += d * d;
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss[0] = s[0] / (float)n;
}

// dZ = dY * act'(Y) in place (tanh: 1 - Y^2)
__global__ void act_backward(const float* __restrict__ Y, float* dY, int n, int act) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n && act) dY[e] *= 1.0f - Y[e] * Y[e];
}

// dW[i, j] = sum_r X[r, i] dZ[r, j]; db[j] = sum_r dZ[r, j]
__global__ void dense_wgrad(const float* __restrict__ X, const float* __restrict__ dZ, float* dW, float* db, int batch,
                            int nin, int nout) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nin * nout) {
        const int i = e / nout, j = e % nout;
        float g = 0.0f;
        for (int r = 0; r < batch; ++r) g += X[(size_t)r * nin + i] * dZ[(size_t)r * nout + j];
        dW[e] = g;
    } else if (e < nin * nout + nout) {
        const int j = e - nin * nout;
        float g = 0.0f;
        for (int r = 0; r < batch; ++r) g += dZ[(size_t)r * nout + j];
        db[j] = g;
    }
}

// dX[r, i] = sum_j dZ[r, j] W[i, j]
__global__ void dense_xgrad(const float* __restrict__ dZ, const float* __restrict__ W, float* dX, int batch, int nin,
                            int nout) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= batch * nin) return;
    const int r = e / nin, i = e % nin;
    float g = 0.0f;
    for (int j = 0; j < nout; ++j) g += dZ[(size_t)r * nout + j] * W[(size_t)i * nout + j];
    dX[e] = g;
}

__global__ void adam_step(float* p, const float* __restrict__ g, float* m, float* v, int n, float lr, float b1, float b2,
                          float eps, float c1, float c2) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    m[e] = b1 * m[e] + (1.0f - b1) * g[e];
    v[e] = b2 * v[e] + (1.0f - b2) * g[e] * g[e];
    const float mh = m[e] / c1, vh = v[e] / c2;
    p[e] -= lr * mh / (sqrtf(vh) + eps);
}

int blocks(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

struct pffrg_mlp {
    int nlayers = 0;               // dense layers (tanh on all but the last)
    int sizes[kMaxLayers + 1] = {};
    long long nparams = 0;
    float* params = nullptr;       // per layer: W[nin][nout] then b[nout]
    float* grads = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    long long adam_t = 0;
    float* act = nullptr;          // activations of all layers for a batch (input copied in)
    float* dact = nullptr;
    int act_batch = 0;
    float* target = nullptr;
    float* loss = nullptr;
    float* dec_basis = nullptr;    // decoder: out[d] = mean[d] + sum_k z[k] basis[k][d]
    float* dec_mean = nullptr;
    int dec_k = 0;
    long long dec_d = 0;
    float* dec_out = nullptr;
    cudaStream_t st = nullptr;
    std::string err;
    long long woff(int l) const {
        long long o = 0;
        for (int k = 0; k < l; ++k) o += (long long)sizes[k] * sizes[k + 1] + sizes[k + 1];
        return o;
    }
    long long aoff(int l) const {  // activation offset of layer output l (0 = the input)
        long long o = 0;
        for (int k = 0; k < l; ++k) o += (long long)act_batch * sizes[k];
        return o;
    }
};

#define MLP_CK(call)                                                             \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if (e_ != cudaSuccess) {                                                 \
            h->err = std::string(#call) + ": " + cudaGetErrorString(e_);         \
            return PFFRG_E_CUDA;                                                 \
        }                                                                        \
    } while (0)

namespace {

int ensure_batch(pffrg_mlp* h, int batch) {
    if (batch <= h->act_batch && h->act) return 0;
    if (h->act) cudaFree(h->act);
    if (h->dact) cudaFree(h->dact);
    if (h->target) cudaFree(h->target);
    h->act = h->dact = h->target = nullptr;
    h->act_batch = batch;
    long long tot = 0;
    for (int l = 0; l <= h->nlayers; ++l) tot += (long long)batch * h->sizes[l];
    MLP_CK(cudaMalloc(&h->act, sizeof(float) * tot));
    MLP_CK(cudaMalloc(&h->dact, sizeof(float) * tot));
    MLP_CK(cudaMalloc(&h->target, sizeof(float) * (size_t)batch * h->sizes[h->nlayers]));
    return 0;
}

int forward(pffrg_mlp* h, int batch) {
    for (int l = 0; l < h->nlayers; ++l) {
        const float* W = h->params + h->woff(l);
        const float* b = W + (long long)h->sizes[l] * h->sizes[l + 1];
        const long long n = (long long)batch * h->sizes[l + 1];
        dense_forward<<<blocks(n, 128), 128, 0, h->st>>>(h->act + h->aoff(l), W, b, h->act + h->aoff(l + 1), batch,
                                                        h->sizes[l], h->sizes[l + 1], l + 1 < h->nlayers);
        MLP_CK(cudaGetLastError());
    }
    return 0;
}

// gradients of the mean-squared error over the batch into h->grads; loss into h->loss
int backward(pffrg_mlp* h, int batch) {
    const int L = h->nlayers;
    const int nout = h->sizes[L];
    const int n = batch * nout;
    const float* Y = h->act + h->aoff(L);
    mse_loss<<<1, 256, 0, h->st>>>(Y, h->target, n, h->loss);
    mse_grad<<<blocks(n, 256), 256, 0, h->st>>>(Y, h->target, h->dact + h->aoff(L), n, 2.0f / (float)n);
    MLP_CK(cudaGetLastError());
    for (int l = L - 1; l >= 0; --l) {
        const int nin = h->sizes[l], no = h->sizes[l + 1];
        float* dZ = h->dact + h->aoff(l + 1);
        act_backward<<<blocks((long long)batch * no, 256), 256, 0, h->st>>>(h->act + h->aoff(l + 1), dZ, batch * no,
                                                                            l + 1 < L);
        float* dW = h->grads + h->woff(l);
        float* db = dW + (long long)nin * no;
        dense_wgrad<<<blocks((long long)nin * no + no, 128), 128, 0, h->st>>>(h->act + h->aoff(l), dZ, dW, db, batch,
                                                                            nin, no);
        if (l > 0)
            dense_xgrad<<<blocks((long long)batch * nin, 128), 128, 0, h->st>>>(dZ, h->params + h->woff(l),
                                                                               h->dact + h->aoff(l), batch, nin, no);
        MLP_CK(cudaGetLastError());
    }
    return 0;
}

}  // namespace

extern "C" {

pffrg_mlp* pffrg_mlp_create(int nlayers, const int* sizes, unsigned seed) {
    if (nlayers < 1 || nlayers > kMaxLayers || !sizes) return nullptr;
    pffrg_mlp* h = new pffrg_mlp();
    h->nlayers = nlayers;
    for (int l = 0; l <= nlayers; ++l) {
        if (sizes[l] < 1) {
            delete h;
            return nullptr;
        }
        h->sizes[l] = sizes[l];
    }
    h->nparams = h->woff(nlayers);
    // Xavier-uniform weights, zero biases, from a seeded generator
    std::vector<float> p((size_t)h->nparams, 0.0f);
    std::mt19937 gen(seed);
    for (int l = 0; l < nlayers; ++l) {
        const float a = std::sqrt(6.0f / (float)(sizes[l] + sizes[l + 1]));
        std::uniform_real_distribution<float> U(-a, a);
        float* W = p.data() + h->woff(l);
        for (long long k = 0; k < (long long)sizes[l] * sizes[l + 1]; ++k) W[k] = U(gen);
    }
    bool ok = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&h->params, sizeof(float) * h->nparams) == cudaSuccess &&
              cudaMalloc(&h->grads, sizeof(float) * h->nparams) == cudaSuccess &&
              cudaMalloc(&h->adam_m, sizeof(float) * h->nparams) == cudaSuccess &&
              cudaMalloc(&h->adam_v, sizeof(float) * h->nparams) == cudaSuccess &&
              cudaMalloc(&h->loss, sizeof(float)) == cudaSuccess;
    ok = ok && cudaMemcpy(h->params, p.data(), sizeof(float) * h->nparams, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(h->adam_m, 0, sizeof(float) * h->nparams) == cudaSuccess &&
         cudaMemset(h->adam_v, 0, sizeof(float) * h->nparams) == cudaSuccess;
    if (!ok) {
        pffrg_mlp_destroy(h);
        return nullptr;
    }
    return h;
}

void pffrg_mlp_destroy(pffrg_mlp* h) {
    if (!h) return;
    if (h->st) cudaStreamSynchronize(h->st);
    for (float* p : {h->params, h->grads, h->adam_m, h->adam_v, h->act, h->dact, h->target, h->loss, h->dec_basis,
                     h->dec_mean, h->dec_out})
        if (p) cudaFree(p);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
}

const char* pffrg_mlp_last_error(const pffrg_mlp* h) { return h ? h->err.c_str() : "null network"; }

int64_t pffrg_mlp_num_params(const pffrg_mlp* h) { return h ? h->nparams : 0; }

int pffrg_mlp_get_params(pffrg_mlp* h, float* out) {
    if (!h || !out) return PFFRG_E_ARGS;
    MLP_CK(cudaMemcpyAsync(out, h->params, sizeof(float) * h->nparams, cudaMemcpyDeviceToHost, h->st));
    MLP_CK(cudaStreamSynchronize(h->st));
    return 0;
}

int pffrg_mlp_set_params(pffrg_mlp* h, const float* in) {
    if (!h || !in) return PFFRG_E_ARGS;
    MLP_CK(cudaMemcpyAsync(h->params, in, sizeof(float) * h->nparams, cudaMemcpyHostToDevice, h->st));
    MLP_CK(cudaStreamSynchronize(h->st));
    return 0;
}

int pffrg_mlp_forward(pffrg_mlp* h, const float* X, int batch, float* Y) {
    if (!h || !X || !Y || batch < 1) return PFFRG_E_ARGS;
    if (int rc = ensure_batch(h, batch)) return rc;
    MLP_CK(cudaMemcpyAsync(h->act, X, sizeof(float) * (size_t)batch * h->sizes[0], cudaMemcpyHostToDevice, h->st));
    if (int rc = forward(h, batch)) return rc;
    MLP_CK(cudaMemcpyAsync(Y, h->act + h->aoff(h->nlayers), sizeof(float) * (size_t)batch * h->sizes[h->nlayers],
                           cudaMemcpyDeviceToHost, h->st));
    MLP_CK(cudaStreamSynchronize(h->st));
    return 0;
}

int pffrg_mlp_gradient(pffrg_mlp* h, const float* X, const float* T, int batch, float* grads, float* loss) {
    if (!h || !X || !T || batch < 1) return PFFRG_E_ARGS;
    if (int rc = ensure_batch(h, batch)) return rc;
    MLP_CK(cudaMemcpyAsync(h->act, X, sizeof(float) * (size_t)batch * h->sizes[0], cudaMemcpyHostToDevice, h->st));
    MLP_CK(cudaMemcpyAsync(h->target, T, sizeof(float) * (size_t)batch * h->sizes[h->nlayers], cudaMemcpyHostToDevice,
                           h->st));
    if (int rc = forward(h, batch)) return rc;
    if (int rc = backward(h, batch)) return rc;
    if (grads) MLP_CK(cudaMemcpyAsync(grads, h->grads, sizeof(float) * h->nparams, cudaMemcpyDeviceToHost, h->st));
    if (loss) MLP_CK(cudaMemcpyAsync(loss, h->loss, sizeof(float), cudaMemcpyDeviceToHost, h->st));
    MLP_CK(cudaStreamSynchronize(h->st));
    return 0;
}

int pffrg_mlp_train(pffrg_mlp* h, const float* X, const float* T, int batch, int epochs, float lr, float* loss) {
    if (!h || !X || !T || batch < 1 || epochs < 0) return PFFRG_E_ARGS;
    if (int rc = ensure_batch(h, batch)) return rc;
    MLP_CK(cudaMemcpyAsync(h->act, X, sizeof(float) * (size_t)batch * h->sizes[0], cudaMemcpyHostToDevice, h->st));
    MLP_CK(cudaMemcpyAsync(h->target, T, sizeof(float) * (size_t)batch * h->sizes[h->nlayers], cudaMemcpyHostToDevice,
                           h->st));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int ep = 0; ep < epochs; ++ep) {
        if (int rc = forward(h, batch)) return rc;
        if (int rc = backward(h, batch)) return rc;
        ++h->adam_t;
        const float c1 = 1.0f - std::pow(b1, (float)h->adam_t), c2 = 1.0f - std::pow(b2, (float)h->adam_t);
        adam_step<<<blocks(h->nparams, 256), 256, 0, h->st>>>(h->params, h->grads, h->adam_m, h->adam_v,
                                                              (int)h->nparams, lr, b1, b2, eps, c1, c2);
        MLP_CK(cudaGetLastError());
    }
    if (int rc = forward(h, batch)) return rc;
    if (int rc = backward(h, batch)) return rc;
    if (loss) MLP_CK(cudaMemcpyAsync(loss, h->loss, sizeof(float), cudaMemcpyDeviceToHost, h->st));
    MLP_CK(cudaStreamSynchronize(h->st));
    return 0;
}

int pffrg_mlp_set_decoder(pffrg_mlp* h, const float* basis, const float* mean, int k, int64_t d) {
    if (!h || !basis || !mean || k != h->sizes[h->nlayers] || d < 1) return PFFRG_E_ARGS;
    for (float* p : {h->dec_basis, h->dec_mean, h->dec_out})
        if (p) cudaFree(p);
    h->dec_basis = h->dec_mean = h->dec_out = nullptr;
    MLP_CK(cudaMalloc(&h->dec_basis, sizeof(float) * (size_t)k * d));
    MLP_CK(cudaMalloc(&h->dec_mean, sizeof(float) * (size_t)d));
    MLP_CK(cudaMalloc(&h->dec_out, sizeof(float) * (size_t)d));
    MLP_CK(cudaMemcpyAsync(h->dec_basis, basis, sizeof(float) * (size_t)k * d, cudaMemcpyHostToDevice, h->st));
    MLP_CK(cudaMemcpyAsync(h->dec_mean, mean, sizeof(float) * (size_t)d, cudaMemcpyHostToDevice, h->st));
    MLP_CK(cudaStreamSynchronize(h->st));
    h->dec_k = k;
    h->dec_d = d;
    return 0;
}

int pffrg_mlp_predict(pffrg_mlp* h, const float* x, float* out) {
    // one sample: z = network(x), out = mean + z basis (the decoder as one more dense layer)
    if (!h || !x || !out || !h->dec_basis) return PFFRG_E_ARGS;
    if (int rc = ensure_batch(h, 1)) return rc;
    MLP_CK(cudaMemcpyAsync(h->act, x, sizeof(float) * h->sizes[0], cudaMemcpyHostToDevice, h->st));
    if (int rc = forward(h, 1)) return rc;
    dense_forward<<<blocks(h->dec_d, 256), 256, 0, h->st>>>(h->act + h->aoff(h->nlayers), h->dec_basis, h->dec_mean,
                                                            h->dec_out, 1, h->dec_k, (int)h->dec_d, 0);
    MLP_CK(cudaGetLastError());
    MLP_CK(cudaMemcpyAsync(out, h->dec_out, sizeof(float) * (size_t)h->dec_d, cudaMemcpyDeviceToHost, h->st));
    MLP_CK(cudaStreamSynchronize(h->st));
    return 0;
}

}  // extern "C"
