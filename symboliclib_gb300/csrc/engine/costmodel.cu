// Learned schedule cost model: a small FP32 multilayer perceptron
// (inputs -> hidden -> hidden -> 1, ReLU) that predicts the log run time of a
// unit under a schedule from plan and schedule features.  Training and
// inference run on the GPU with the kernels below (dense forward, backward,
// Adam update); the training data are the autotuner's own timings.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "symgb.h"
#include "unit.hpp"

namespace {

constexpr int kTile = 32;  // samples per block in the dense kernels

// Y[n, o] = act(b[o] + sum_i X[n, i] W[i, o]); W (in x out) staged in shared memory.
__global__ void denseForward(const float* __restrict__ X, const float* __restrict__ W, const float* __restrict__ b,
                             float* __restrict__ Y, int n, int in, int out, int relu) {
    extern __shared__ float sW[];
    for (int q = threadIdx.x; q < in * out; q += blockDim.x) sW[q] = W[q];
    __syncthreads();
    const int row0 = blockIdx.x * kTile;
    for (int q = threadIdx.x; q < kTile * out; q += blockDim.x) {
        const int r = row0 + q / out, o = q % out;
        if (r >= n) continue;
        float acc = b[o];
        const float* x = X + (std::size_t)r * in;
        for (int i = 0; i < in; ++i) acc = fmaf(x[i], sW[i * out + o], acc);
        Y[(std::size_t)r * out + o] = relu ? fmaxf(acc, 0.f) : acc;
    }
}

// dZ = dY * relu'(Y) (in place when relu), per element.
__global__ void reluBackward(float* __restrict__ dY, const float* __restrict__ Y, std::size_t count) {
    const std::size_t q = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < count && Y[q] <= 0.f) dY[q] = 0.f;
}

// dW[i, o] = sum_n X[n, i] dZ[n, o]; db[o] = sum_n dZ[n, o].  One block per
// weight column o; threads stride over inputs i and samples.
__global__ void denseGradW(const float* __restrict__ X, const float* __restrict__ dZ, float* __restrict__ dW,
                           float* __restrict__ db, int n, int in, int out) {
    const int o = blockIdx.x;
    __shared__ float red[256];
    for (int i = -1; i < in; ++i) {  // i = -1: bias
        float acc = 0.f;
        for (int r = threadIdx.x; r < n; r += blockDim.x)
            acc += dZ[(std::size_t)r * out + o] * (i < 0 ? 1.f : X[(std::size_t)r * in + i]);
        red[threadIdx.x] = acc;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (i < 0)
                db[o] = red[0];
            else
                dW[i * out + o] = red[0];
        }
        __syncthreads();
    }
}

// dX[n, i] = sum_o dZ[n, o] W[i, o]
__global__ void denseGradX(const float* __restrict__ dZ, const float* __restrict__ W, float* __restrict__ dX, int n,
                           int in, int out) {
    const std::size_t q = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (std::size_t)n * in) return;
    const int r = (int)(q / in), i = (int)(q % in);
    float acc = 0.f;
    for (int o = 0; o < out; ++o) acc = fmaf(dZ[(std::size_t)r * out + o], W[i * out + o], acc);
    dX[q] = acc;
}

// d = 2 (pred - y) / n  and  per-sample squared error.
__global__ void mseBackward(const float* __restrict__ pred, const float* __restrict__ y, float* __restrict__ d,
                            float* __restrict__ sq, int n) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float e = pred[r] - y[r];
    d[r] = 2.f * e / n;
    sq[r] = e * e;
}

__global__ void adamStep(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                         int count, float lr, float b1, float b2, float c1, float c2, float eps) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count) return;
    const float gi = g[q];
    m[q] = b1 * m[q] + (1.f - b1) * gi;
    v[q] = b2 * v[q] + (1.f - b2) * gi * gi;
    p[q] -= lr * (m[q] / c1) / (sqrtf(v[q] / c2) + eps);
}

}  // namespace

struct symgb_mlp {
    int in = 0, hidden = 0;
    // parameter layout: W1 (in x h), b1 (h), W2 (h x h), b2 (h), W3 (h x 1), b3 (1)
    std::size_t oW1, ob1, oW2, ob2, oW3, ob3, count;
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
    float *X = nullptr, *y = nullptr, *h1 = nullptr, *h2 = nullptr, *out = nullptr, *d3 = nullptr, *d2 = nullptr,
          *d1 = nullptr, *sq = nullptr;
    int cap = 0, step = 0;
    ~symgb_mlp() {
        for (float* p : {params, grads, m, v, X, y, h1, h2, out, d3, d2, d1, sq})
            if (p) cudaFree(p);
    }
};

namespace {

int mlpFail(int code, const std::string& msg) { return symgb::engine::setLastError(code, msg); }

#define MLP_CUDA(call)                                                                                      \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) return mlpFail(SYMGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int ensureBatch(symgb_mlp* net, int n) {
    if (n <= net->cap) return SYMGB_OK;
    for (float** p : {&net->X, &net->y, &net->h1, &net->h2, &net->out, &net->d3, &net->d2, &net->d1, &net->sq})
        if (*p) {
            cudaFree(*p);
            *p = nullptr;
        }
    const std::size_t h = net->hidden;
    MLP_CUDA(cudaMalloc(&net->X, sizeof(float) * n * net->in));
    MLP_CUDA(cudaMalloc(&net->y, sizeof(float) * n));
    MLP_CUDA(cudaMalloc(&net->h1, sizeof(float) * n * h));
    MLP_CUDA(cudaMalloc(&net->h2, sizeof(float) * n * h));
    MLP_CUDA(cudaMalloc(&net->out, sizeof(float) * n));
    MLP_CUDA(cudaMalloc(&net->d3, sizeof(float) * n));
    MLP_CUDA(cudaMalloc(&net->d2, sizeof(float) * n * h));
    MLP_CUDA(cudaMalloc(&net->d1, sizeof(float) * n * h));
    MLP_CUDA(cudaMalloc(&net->sq, sizeof(float) * n));
    net->cap = n;
    return SYMGB_OK;
}

void forward(symgb_mlp* net, int n) {
    const int h = net->hidden, blocks = (n + kTile - 1) / kTile;
    const float* P = net->params;
    denseForward<<<blocks, 256, sizeof(float) * net->in * h>>>(net->X, P + net->oW1, P + net->ob1, net->h1, n, net->in, h, 1);
    denseForward<<<blocks, 256, sizeof(float) * h * h>>>(net->h1, P + net->oW2, P + net->ob2, net->h2, n, h, h, 1);
    denseForward<<<blocks, 256, sizeof(float) * h>>>(net->h2, P + net->oW3, P + net->ob3, net->out, n, h, 1, 0);
}

// Gradient of the mean squared error into net->grads.
void backward(symgb_mlp* net, int n) {
    const int h = net->hidden;
    const float* P = net->params;
    float* G = net->grads;
    mseBackward<<<(n + 255) / 256, 256>>>(net->out, net->y, net->d3, net->sq, n);
    denseGradW<<<1, 256>>>(net->h2, net->d3, G + net->oW3, G + net->ob3, n, h, 1);
    denseGradX<<<(unsigned)(((std::size_t)n * h + 255) / 256), 256>>>(net->d3, P + net->oW3, net->d2, n, h, 1);
    reluBackward<<<(unsigned)(((std::size_t)n * h + 255) / 256), 256>>>(net->d2, net->h2, (std::size_t)n * h);
    denseGradW<<<h, 256>>>(net->h1, net->d2, G + net->oW2, G + net->ob2, n, h, h);
    denseGradX<<<(unsigned)(((std::size_t)n * h + 255) / 256), 256>>>(net->d2, P + net->oW2, net->d1, n, h, h);
    reluBackward<<<(unsigned)(((std::size_t)n * h + 255) / 256), 256>>>(net->d1, net->h1, (std::size_t)n * h);
    denseGradW<<<h, 256>>>(net->X, net->d1, G + net->oW1, G + net->ob1, n, net->in, h);
}

int upload(symgb_mlp* net, const float* X, const float* y, int n) {
    if (int e = ensureBatch(net, n)) return e;
    MLP_CUDA(cudaMemcpy(net->X, X, sizeof(float) * n * net->in, cudaMemcpyHostToDevice));
    if (y) MLP_CUDA(cudaMemcpy(net->y, y, sizeof(float) * n, cudaMemcpyHostToDevice));
    return SYMGB_OK;
}

int meanLoss(symgb_mlp* net, int n, float* loss) {
    std::vector<float> sq(n);
    MLP_CUDA(cudaMemcpy(sq.data(), net->sq, sizeof(float) * n, cudaMemcpyDeviceToHost));
    double s = 0;
    for (float e : sq) s += e;
    *loss = (float)(s / n);
    return SYMGB_OK;
}

}  // namespace

extern "C" {

int symgb_mlp_create(int inputs, int hidden, unsigned long long seed, symgb_mlp_t* out) {
    if (!out || inputs <= 0 || hidden <= 0 || hidden > 256 || inputs > 256) return mlpFail(SYMGB_ERR_ARGUMENT, "bad MLP shape");
    std::unique_ptr<symgb_mlp> net(new symgb_mlp());
    net->in = inputs;
    net->hidden = hidden;
    std::size_t o = 0;
    net->oW1 = o; o += (std::size_t)inputs * hidden;
    net->ob1 = o; o += hidden;
    net->oW2 = o; o += (std::size_t)hidden * hidden;
    net->ob2 = o; o += hidden;
    net->oW3 = o; o += hidden;
    net->ob3 = o; o += 1;
    net->count = o;
    // He-style initialisation from a seeded generator (host), biases zero.
    std::vector<float> p(o, 0.f);
    std::uint64_t s = seed * 0x9e3779b97f4a7c15ULL + 1;
    auto uni = [&]() {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        return (float)((s >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
    };
    const float a1 = std::sqrt(6.f / inputs), a2 = std::sqrt(6.f / hidden);
    for (std::size_t q = 0; q < (std::size_t)inputs * hidden; ++q) p[net->oW1 + q] = a1 * uni();
    for (std::size_t q = 0; q < (std::size_t)hidden * hidden; ++q) p[net->oW2 + q] = a2 * uni();
    for (int q = 0; q < hidden; ++q) p[net->oW3 + q] = a2 * uni();
    for (float** b : {&net->params, &net->grads, &net->m, &net->v}) MLP_CUDA(cudaMalloc(b, sizeof(float) * o));
    MLP_CUDA(cudaMemcpy(net->params, p.data(), sizeof(float) * o, cudaMemcpyHostToDevice));
    MLP_CUDA(cudaMemset(net->m, 0, sizeof(float) * o));
    MLP_CUDA(cudaMemset(net->v, 0, sizeof(float) * o));
    *out = net.release();
    return SYMGB_OK;
}

int symgb_mlp_num_params(symgb_mlp_t net) { return net ? (int)net->count : 0; }

int symgb_mlp_get_params(symgb_mlp_t net, float* p) {
    if (!net || !p) return mlpFail(SYMGB_ERR_ARGUMENT, "null argument");
    MLP_CUDA(cudaMemcpy(p, net->params, sizeof(float) * net->count, cudaMemcpyDeviceToHost));
    return SYMGB_OK;
}

int symgb_mlp_set_params(symgb_mlp_t net, const float* p) {
    if (!net || !p) return mlpFail(SYMGB_ERR_ARGUMENT, "null argument");
    MLP_CUDA(cudaMemcpy(net->params, p, sizeof(float) * net->count, cudaMemcpyHostToDevice));
    MLP_CUDA(cudaMemset(net->m, 0, sizeof(float) * net->count));
    MLP_CUDA(cudaMemset(net->v, 0, sizeof(float) * net->count));
    net->step = 0;
    return SYMGB_OK;
}

int symgb_mlp_forward(symgb_mlp_t net, const float* X, int n, float* y) {
    if (!net || !X || !y || n <= 0) return mlpFail(SYMGB_ERR_ARGUMENT, "bad forward arguments");
    if (int e = upload(net, X, nullptr, n)) return e;
    forward(net, n);
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaMemcpy(y, net->out, sizeof(float) * n, cudaMemcpyDeviceToHost));
    return SYMGB_OK;
}

int symgb_mlp_gradient(symgb_mlp_t net, const float* X, const float* y, int n, float* grad, float* loss) {
    if (!net || !X || !y || !grad || n <= 0) return mlpFail(SYMGB_ERR_ARGUMENT, "bad gradient arguments");
    if (int e = upload(net, X, y, n)) return e;
    forward(net, n);
    backward(net, n);
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaMemcpy(grad, net->grads, sizeof(float) * net->count, cudaMemcpyDeviceToHost));
    if (loss) return meanLoss(net, n, loss);
    return SYMGB_OK;
}

int symgb_mlp_train(symgb_mlp_t net, const float* X, const float* y, int n, int epochs, float lr, float* loss) {
    if (!net || !X || !y || n <= 0 || epochs < 0) return mlpFail(SYMGB_ERR_ARGUMENT, "bad training arguments");
    if (int e = upload(net, X, y, n)) return e;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const int blocks = (int)((net->count + 255) / 256);
    for (int ep = 0; ep < epochs; ++ep) {
        forward(net, n);
        backward(net, n);
        ++net->step;
        const float c1 = 1.f - std::pow(b1, (float)net->step), c2 = 1.f - std::pow(b2, (float)net->step);
        adamStep<<<blocks, 256>>>(net->params, net->grads, net->m, net->v, (int)net->count, lr, b1, b2, c1, c2, eps);
    }
    MLP_CUDA(cudaGetLastError());
    forward(net, n);
    mseBackward<<<(n + 255) / 256, 256>>>(net->out, net->y, net->d3, net->sq, n);
    MLP_CUDA(cudaDeviceSynchronize());
    if (loss) return meanLoss(net, n, loss);
    return SYMGB_OK;
}

void symgb_mlp_destroy(symgb_mlp_t net) { delete net; }

}  // extern "C"
