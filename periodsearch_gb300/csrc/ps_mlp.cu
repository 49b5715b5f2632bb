// ps_mlp.cu -- training and inference kernels of the learned early-stop
// predictor: a 10-64-64-1 multilayer perceptron with GELU activations in
// FP32.  It maps the first K iterations of an LM fit (the screening depth:
// accepted chi^2 ratios and lambda every K/4 iterations, Ndata, period) to
// log(final rms / rms after those iterations).  Parameters live in one float array (layout kMlp* in
// ps_engine.h): input mean/std, W1[64][10], b1, W2[64][64], b2, W3[64], b3,
// target mean/std.  Standardisation constants are computed on the host;
// training updates W1..b3 with Adam on mean squared error.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <random>
#include <vector>

#include "ps_engine.h"

namespace psg {

namespace {

__device__ inline float gelu_f(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ inline float gelu_grad(float x)
{
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// x_std[b][i] = (x[idx[b]][i] - mu[i]) / sd[i], y_std[b] likewise.
__global__ void gather_std(const float *x, const float *y, const int *idx, const float *P, float *xs, float *ys,
                           int B)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < B * kFeat) {
        const int b = t / kFeat, i = t - b * kFeat;
        const int r = idx ? idx[b] : b;
        xs[t] = (x[static_cast<size_t>(r) * kFeat + i] - P[kMlpMu + i]) / P[kMlpSd + i];
    }
    if (t < B && y) {
        const int r = idx ? idx[t] : t;
        ys[t] = (y[r] - P[kMlpYMu]) / P[kMlpYSd];
    }
}

// z[b][u] = bias[u] + sum_i W[u][i] in[b][i]; h = gelu(z).
__global__ void dense_fwd(const float *in, const float *W, const float *bias, float *z, float *h, int B, int din,
                          int dout)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= B * dout) return;
    const int b = t / dout, u = t - b * dout;
    float acc = bias[u];
    for (int i = 0; i < din; i++) acc = fmaf(W[u * din + i], in[static_cast<size_t>(b) * din + i], acc);
    z[t] = acc;
    h[t] = gelu_f(acc);
}

// out[b] = b3 + W3 . h2[b]; dout[b] = 2 (out - y) / B; loss partial per block.
__global__ void out_layer(const float *h2, const float *W3, const float *b3, const float *ys, float *out, float *dout,
                          float *loss, int B)
{
    __shared__ float red[256];
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (b < B) {
        float acc = b3[0];
        for (int j = 0; j < kHidden; j++) acc = fmaf(W3[j], h2[static_cast<size_t>(b) * kHidden + j], acc);
        out[b] = acc;
        if (ys) {
            const float d = acc - ys[b];
            dout[b] = 2.f * d / B;
            l = d * d / B;
        }
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0 && loss) atomicAdd(loss, red[0]);
}

// dz2[b][u] = dout[b] W3[u] gelu'(z2[b][u]); grads of W3, b3.
__global__ void out_back(const float *dout, const float *W3, const float *z2, const float *h2, float *dz2, float *gW3,
                         float *gb3, int B)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < B * kHidden) {
        const int b = t / kHidden, u = t - b * kHidden;
        dz2[t] = dout[b] * W3[u] * gelu_grad(z2[t]);
    }
    if (t < kHidden) {
        float g = 0.f;
        for (int b = 0; b < B; b++) g = fmaf(dout[b], h2[static_cast<size_t>(b) * kHidden + t], g);
        gW3[t] = g;
    }
    if (t == 0) {
        float g = 0.f;
        for (int b = 0; b < B; b++) g += dout[b];
        gb3[0] = g;
    }
}

// gW[u][i] = sum_b dz[b][u] in[b][i]; gb[u] = sum_b dz[b][u].
__global__ void dense_grad_params(const float *dz, const float *in, float *gW, float *gb, int B, int din, int dout)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < dout * din) {
        const int u = t / din, i = t - u * din;
        float g = 0.f;
        for (int b = 0; b < B; b++) g = fmaf(dz[static_cast<size_t>(b) * dout + u], in[static_cast<size_t>(b) * din + i], g);
        gW[t] = g;
    }
    if (t < dout) {
        float g = 0.f;
        for (int b = 0; b < B; b++) g += dz[static_cast<size_t>(b) * dout + t];
        gb[t] = g;
    }
}

// dzprev[b][i] = gelu'(zprev[b][i]) sum_u dz[b][u] W[u][i].
__global__ void dense_grad_input(const float *dz, const float *W, const float *zprev, float *dzprev, int B, int din,
                                 int dout)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= B * din) return;
    const int b = t / din, i = t - b * din;
    float g = 0.f;
    for (int u = 0; u < dout; u++) g = fmaf(dz[static_cast<size_t>(b) * dout + u], W[u * din + i], g);
    dzprev[t] = g * gelu_grad(zprev[t]);
}

__global__ void adam_step(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2,
                          float eps, float c1, float c2)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float gi = g[t];
    const float mi = b1 * m[t] + (1.f - b1) * gi;
    const float vi = b2 * v[t] + (1.f - b2) * gi * gi;
    m[t] = mi;
    v[t] = vi;
    p[t] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

inline int blocks(int n) { return (n + 255) / 256; }

// Device buffers of one forward/backward pass over a batch of B samples.
struct Pass {
    int B;
    float *xs, *ys, *z1, *h1, *z2, *h2, *out, *dout, *dz2, *dz1, *loss;
};

cudaError_t pass_alloc(Pass &ps, int B)
{
    ps.B = B;
    size_t n = static_cast<size_t>(B) * (kFeat + 1 + 4 * kHidden + 2 + 2 * kHidden) + 1;
    float *base = nullptr;
    cudaError_t e = cudaMalloc(&base, n * sizeof(float));
    if (e != cudaSuccess) return e;
    float *q = base;
    auto take = [&q](size_t k) {
        float *r = q;
        q += k;
        return r;
    };
    ps.xs = take(static_cast<size_t>(B) * kFeat);
    ps.ys = take(B);
    ps.z1 = take(static_cast<size_t>(B) * kHidden);
    ps.h1 = take(static_cast<size_t>(B) * kHidden);
    ps.z2 = take(static_cast<size_t>(B) * kHidden);
    ps.h2 = take(static_cast<size_t>(B) * kHidden);
    ps.out = take(B);
    ps.dout = take(B);
    ps.dz2 = take(static_cast<size_t>(B) * kHidden);
    ps.dz1 = take(static_cast<size_t>(B) * kHidden);
    ps.loss = take(1);
    return cudaSuccess;
}

// Forward (and, with targets, backward into grad) of one batch.
void run_pass(const Pass &ps, const float *d_x, const float *d_y, const int *d_idx, const float *P, float *G,
              cudaStream_t st)
{
    const int B = ps.B;
    gather_std<<<blocks(B * kFeat), 256, 0, st>>>(d_x, d_y, d_idx, P, ps.xs, ps.ys, B);
    dense_fwd<<<blocks(B * kHidden), 256, 0, st>>>(ps.xs, P + kMlpW1, P + kMlpB1, ps.z1, ps.h1, B, kFeat, kHidden);
    dense_fwd<<<blocks(B * kHidden), 256, 0, st>>>(ps.h1, P + kMlpW2, P + kMlpB2, ps.z2, ps.h2, B, kHidden, kHidden);
    cudaMemsetAsync(ps.loss, 0, sizeof(float), st);
    out_layer<<<blocks(B), 256, 0, st>>>(ps.h2, P + kMlpW3, P + kMlpB3, d_y ? ps.ys : nullptr, ps.out, ps.dout,
                                         ps.loss, B);
    if (!d_y || !G) return;
    out_back<<<blocks(B * kHidden), 256, 0, st>>>(ps.dout, P + kMlpW3, ps.z2, ps.h2, ps.dz2, G + kMlpW3, G + kMlpB3,
                                                  B);
    dense_grad_params<<<blocks(kHidden * kHidden), 256, 0, st>>>(ps.dz2, ps.h1, G + kMlpW2, G + kMlpB2, B, kHidden,
                                                                 kHidden);
    dense_grad_input<<<blocks(B * kHidden), 256, 0, st>>>(ps.dz2, P + kMlpW2, ps.z1, ps.dz1, B, kHidden, kHidden);
    dense_grad_params<<<blocks(kHidden * kFeat), 256, 0, st>>>(ps.dz1, ps.xs, G + kMlpW1, G + kMlpB1, B, kFeat,
                                                               kHidden);
}

}  // namespace

int mlp_grad(const float *h_P, const float *h_x, const float *h_y, int n, float *h_loss, float *h_G)
{
    float *d = nullptr;
    size_t nx = static_cast<size_t>(n) * kFeat;
    cudaError_t e = cudaMalloc(&d, (nx + n + 2 * kMlpFloats) * sizeof(float));
    if (e != cudaSuccess) return static_cast<int>(e);
    float *dx = d, *dy = dx + nx, *dP = dy + n, *dG = dP + kMlpFloats;
    cudaMemcpy(dx, h_x, nx * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(dy, h_y, n * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(dP, h_P, kMlpFloats * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemset(dG, 0, kMlpFloats * sizeof(float));
    Pass ps{};
    e = pass_alloc(ps, n);
    if (e == cudaSuccess) {
        run_pass(ps, dx, dy, nullptr, dP, dG, nullptr);
        cudaMemcpy(h_G, dG, kMlpFloats * sizeof(float), cudaMemcpyDeviceToHost);
        cudaMemcpy(h_loss, ps.loss, sizeof(float), cudaMemcpyDeviceToHost);
        e = cudaGetLastError();
        cudaFree(ps.xs);
    }
    cudaFree(d);
    return static_cast<int>(e);
}

int mlp_predict(const float *h_P, const float *h_x, int n, float *h_out)
{
    float *d = nullptr;
    size_t nx = static_cast<size_t>(n) * kFeat;
    cudaError_t e = cudaMalloc(&d, (nx + kMlpFloats) * sizeof(float));
    if (e != cudaSuccess) return static_cast<int>(e);
    float *dx = d, *dP = dx + nx;
    cudaMemcpy(dx, h_x, nx * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(dP, h_P, kMlpFloats * sizeof(float), cudaMemcpyHostToDevice);
    Pass ps{};
    e = pass_alloc(ps, n);
    if (e == cudaSuccess) {
        run_pass(ps, dx, nullptr, nullptr, dP, nullptr, nullptr);
        std::vector<float> out(n);
        cudaMemcpy(out.data(), ps.out, n * sizeof(float), cudaMemcpyDeviceToHost);
        std::vector<float> P(h_P, h_P + kMlpFloats);
        for (int i = 0; i < n; i++) h_out[i] = out[i] * P[kMlpYSd] + P[kMlpYMu];
        e = cudaGetLastError();
        cudaFree(ps.xs);
    }
    cudaFree(d);
    return static_cast<int>(e);
}

int mlp_train(float *h_P, const float *h_x, const float *h_y, int n, int epochs, int batch, float lr, uint64_t seed,
              float *h_loss_hist)
{
    const int B = std::min(batch, n);
    const int steps_per_epoch = n / B;
    float *d = nullptr;
    size_t nx = static_cast<size_t>(n) * kFeat;
    cudaError_t e = cudaMalloc(&d, (nx + n + 4 * kMlpFloats) * sizeof(float) + static_cast<size_t>(n) * sizeof(int));
    if (e != cudaSuccess) return static_cast<int>(e);
    float *dx = d, *dy = dx + nx, *dP = dy + n, *dG = dP + kMlpFloats, *dm = dG + kMlpFloats, *dv = dm + kMlpFloats;
    int *didx = reinterpret_cast<int *>(dv + kMlpFloats);
    cudaMemcpy(dx, h_x, nx * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(dy, h_y, n * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(dP, h_P, kMlpFloats * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemset(dm, 0, 2 * kMlpFloats * sizeof(float));
    Pass ps{};
    e = pass_alloc(ps, B);
    if (e != cudaSuccess) {
        cudaFree(d);
        return static_cast<int>(e);
    }
    std::mt19937_64 rng(seed);
    std::vector<int> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    const int ntrain = kMlpB3 + 1 - kMlpW1;  // W1 .. b3
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    long long t = 0;
    for (int ep = 0; ep < epochs; ep++) {
        std::shuffle(perm.begin(), perm.end(), rng);
        cudaMemcpy(didx, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice);
        double loss = 0;
        for (int sidx = 0; sidx < steps_per_epoch; sidx++) {
            run_pass(ps, dx, dy, didx + static_cast<size_t>(sidx) * B, dP, dG, nullptr);
            t++;
            const float c1 = 1.f - std::pow(b1, static_cast<float>(t)), c2 = 1.f - std::pow(b2, static_cast<float>(t));
            adam_step<<<blocks(ntrain), 256>>>(dP + kMlpW1, dG + kMlpW1, dm + kMlpW1, dv + kMlpW1, ntrain, lr, b1, b2,
                                               eps, c1, c2);
            float l = 0;
            cudaMemcpy(&l, ps.loss, sizeof(float), cudaMemcpyDeviceToHost);
            loss += l;
        }
        if (h_loss_hist) h_loss_hist[ep] = static_cast<float>(loss / std::max(steps_per_epoch, 1));
    }
    cudaMemcpy(h_P, dP, kMlpFloats * sizeof(float), cudaMemcpyDeviceToHost);
    e = cudaGetLastError();
    cudaFree(ps.xs);
    cudaFree(d);
    return static_cast<int>(e);
}

}  // namespace psg
