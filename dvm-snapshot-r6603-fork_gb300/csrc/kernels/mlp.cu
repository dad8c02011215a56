// The tuner's learned cost model: a 3-layer FP32 MLP (D -> 128 -> 128 -> 1,
// ReLU), trained with hand-written forward, backward and Adam kernels.
//
// Parameters are one packed FP32 vector: W1[H][D], b1[H], W2[H][H], b2[H],
// W3[H], b3.  Training minimises the mean squared error of the predicted
// log-time.  Every sum runs in a fixed order inside one thread (no atomics),
// so a training run is deterministic; the backward pass is checked against a
// float64 numpy restatement (oracle/mlp_ref.py).
//
// The matrices are small (H = 128, D = 24), so these are FP32 CUDA-core tiles:
// the model costs microseconds next to the loops it ranks.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../../include/dvmh_gb.h"
#include "../../../include/dvmh_gb_kernels.h"

namespace {

constexpr int D = DVMHGB_TUNE_NF, H = 128;
constexpr long OFF_W1 = 0, OFF_B1 = OFF_W1 + (long)H * D, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + (long)H * H,
               OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H, NPARAM = OFF_B3 + 1;
constexpr int T = 32;  // GEMM tile

// Y[n][o] = act(X[n][i] . W[o][i]^T + b[o]);  one thread = 4 rows of one column
__global__ void __launch_bounds__(256) kLinear(const float *X, const float *W, const float *b, float *Y, long n,
                                               int in, int out, int relu) {
    __shared__ float As[T][T + 1], Bs[T][T + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const long r0 = (long)blockIdx.y * T;
    const int c0 = blockIdx.x * T;
    float acc[4] = {0, 0, 0, 0};
    for (int k0 = 0; k0 < in; k0 += T) {
        for (int r = ty; r < T; r += 8) {
            long row = r0 + r;
            As[r][tx] = (row < n && k0 + tx < in) ? X[row * in + k0 + tx] : 0.0f;
            Bs[r][tx] = (c0 + r < out && k0 + tx < in) ? W[(long)(c0 + r) * in + k0 + tx] : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < T; k++) {
            float bv = Bs[tx][k];
#pragma unroll
            for (int q = 0; q < 4; q++) acc[q] = fmaf(As[ty + 8 * q][k], bv, acc[q]);
        }
        __syncthreads();
    }
    const int col = c0 + tx;
    if (col < out)
        for (int q = 0; q < 4; q++) {
            long row = r0 + ty + 8 * q;
            if (row < n) {
                float v = acc[q] + b[col];
                Y[row * out + col] = relu ? fmaxf(v, 0.0f) : v;
            }
        }
}

// dX[n][i] = dY[n][o] . W[o][i]
__global__ void __launch_bounds__(256) kBackData(const float *dY, const float *W, float *dX, long n, int in,
                                                 int out) {
    __shared__ float As[T][T + 1], Bs[T][T + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const long r0 = (long)blockIdx.y * T;
    const int c0 = blockIdx.x * T;
    float acc[4] = {0, 0, 0, 0};
    for (int k0 = 0; k0 < out; k0 += T) {
        for (int r = ty; r < T; r += 8) {
            long row = r0 + r;
            As[r][tx] = (row < n && k0 + tx < out) ? dY[row * out + k0 + tx] : 0.0f;
            Bs[r][tx] = (k0 + r < out && c0 + tx < in) ? W[(long)(k0 + r) * in + c0 + tx] : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < T; k++) {
            float bv = Bs[k][tx];
#pragma unroll
            for (int q = 0; q < 4; q++) acc[q] = fmaf(As[ty + 8 * q][k], bv, acc[q]);
        }
        __syncthreads();
    }
    const int col = c0 + tx;
    if (col < in)
        for (int q = 0; q < 4; q++) {
            long row = r0 + ty + 8 * q;
            if (row < n) dX[row * in + col] = acc[q];
        }
}

// dW[o][i] = sum_n dY[n][o] X[n][i], db[o] = sum_n dY[n][o]; rows summed in order
__global__ void __launch_bounds__(256) kBackWeight(const float *dY, const float *X, float *dW, float *db, long n,
                                                   int in, int out) {
    __shared__ float Ys[T][T + 1], Xs[T][T + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int o0 = blockIdx.y * T, i0 = blockIdx.x * T;
    float acc[4] = {0, 0, 0, 0}, bacc = 0;
    for (long n0 = 0; n0 < n; n0 += T) {
        for (int r = ty; r < T; r += 8) {
            long row = n0 + r;
            Ys[r][tx] = (row < n && o0 + tx < out) ? dY[row * out + o0 + tx] : 0.0f;
            Xs[r][tx] = (row < n && i0 + tx < in) ? X[row * in + i0 + tx] : 0.0f;
        }
        __syncthreads();
        for (int k = 0; k < T; k++) {
            float xv = Xs[k][tx];
#pragma unroll
            for (int q = 0; q < 4; q++) acc[q] = fmaf(Ys[k][ty + 8 * q], xv, acc[q]);
        }
        if (blockIdx.x == 0 && ty == 0)
            for (int k = 0; k < T; k++) bacc += Ys[k][tx];
        __syncthreads();
    }
    for (int q = 0; q < 4; q++) {
        int o = o0 + ty + 8 * q, i = i0 + tx;
        if (o < out && i < in) dW[(long)o * in + i] = acc[q];
    }
    if (blockIdx.x == 0 && ty == 0 && o0 + tx < out) db[o0 + tx] = bacc;
}

__global__ void kReluMask(float *dZ, const float *A, long cnt) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cnt; i += (long)gridDim.x * blockDim.x)
        if (A[i] <= 0.0f) dZ[i] = 0.0f;
}

// d = 2 (pred - y) / n; per-block partial sums of (pred - y)^2 in fixed order
__global__ void kMse(const float *pred, const float *y, long n, float *d, float *part) {
    __shared__ float sh[256];
    float s = 0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float e = pred[i] - y[i];
        d[i] = 2.0f * e / (float)n;
        s += e * e;
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void kLossFinish(const float *part, int nb, long n, float *loss) {
    float s = 0;
    for (int i = 0; i < nb; i++) s += part[i];
    *loss = s / (float)n;
}

__global__ void kAdam(float *p, const float *g, float *m, float *v, long cnt, float lr, float b1, float b2, float eps,
                      float c1, float c2) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cnt; i += (long)gridDim.x * blockDim.x) {
        float mi = b1 * m[i] + (1 - b1) * g[i];
        float vi = b2 * v[i] + (1 - b2) * g[i] * g[i];
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// He-style uniform initialisation from a counter-based hash (splitmix64)
__global__ void kInit(float *p, unsigned long long seed) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < NPARAM; i += (long)gridDim.x * blockDim.x) {
        unsigned long long z = seed + (unsigned long long)(i + 1) * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        float u = (float)(z >> 40) * (1.0f / 16777216.0f) * 2.0f - 1.0f;
        float scale = i < OFF_B1 ? sqrtf(6.0f / D) : (i < OFF_W2 ? 0.0f : (i < OFF_B2 ? sqrtf(6.0f / H)
                      : (i < OFF_W3 ? 0.0f : (i < OFF_B3 ? sqrtf(3.0f / H) : 0.0f))));
        p[i] = u * scale;
    }
}

dim3 gridFor(long rows, int cols) { return dim3((unsigned)((cols + T - 1) / T), (unsigned)((rows + T - 1) / T)); }

}  // namespace

extern "C" {

long dvmhgb_mlp_nparams(void) { return NPARAM; }

// work floats for n rows: H1, H2, dZ2, dZ1 (n x H each), pred and its gradient, loss partials
long dvmhgb_mlp_work_floats(long n) { return 4 * n * H + 2 * n + 1024; }

int dvmhgb_mlp_init(float *params, unsigned long long seed, void *stream) {
    if (!params) return -1;
    kInit<<<64, 256, 0, (cudaStream_t)stream>>>(params, seed);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int dvmhgb_mlp_forward(const float *P, const float *X, long n, float *pred, float *work, void *stream) {
    if (!P || !X || !pred || !work || n < 1) return -1;
    cudaStream_t s = (cudaStream_t)stream;
    float *H1 = work, *H2 = work + n * H;
    dim3 blk(T, 8);
    kLinear<<<gridFor(n, H), blk, 0, s>>>(X, P + OFF_W1, P + OFF_B1, H1, n, D, H, 1);
    kLinear<<<gridFor(n, H), blk, 0, s>>>(H1, P + OFF_W2, P + OFF_B2, H2, n, H, H, 1);
    kLinear<<<gridFor(n, 1), blk, 0, s>>>(H2, P + OFF_W3, P + OFF_B3, pred, n, H, 1, 0);
    dvmhgb_count_launches(3);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// gradient of the mean squared error of the prediction w.r.t. every parameter
int dvmhgb_mlp_loss_grad(const float *P, const float *X, const float *y, long n, float *grad, float *loss,
                         float *work, void *stream) {
    if (!P || !X || !y || !grad || !work || n < 1) return -1;
    cudaStream_t s = (cudaStream_t)stream;
    float *H1 = work, *H2 = work + n * H, *dZ2 = work + 2 * n * H, *dZ1 = work + 3 * n * H;
    float *pred = work + 4 * n * H, *dP = pred + n, *part = dP + n;
    if (dvmhgb_mlp_forward(P, X, n, pred, work, stream) != 0) return -1;
    const int nb = 256;
    kMse<<<nb, 256, 0, s>>>(pred, y, n, dP, part);
    if (loss) kLossFinish<<<1, 1, 0, s>>>(part, nb, n, loss);
    dim3 blk(T, 8);
    // layer 3: pred = H2 . W3 + b3
    kBackWeight<<<dim3((H + T - 1) / T, 1), blk, 0, s>>>(dP, H2, grad + OFF_W3, grad + OFF_B3, n, H, 1);
    kBackData<<<gridFor(n, H), blk, 0, s>>>(dP, P + OFF_W3, dZ2, n, H, 1);
    kReluMask<<<256, 256, 0, s>>>(dZ2, H2, n * H);
    // layer 2
    kBackWeight<<<dim3((H + T - 1) / T, (H + T - 1) / T), blk, 0, s>>>(dZ2, H1, grad + OFF_W2, grad + OFF_B2, n, H, H);
    kBackData<<<gridFor(n, H), blk, 0, s>>>(dZ2, P + OFF_W2, dZ1, n, H, H);
    kReluMask<<<256, 256, 0, s>>>(dZ1, H1, n * H);
    // layer 1
    kBackWeight<<<dim3((D + T - 1) / T, (H + T - 1) / T), blk, 0, s>>>(dZ1, X, grad + OFF_W1, grad + OFF_B1, n, D, H);
    dvmhgb_count_launches(9);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int dvmhgb_mlp_adam(float *P, const float *grad, float *m, float *v, long step, float lr, void *stream) {
    if (!P || !grad || !m || !v || step < 1) return -1;
    const float b1 = 0.9f, b2 = 0.999f;
    float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    kAdam<<<64, 256, 0, (cudaStream_t)stream>>>(P, grad, m, v, NPARAM, lr, b1, b2, 1e-8f, c1, c2);
    dvmhgb_count_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Minibatch Adam on the GPU: X[n][D], y[n] host arrays (rows in the order given,
// batches taken in order every epoch).  Returns 0; params (NPARAM floats) and
// losses (one per epoch: loss of the last batch) written to host memory.
int dvmhgb_mlp_train(const float *X, const float *y, long n, int epochs, long batch, float lr,
                     unsigned long long seed, float *params, float *losses) {
    if (!X || !y || !params || n < 1 || epochs < 1 || batch < 1) return -1;
    cudaStream_t s = nullptr;
    float *dX, *dY, *dP, *dG, *dM, *dV, *work, *dLoss;
    if (batch > n) batch = n;
    size_t ok = 0;
    ok |= cudaMalloc(&dX, sizeof(float) * n * D);
    ok |= cudaMalloc(&dY, sizeof(float) * n);
    ok |= cudaMalloc(&dP, sizeof(float) * NPARAM);
    ok |= cudaMalloc(&dG, sizeof(float) * NPARAM);
    ok |= cudaMalloc(&dM, sizeof(float) * NPARAM);
    ok |= cudaMalloc(&dV, sizeof(float) * NPARAM);
    ok |= cudaMalloc(&work, sizeof(float) * dvmhgb_mlp_work_floats(batch));
    ok |= cudaMalloc(&dLoss, sizeof(float));
    if (ok) return -1;
    cudaMemcpy(dX, X, sizeof(float) * n * D, cudaMemcpyHostToDevice);
    cudaMemcpy(dY, y, sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemset(dM, 0, sizeof(float) * NPARAM);
    cudaMemset(dV, 0, sizeof(float) * NPARAM);
    dvmhgb_mlp_init(dP, seed, s);
    long step = 0;
    for (int ep = 0; ep < epochs; ep++) {
        for (long b0 = 0; b0 < n; b0 += batch) {
            long nb = (b0 + batch <= n) ? batch : n - b0;
            dvmhgb_mlp_loss_grad(dP, dX + b0 * D, dY + b0, nb, dG, dLoss, work, s);
            dvmhgb_mlp_adam(dP, dG, dM, dV, ++step, lr, s);
        }
        if (losses) cudaMemcpy(&losses[ep], dLoss, sizeof(float), cudaMemcpyDeviceToHost);
    }
    cudaMemcpy(params, dP, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost);
    cudaError_t e = cudaGetLastError();
    cudaFree(dX);
    cudaFree(dY);
    cudaFree(dP);
    cudaFree(dG);
    cudaFree(dM);
    cudaFree(dV);
    cudaFree(work);
    cudaFree(dLoss);
    return e == cudaSuccess ? 0 : -1;
}

}  // extern "C"
