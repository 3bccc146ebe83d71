// Training of the learned form's MLP on the GPU with the project's own FP32
// kernels: tiled SGEMM (forward and both backward products), bias + GELU
// and its derivative, the three-part loss with its gradient, column sums for
// the bias gradients, and Adam.  Also the FP32 forward pass used as the
// reference of the BF16 tensor-core inference.
#include "gcurval_gb300_learned.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "gcv_learned.cuh"

using namespace gcv;

namespace {

thread_local std::string g_err_train;

// ---------------------------------------------------------------- kernels
constexpr int GB = 64, GK = 16;  // SGEMM tile: 64 x 64 outputs, K step 16, 256 threads

// C[M x N] = op(A)[M x K] op(B)[K x N], row-major storage:
// op(A)[m][k] = TA ? A[k * lda + m] : A[m * lda + k]; likewise B with TB.
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) k_sgemm(int M, int N, int K, const float* __restrict__ A, int lda,
                                               const float* __restrict__ B, int ldb, float* __restrict__ C, int ldc)
{
    __shared__ float As[GK][GB + 4];
    __shared__ float Bs[GK][GB + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * GB, n0 = blockIdx.x * GB;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += GK) {
        for (int i = threadIdx.x; i < GK * GB; i += 256) {
            const int kk = i / GB, mm = i % GB;
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < K) ? (TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k]) : 0.0f;
            const int n = n0 + mm;
            Bs[kk][mm] = (n < N && k < K) ? (TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n]) : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            float a[4], bb[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                a[i] = As[kk][ty * 4 + i];
                bb[i] = Bs[kk][tx * 4 + i];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], bb[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
            if (m < M && n < N) C[(size_t)m * ldc + n] = acc[i][j];
        }
}

__device__ __forceinline__ float gelu(float x, float& t)
{
    t = tanhf(GELU_C * (x + GELU_A * x * x * x));
    return 0.5f * x * (1.0f + t);
}
__device__ __forceinline__ float gelu_grad(float x)
{
    float t;
    gelu(x, t);
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * GELU_C * (1.0f + 3.0f * GELU_A * x * x);
}

// Z += bias (per column); H = GELU(Z) when act
__global__ void k_bias_act(float* Z, float* H, const float* bias, int n, int cols, int act)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)n * cols; i += (size_t)gridDim.x * blockDim.x) {
        const float z = Z[i] + bias[i % cols];
        Z[i] = z;
        if (act) {
            float t;
            H[i] = gelu(z, t);
        }
    }
}

// dZ = dH * GELU'(Z)
__global__ void k_act_grad(const float* dH, const float* Z, float* dZ, size_t count)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        dZ[i] = dH[i] * gelu_grad(Z[i]);
}

// loss parts (sums over the batch) and dOut = d(mean loss) / d out
__global__ void k_loss(const float* out, const int* depth, const float* share, const float* tg, int n, float* dOut,
                       float* loss3)
{
    float l0 = 0.0f, l1 = 0.0f, l2 = 0.0f;
    const float inv = 1.0f / (float)n;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const float* o = out + (size_t)r * MLP_OUT;
        float* g = dOut + (size_t)r * MLP_OUT;
        // depth: softmax cross-entropy
        float mx = o[0];
        for (int i = 1; i < MLP_DEPTHS; ++i) mx = fmaxf(mx, o[i]);
        float z = 0.0f;
        for (int i = 0; i < MLP_DEPTHS; ++i) z += expf(o[i] - mx);
        const int d = depth[r];
        l0 += logf(z) + mx - o[d];
        for (int i = 0; i < MLP_DEPTHS; ++i) g[i] = (expf(o[i] - mx) / z - (i == d ? 1.0f : 0.0f)) * inv;
        // split: soft cross-entropy against the leaf shares
        mx = o[MLP_O_SPLIT];
        for (int q = 1; q < 4; ++q) mx = fmaxf(mx, o[MLP_O_SPLIT + q]);
        z = 0.0f;
        for (int q = 0; q < 4; ++q) z += expf(o[MLP_O_SPLIT + q] - mx);
        const float lz = logf(z) + mx;
        for (int q = 0; q < 4; ++q) {
            const float s = share[(size_t)r * 4 + q];
            l1 += s * (lz - o[MLP_O_SPLIT + q]);
            g[MLP_O_SPLIT + q] = (expf(o[MLP_O_SPLIT + q] - mx) / z - s) * inv;
        }
        // t guesses: squared error
        for (int j = 0; j < 8; ++j) {
            const float e = o[MLP_O_T + j] - tg[(size_t)r * 8 + j];
            l2 += 0.5f * e * e;
            g[MLP_O_T + j] = e * inv;
        }
        for (int i = MLP_O_T + 8; i < MLP_OUT; ++i) g[i] = 0.0f;
    }
    for (int o = 16; o > 0; o >>= 1) {
        l0 += __shfl_xor_sync(0xffffffffu, l0, o);
        l1 += __shfl_xor_sync(0xffffffffu, l1, o);
        l2 += __shfl_xor_sync(0xffffffffu, l2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(loss3 + 0, l0);
        atomicAdd(loss3 + 1, l1);
        atomicAdd(loss3 + 2, l2);
    }
}

// db[c] = sum over rows of dZ[r][c] (one thread per column, rows strided)
__global__ void k_colsum(const float* dZ, int n, int cols, float* db)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.0f;
    for (int r = 0; r < n; ++r) s += dZ[(size_t)r * cols + c];
    db[c] = s;
}

__global__ void k_adam(float* w, const float* g, float* m, float* v, int count, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

template <bool TA, bool TB>
void sgemm(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc, cudaStream_t st)
{
    dim3 grid((N + GB - 1) / GB, (M + GB - 1) / GB);
    k_sgemm<TA, TB><<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc);
}

unsigned blocks_for(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 152 * 32); }

}  // namespace

struct gcv_mlp_trainer {
    int max_batch = 0;
    cudaStream_t st = nullptr;
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    float *Z[3] = {}, *H[3] = {}, *out = nullptr, *dOut = nullptr, *dA = nullptr, *dB = nullptr, *loss3 = nullptr;
    long long step = 0;
};

namespace {

gcv_status tfail(gcv_status s, const std::string& m)
{
    g_err_train = m;
    return s;
}

#define TCU(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return tfail(GCV_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// forward pass of n rows of X into tr->Z / H / out
void forward(gcv_mlp_trainer* tr, const float* X, int n)
{
    const float* in = X;
    int fan = MLP_IN;
    const int offW[3] = {MLP_OFF_W1, MLP_OFF_W2, MLP_OFF_W3}, offB[3] = {MLP_OFF_B1, MLP_OFF_B2, MLP_OFF_B3};
    for (int l = 0; l < 3; ++l) {
        sgemm<false, false>(n, MLP_H, fan, in, fan, tr->w + offW[l], MLP_H, tr->Z[l], MLP_H, tr->st);
        k_bias_act<<<blocks_for((size_t)n * MLP_H), 256, 0, tr->st>>>(tr->Z[l], tr->H[l], tr->w + offB[l], n, MLP_H, 1);
        in = tr->H[l];
        fan = MLP_H;
    }
    sgemm<false, false>(n, MLP_OUT, MLP_H, in, MLP_H, tr->w + MLP_OFF_W4, MLP_OUT, tr->out, MLP_OUT, tr->st);
    k_bias_act<<<blocks_for((size_t)n * MLP_OUT), 256, 0, tr->st>>>(tr->out, nullptr, tr->w + MLP_OFF_B4, n, MLP_OUT, 0);
}

// loss and gradients of the mean loss into tr->g
void backward(gcv_mlp_trainer* tr, const float* X, const int* depth, const float* share, const float* tg, int n)
{
    cudaMemsetAsync(tr->loss3, 0, 3 * sizeof(float), tr->st);
    k_loss<<<blocks_for((size_t)n), 256, 0, tr->st>>>(tr->out, depth, share, tg, n, tr->dOut, tr->loss3);
    // output layer
    sgemm<true, false>(MLP_H, MLP_OUT, n, tr->H[2], MLP_H, tr->dOut, MLP_OUT, tr->g + MLP_OFF_W4, MLP_OUT, tr->st);
    k_colsum<<<1, 64, 0, tr->st>>>(tr->dOut, n, MLP_OUT, tr->g + MLP_OFF_B4);
    sgemm<false, true>(n, MLP_H, MLP_OUT, tr->dOut, MLP_OUT, tr->w + MLP_OFF_W4, MLP_OUT, tr->dA, MLP_H, tr->st);
    const int offW[3] = {MLP_OFF_W1, MLP_OFF_W2, MLP_OFF_W3}, offB[3] = {MLP_OFF_B1, MLP_OFF_B2, MLP_OFF_B3};
    for (int l = 2; l >= 0; --l) {
        // dA = dH of layer l -> dB = dZ
        k_act_grad<<<blocks_for((size_t)n * MLP_H), 256, 0, tr->st>>>(tr->dA, tr->Z[l], tr->dB, (size_t)n * MLP_H);
        const float* in = l ? tr->H[l - 1] : X;
        const int fan = l ? MLP_H : MLP_IN;
        sgemm<true, false>(fan, MLP_H, n, in, fan, tr->dB, MLP_H, tr->g + offW[l], MLP_H, tr->st);
        k_colsum<<<1, MLP_H, 0, tr->st>>>(tr->dB, n, MLP_H, tr->g + offB[l]);
        if (l) sgemm<false, true>(n, MLP_H, MLP_H, tr->dB, MLP_H, tr->w + offW[l], MLP_H, tr->dA, MLP_H, tr->st);
    }
}

}  // namespace

extern "C" {

const char* gcv_mlp_last_error(void) { return g_err_train.c_str(); }

int gcv_mlp_param_count(void) { return MLP_NPARAM; }

gcv_status gcv_mlp_trainer_create(gcv_mlp_trainer** out, int max_batch, unsigned long long seed)
{
    if (!out || max_batch < 1) return tfail(GCV_ERR_INVALID, "bad trainer arguments");
    *out = nullptr;
    gcv_mlp_trainer* tr = new gcv_mlp_trainer();
    tr->max_batch = max_batch;
    const size_t P = MLP_NPARAM * sizeof(float);
    const size_t A = (size_t)max_batch * MLP_H * sizeof(float), O = (size_t)max_batch * MLP_OUT * sizeof(float);
    cudaError_t e = cudaSuccess;
    float** bufs[] = {&tr->w, &tr->g, &tr->m, &tr->v};
    for (float** b : bufs)
        if (e == cudaSuccess) e = cudaMalloc(b, P);
    for (int l = 0; l < 3 && e == cudaSuccess; ++l) {
        e = cudaMalloc(&tr->Z[l], A);
        if (e == cudaSuccess) e = cudaMalloc(&tr->H[l], A);
    }
    if (e == cudaSuccess) e = cudaMalloc(&tr->out, O);
    if (e == cudaSuccess) e = cudaMalloc(&tr->dOut, O);
    if (e == cudaSuccess) e = cudaMalloc(&tr->dA, A);
    if (e == cudaSuccess) e = cudaMalloc(&tr->dB, A);
    if (e == cudaSuccess) e = cudaMalloc(&tr->loss3, 3 * sizeof(float));
    if (e != cudaSuccess) {
        gcv_mlp_trainer_destroy(tr);
        return tfail(GCV_ERR_OUT_OF_MEMORY, std::string("trainer buffers: ") + cudaGetErrorString(e));
    }
    // He initialisation (normal, variance 2 / fan_in), zero biases
    std::vector<float> h(MLP_NPARAM, 0.0f);
    std::mt19937_64 rng(seed);
    auto init = [&](int off, int fan_in, int count) {
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / fan_in));
        for (int i = 0; i < count; ++i) h[(size_t)off + i] = nd(rng);
    };
    init(MLP_OFF_W1, MLP_IN, MLP_IN * MLP_H);
    init(MLP_OFF_W2, MLP_H, MLP_H * MLP_H);
    init(MLP_OFF_W3, MLP_H, MLP_H * MLP_H);
    init(MLP_OFF_W4, MLP_H, MLP_H * MLP_OUT);
    if (cudaMemcpy(tr->w, h.data(), P, cudaMemcpyHostToDevice) != cudaSuccess || cudaMemset(tr->m, 0, P) != cudaSuccess ||
        cudaMemset(tr->v, 0, P) != cudaSuccess) {
        gcv_mlp_trainer_destroy(tr);
        return tfail(GCV_ERR_CUDA, "trainer initialisation");
    }
    *out = tr;
    return GCV_OK;
}

gcv_status gcv_mlp_trainer_destroy(gcv_mlp_trainer* tr)
{
    if (!tr) return GCV_OK;
    float* bufs[] = {tr->w, tr->g, tr->m, tr->v, tr->Z[0], tr->Z[1], tr->Z[2], tr->H[0], tr->H[1], tr->H[2],
                     tr->out, tr->dOut, tr->dA, tr->dB, tr->loss3};
    for (float* b : bufs)
        if (b) cudaFree(b);
    delete tr;
    return GCV_OK;
}

gcv_status gcv_mlp_trainer_set_weights(gcv_mlp_trainer* tr, const float* host_w)
{
    if (!tr || !host_w) return tfail(GCV_ERR_INVALID, "NULL argument");
    TCU(cudaMemcpy(tr->w, host_w, MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    return GCV_OK;
}

gcv_status gcv_mlp_trainer_get_weights(gcv_mlp_trainer* tr, float* host_w)
{
    if (!tr || !host_w) return tfail(GCV_ERR_INVALID, "NULL argument");
    TCU(cudaMemcpy(host_w, tr->w, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return GCV_OK;
}

gcv_status gcv_mlp_trainer_forward(gcv_mlp_trainer* tr, const float* d_X, int n, float* d_out)
{
    if (!tr || !d_X || !d_out || n < 0 || n > tr->max_batch) return tfail(GCV_ERR_INVALID, "bad forward arguments");
    if (n == 0) return GCV_OK;
    forward(tr, d_X, n);
    TCU(cudaMemcpyAsync(d_out, tr->out, (size_t)n * MLP_OUT * sizeof(float), cudaMemcpyDeviceToDevice, tr->st));
    TCU(cudaStreamSynchronize(tr->st));
    TCU(cudaGetLastError());
    return GCV_OK;
}

gcv_status gcv_mlp_trainer_gradients(gcv_mlp_trainer* tr, const float* d_X, const int* d_depth, const float* d_share,
                                     const float* d_tguess, int n, float* host_grad, float* host_loss3)
{
    if (!tr || !d_X || !d_depth || !d_share || !d_tguess || n < 1 || n > tr->max_batch)
        return tfail(GCV_ERR_INVALID, "bad gradient arguments");
    forward(tr, d_X, n);
    backward(tr, d_X, d_depth, d_share, d_tguess, n);
    TCU(cudaStreamSynchronize(tr->st));
    TCU(cudaGetLastError());
    if (host_grad) TCU(cudaMemcpy(host_grad, tr->g, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    if (host_loss3) {
        TCU(cudaMemcpy(host_loss3, tr->loss3, 3 * sizeof(float), cudaMemcpyDeviceToHost));
        for (int i = 0; i < 3; ++i) host_loss3[i] /= (float)n;
    }
    return GCV_OK;
}

gcv_status gcv_mlp_trainer_step(gcv_mlp_trainer* tr, const float* d_X, const int* d_depth, const float* d_share,
                                const float* d_tguess, int n, float lr, float* host_loss3)
{
    gcv_status s = gcv_mlp_trainer_gradients(tr, d_X, d_depth, d_share, d_tguess, n, nullptr, host_loss3);
    if (s != GCV_OK) return s;
    tr->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)tr->step), c2 = 1.0f - std::pow(b2, (float)tr->step);
    k_adam<<<blocks_for(MLP_NPARAM), 256, 0, tr->st>>>(tr->w, tr->g, tr->m, tr->v, MLP_NPARAM, lr, b1, b2, 1e-8f, c1, c2);
    TCU(cudaGetLastError());
    return GCV_OK;
}

}  // extern "C"
