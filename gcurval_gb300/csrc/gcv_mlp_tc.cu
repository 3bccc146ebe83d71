// BF16 tensor-core inference of the learned form's MLP (tcgen05, sm_103a).
//
// One CTA = four warpgroups; each warpgroup runs its own tiles of 128
// intervals (M = 128 rows, one row per thread and TMEM lane):
//   features (bf16 rows written by the set-up kernels, or FP32 rows for the
//   raw-output entry point) -> bf16 tile X [128 x 16]
//   D = X W1        1 x tcgen05.mma (K = 16), D in TMEM (128 lanes x 128 cols, FP32)
//   H1 = 2 GELU(D + b1) -> bf16 tile [128 x 128] in shared memory (the
//        factor 2 is taken back by W2, W3, W4 stored halved: exact in bf16)
//   D = H1 W2, H2, D = H2 W3, H3: 8 MMAs each (K = 128 in steps of 16)
//   D = H3 W4 (N = 32): outputs -> start depths of the length walk (or raw)
// The transposed weights W^T (N x K) stay in shared memory for the whole
// kernel; operands use the no-swizzle K-major core-matrix layout (8 rows x
// 16 bytes per core matrix; LBO = 128 B between core matrices along K,
// SBO between 8-row groups).  One thread per warpgroup issues the MMAs and
// commits them to the warpgroup's mbarrier; every wait is bounded and a
// timeout is reported through an error word, after which the kernel still
// releases its tensor memory.
#include "gcurval_gb300_learned.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "gcv_learned.cuh"

namespace gcv {

namespace {

// byte offsets of the weight image (identical in global and shared memory)
constexpr int WB_W4 = 0;                                // W4^T [32][128]
constexpr int WB_W1 = WB_W4 + MLP_OUT * MLP_H * 2;      // W1^T [128][16]
constexpr int WB_W2 = WB_W1 + MLP_H * MLP_IN * 2;       // W2^T [128][128]
constexpr int WB_W3 = WB_W2 + MLP_H * MLP_H * 2;        // W3^T [128][128]
constexpr int WB_B4 = WB_W3 + MLP_H * MLP_H * 2;        // b4 (32), FP32
constexpr int WB_BH = WB_B4 + MLP_OUT * 4;              // b1, b2, b3 (128 each), bf16 pairs
constexpr int WB_BYTES = WB_BH + 3 * MLP_H * 2;
constexpr int NWG = 4;                                  // warpgroups per CTA
constexpr int SM_X = (WB_BYTES + 127) / 128 * 128;      // NWG X tiles [128][16] bf16
constexpr int X_BYTES = 128 * MLP_IN * 2;
constexpr int SM_A = SM_X + NWG * X_BYTES;              // NWG H tiles [128][128] bf16
constexpr int A_BYTES = 128 * MLP_H * 2;
constexpr int SM_BAR = SM_A + NWG * A_BYTES;            // NWG mbarriers, the TMEM address
constexpr int SM_BYTES = SM_BAR + 8 * NWG + 16;
constexpr int TC_THREADS = 128 * NWG;
constexpr int TMEM_COLS = 128 * NWG;                    // 128 FP32 columns per warpgroup
constexpr long long WAIT_LIMIT = 1ll << 24;

// canonical no-swizzle K-major offset of element (row, k) in a tile with K columns
__host__ __device__ constexpr int kmaj_off(int row, int k, int K)
{
    return (row >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, LBO, SBO (bytes, >> 4), version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: D F32, A and B BF16, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    for (long long i = 0; i < WAIT_LIMIT; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void wg_sync(int wg) { asm volatile("bar.sync %0, 128;" ::"r"(1 + wg) : "memory"); }
// barrier of the warpgroup that also ANDs a flag over its 128 threads
__device__ __forceinline__ bool wg_all(int wg, bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(1 + wg)
        : "memory");
    return r != 0;
}

// N consecutive FP32 columns of this thread's TMEM lane (load and wait in one
// statement: the destination registers are written asynchronously until the
// wait, so no compiler-inserted copy may touch them in between)
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t* r)
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r)
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
}

// Twice the GELU of two accumulator values plus their bias, in packed bf16x2
// arithmetic (the activations are stored as bf16 for the next layer
// anyway): with x = acc + b, 2 GELU(x) = x (1 + tanh(x (c + c a x^2))),
// c = sqrt(2/pi), a = 0.044715.  Six instructions per pair.
__device__ __forceinline__ uint32_t gelu2_bf16x2(float x0, float x1, uint32_t b)
{
    uint32_t x, r;
    asm("cvt.rn.bf16x2.f32 %0, %2, %1;" : "=r"(x) : "f"(x0), "f"(x1));
    asm("{\n\t.reg .b32 xb, x2, y, u, t;\n\t"
        "add.rn.bf16x2 xb, %1, %2;\n\t"      // + bias
        "mul.rn.bf16x2 x2, xb, xb;\n\t"
        "fma.rn.bf16x2 y, x2, %3, %4;\n\t"   // c a x^2 + c
        "mul.rn.bf16x2 u, xb, y;\n\t"
        "tanh.approx.bf16x2 t, u;\n\t"
        "fma.rn.bf16x2 %0, t, xb, xb;\n\t}\n"
        : "=r"(r)
        : "r"(x), "r"(b), "r"(0x3D123D12u), "r"(0x3F4C3F4Cu));
    return r;
}

// 8 values -> 8 bf16 at a 16-byte aligned shared address
__device__ __forceinline__ void st_bf16x8(uint8_t* p, const float* v)
{
    __nv_bfloat162 h[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    *reinterpret_cast<uint4*>(p) = *reinterpret_cast<const uint4*>(h);
}

struct TcArgs {
    const float* feat;  // n rows of MLP_IN features (FP32), or
    const uint4* feat16;  // n rows of MLP_IN bf16 features (two uint4 per row)
    int64_t n;
    // product path: start depths of intervals list[row0 + row] (list NULL: row0 + row)
    const int* list;
    int64_t row0;
    int max_depth;
    uint32_t* starts;
    // test path: raw outputs
    float* out;
    const uint8_t* w;  // weight image (WB_BYTES)
    unsigned* err;
};

// STARTS: start depths out; else the raw outputs.  BF16IN: the rows come as
// bf16 (feat16) and go to the operand tile as they are.
template <bool STARTS, bool BF16IN>
__global__ void __launch_bounds__(TC_THREADS, 1) k_mlp_tc(TcArgs A)
{
    extern __shared__ __align__(1024) uint8_t sm[];
    const int tid = threadIdx.x, wg = tid >> 7, t = tid & 127, warp = tid >> 5;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + SM_BAR);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + SM_BAR + 8 * NWG);
    const float* bias4 = reinterpret_cast<const float*>(sm + WB_B4);
    const uint32_t* bias_h = reinterpret_cast<const uint32_t*>(sm + WB_BH);

    // weights into shared memory
    for (int i = tid; i < WB_BYTES / 16; i += TC_THREADS)
        reinterpret_cast<uint4*>(sm)[i] = reinterpret_cast<const uint4*>(A.w)[i];
    if (tid == 0) {
        for (int i = 0; i < NWG; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[i])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t tcol = tmem + 128u * wg;                         // this warpgroup's columns
    const uint32_t tlane = tcol + ((uint32_t)(32 * (warp & 3)) << 16);  // this warp's lanes
    uint8_t* X = sm + SM_X + wg * X_BYTES;
    uint8_t* H = sm + SM_A + wg * A_BYTES;
    const uint32_t bar = smem_u32(&bars[wg]);
    uint32_t parity = 0;
    bool ok = true;

    const int64_t tiles = (A.n + 127) / 128;
    float4 nxt[BF16IN ? 1 : MLP_IN / 4];
    uint4 nxt16[2];
    auto load_rows = [&](int64_t tl) {
        const int64_t r = tl * 128 + t;
        if constexpr (BF16IN) {
            nxt16[0] = r < A.n ? A.feat16[2 * r] : make_uint4(0u, 0u, 0u, 0u);
            nxt16[1] = r < A.n ? A.feat16[2 * r + 1] : make_uint4(0u, 0u, 0u, 0u);
        } else {
            const float4* src = reinterpret_cast<const float4*>(A.feat + r * MLP_IN);
#pragma unroll
            for (int i = 0; i < MLP_IN / 4; ++i) nxt[i] = r < A.n ? src[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    };
    load_rows((int64_t)blockIdx.x * NWG + wg);
    for (int64_t tile = (int64_t)blockIdx.x * NWG + wg; tile < tiles && ok; tile += (int64_t)gridDim.x * NWG) {
        const int64_t row = tile * 128 + t;
        const bool live = row < A.n;
        // the interval this row's start depths go to, fetched now: its load
        // latency then hides behind the four layers
        int64_t out_s = 0;
        if constexpr (STARTS) out_s = live ? (A.list ? (int64_t)A.list[A.row0 + row] : A.row0 + row) : 0;
        // ---- features -> X (bf16, K-major core matrices, K = 16); the next
        // tile's rows are fetched now and used one iteration later
        if constexpr (BF16IN) {
            const uint4 x0 = nxt16[0], x1 = nxt16[1];
            load_rows(tile + (int64_t)gridDim.x * NWG);
            *reinterpret_cast<uint4*>(X + kmaj_off(t, 0, MLP_IN)) = x0;
            *reinterpret_cast<uint4*>(X + kmaj_off(t, 8, MLP_IN)) = x1;
        } else {
            float f[MLP_IN];
#pragma unroll
            for (int i = 0; i < MLP_IN / 4; ++i) {
                f[4 * i] = nxt[i].x;
                f[4 * i + 1] = nxt[i].y;
                f[4 * i + 2] = nxt[i].z;
                f[4 * i + 3] = nxt[i].w;
            }
            load_rows(tile + (int64_t)gridDim.x * NWG);
            st_bf16x8(X + kmaj_off(t, 0, MLP_IN), f);
            st_bf16x8(X + kmaj_off(t, 8, MLP_IN), f + 8);
        }
        fence_async_smem();
        fence_before();
        wg_sync(wg);
        fence_after();
        // ---- four layers
        for (int layer = 0; layer < 4 && ok; ++layer) {
            const int N = layer == 3 ? MLP_OUT : MLP_H;
            if (t == 0) {
                const uint32_t idesc = idesc_bf16(128, N);
                const uint32_t wbase = smem_u32(sm) + (layer == 0 ? WB_W1 : layer == 1 ? WB_W2 : layer == 2 ? WB_W3 : WB_W4);
                if (layer == 0) {
                    mma_bf16(tcol, sdesc(smem_u32(X), 128, (MLP_IN / 8) * 128), sdesc(wbase, 128, (MLP_IN / 8) * 128),
                             idesc, 0u);
                } else {
#pragma unroll 1
                    for (int ks = 0; ks < MLP_H / 16; ++ks)  // K steps of 16 = two core matrices
                        mma_bf16(tcol, sdesc(smem_u32(H) + ks * 256, 128, (MLP_H / 8) * 128),
                                 sdesc(wbase + ks * 256, 128, (MLP_H / 8) * 128), idesc, ks > 0 ? 1u : 0u);
                }
                mma_commit(bar);
            }
            ok = wg_all(wg, mbar_wait(bar, parity));  // uniform over the warpgroup
            parity ^= 1u;
            fence_after();
            if (!ok) break;
            if (layer < 3) {
                // epilogue: bias + GELU -> bf16 H (the MMAs reading H have completed)
                const uint32_t* bl = bias_h + layer * (MLP_H / 2);
                // 64 columns per TMEM load (two loads per layer)
#pragma unroll 1
                for (int c2 = 0; c2 < MLP_H / 64; ++c2) {
                    uint32_t v[64];
                    tmem_ld64(tlane + 64u * c2, v);
#pragma unroll
                    for (int half = 0; half < 2; ++half) {
                        const int c = 2 * c2 + half;
                        uint32_t h[16];
#pragma unroll
                        for (int i = 0; i < 16; ++i)
                            h[i] = gelu2_bf16x2(__uint_as_float(v[32 * half + 2 * i]),
                                                __uint_as_float(v[32 * half + 2 * i + 1]), bl[16 * c + i]);
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            *reinterpret_cast<uint4*>(H + kmaj_off(t, 32 * c + 8 * q, MLP_H)) =
                                make_uint4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
                    }
                }
                fence_async_smem();
                fence_before();
                wg_sync(wg);
                fence_after();
            } else {
                uint32_t r[32];
                tmem_ld32(tlane, r);
                float o[32];
#pragma unroll
                for (int i = 0; i < 32; ++i) o[i] = __uint_as_float(r[i]) + bias4[i];
                if (live) {
                    if constexpr (STARTS) {
                        A.starts[out_s] = quarter_depths(o, A.max_depth);
                    } else {
#pragma unroll
                        for (int i = 0; i < 32; ++i) A.out[row * MLP_OUT + i] = o[i];
                    }
                }
                // TMEM columns are reused by the next tile's first MMA
                fence_before();
                wg_sync(wg);
                fence_after();
            }
        }
    }
    if (!ok && t == 0) atomicOr(A.err, 1u);
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

int sm_count_tc()
{
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <bool STARTS, bool BF16IN = false>
cudaError_t launch_tc(const TcArgs& A, cudaStream_t stream)
{
    cudaError_t e = cudaFuncSetAttribute(k_mlp_tc<STARTS, BF16IN>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_BYTES);
    if (e != cudaSuccess) return e;
    const int64_t tiles = (A.n + 127) / 128;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((tiles + NWG - 1) / NWG, sm_count_tc()));
    k_mlp_tc<STARTS, BF16IN><<<grid, TC_THREADS, SM_BYTES, stream>>>(A);
    return cudaGetLastError();
}

// host: packed FP32 weights -> the bf16 weight image
std::vector<uint8_t> weight_image(const float* w)
{
    std::vector<uint8_t> img(WB_BYTES, 0);
    // W[k][n] (K x N) -> W^T core-matrix tile, times `scale` (1 or 1/2: exact)
    auto put = [&](int base, int N, int K, int off, float scale) {
        for (int n = 0; n < N; ++n)
            for (int k = 0; k < K; ++k) {
                const __nv_bfloat16 h = __float2bfloat16_rn(w[off + k * N + n] * scale);
                std::memcpy(&img[(size_t)base + kmaj_off(n, k, K)], &h, 2);
            }
    };
    // the hidden activations are stored as 2 GELU: the layers reading them
    // take the 1/2
    put(WB_W1, MLP_H, MLP_IN, MLP_OFF_W1, 1.0f);
    put(WB_W2, MLP_H, MLP_H, MLP_OFF_W2, 0.5f);
    put(WB_W3, MLP_H, MLP_H, MLP_OFF_W3, 0.5f);
    put(WB_W4, MLP_OUT, MLP_H, MLP_OFF_W4, 0.5f);
    std::memcpy(&img[WB_B4], w + MLP_OFF_B4, MLP_OUT * 4);
    const int boff[3] = {MLP_OFF_B1, MLP_OFF_B2, MLP_OFF_B3};
    for (int l = 0; l < 3; ++l)
        for (int i = 0; i < MLP_H; ++i) {
            const __nv_bfloat16 h = __float2bfloat16_rn(w[boff[l] + i]);
            std::memcpy(&img[(size_t)WB_BH + (size_t)(l * MLP_H + i) * 2], &h, 2);
        }
    return img;
}

}  // namespace

size_t mlp_dev_bytes() { return WB_BYTES; }

cudaError_t mlp_upload_bf16(const float* host_w, void** w_dev)
{
    const std::vector<uint8_t> img = weight_image(host_w);
    cudaError_t e = cudaMalloc(w_dev, WB_BYTES + sizeof(unsigned));
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(*w_dev, img.data(), WB_BYTES, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset((uint8_t*)*w_dev + WB_BYTES, 0, sizeof(unsigned));
    return e;
}

cudaError_t mlp_starts_launch_bf16(const uint4* feat16, const int* list, int64_t n, const void* w_dev, int max_depth,
                                   uint32_t* starts, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    TcArgs A{};
    A.feat16 = feat16;
    A.n = n;
    A.list = list;
    A.row0 = 0;
    A.max_depth = max_depth;
    A.starts = starts;
    A.w = (const uint8_t*)w_dev;
    A.err = (unsigned*)((uint8_t*)w_dev + WB_BYTES);
    return launch_tc<true, true>(A, stream);
}

}  // namespace gcv

extern "C" gcv_status gcv_mlp_infer(const float* host_weights, const float* d_features, int n, float* d_out)
{
    using namespace gcv;
    if (!host_weights || (n > 0 && (!d_features || !d_out)) || n < 0) return GCV_ERR_INVALID;
    if (reinterpret_cast<uintptr_t>(d_features) % 16) return GCV_ERR_INVALID;  // rows are read as float4
    if (n == 0) return GCV_OK;
    void* w = nullptr;
    cudaError_t e = mlp_upload_bf16(host_weights, &w);
    if (e == cudaSuccess) {
        TcArgs A{};
        A.feat = d_features;
        A.out = d_out;
        A.n = n;
        A.w = (const uint8_t*)w;
        A.err = (unsigned*)((uint8_t*)w + WB_BYTES);
        e = launch_tc<false>(A, nullptr);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    unsigned err = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&err, (uint8_t*)w + WB_BYTES, sizeof(err), cudaMemcpyDeviceToHost);
    if (w) cudaFree(w);
    if (e != cudaSuccess) return GCV_ERR_CUDA;
    return err ? GCV_ERR_TIMEOUT : GCV_OK;
}
