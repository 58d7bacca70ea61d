// gy_mlp.cu -- BF16 tensor-core (tcgen05 + TMEM) kernels of the learned Drucker-Prager
// surrogate, and the plain GEMM they are checked against.
#include <algorithm>
#include <cstdint>

#include <cuda_bf16.h>

#include "../../include/graphyt_gpu.h"
#include "gy_kernels.cuh"
#include "gy_tc.cuh"

namespace gy {

// ---------------------------------------------------------------------------------------
// C[M x N] = A[M x K] * B[N x K]^T, BF16 in, FP32 out: one 128-row tile per CTA, the whole K
// staged in shared memory (K <= TC_GEMM_KMAX), one MMA per 16 columns of K.
constexpr int TC_GEMM_KMAX = 256;
constexpr int TC_GEMM_NMAX = 256;
constexpr int TC_GEMM_SMEM = (128 + TC_GEMM_NMAX) * TC_GEMM_KMAX * 2 + 1024;

// copy a R x K row-major bf16 matrix (rows r0..r0+R of a global matrix with leading
// dimension K) into the K-major no-swizzle layout, 16 bytes (8 columns) per copy
__device__ __forceinline__ void stage_kmajor(unsigned char *dst, const uint16_t *src, int R, int K, int rows_valid)
{
    const int chunks = R * (K / 8);
    for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
        const int r = c / (K / 8), kb = c - r * (K / 8);
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (r < rows_valid) v = *reinterpret_cast<const uint4 *>(src + (size_t)r * K + kb * 8);
        *reinterpret_cast<uint4 *>(dst + tc_off(r, kb * 8, K)) = v;
    }
}

__global__ void __launch_bounds__(128) k_tc_gemm(const uint16_t *A, const uint16_t *B, float *C, int M, int N, int K,
                                                 int *status)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    unsigned char *sA = smem;
    unsigned char *sB = smem + 128 * K * 2;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int row0 = blockIdx.x * 128;
    uint32_t ncols = 32;
    while ((int)ncols < N) ncols <<= 1;
    if (warp == 0) tmem_alloc(&tbase, ncols);
    if (tid == 0) {
        mbar_init(&mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    stage_kmajor(sA, A + (size_t)row0 * K, 128, K, min(128, M - row0));
    stage_kmajor(sB, B, N, K, N);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = tbase;
    if (tid == 0) {
        const uint32_t idesc = tc_idesc_bf16(128, N);
        const uint32_t sbo = (uint32_t)(K / 8) * 128;
        for (int j = 0; j < K / 16; j++) {
            const uint64_t ad = tc_sdesc(smem_u32(sA) + 256 * j, 128, sbo);
            const uint64_t bd = tc_sdesc(smem_u32(sB) + 256 * j, 128, sbo);
            tc_mma(tm, ad, bd, idesc, j > 0);
        }
        tc_commit(&mbar);
    }
    // the tensor-memory loads below are warp-collective: every thread takes the same branch
    const bool ok = __syncthreads_and(mbar_wait(&mbar, 0)) != 0;
    tc_fence_after();
    if (ok) {
        const int r = row0 + tid;
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tmem_ld16(tmem_at(tm, 32 * warp, c), v);
            if (r < M)
#pragma unroll
                for (int i = 0; i < 16; i++) C[(size_t)r * N + c + i] = v[i];
        }
    } else if (tid == 0 && status) {
        atomicOr(status, ERR_TC_TIMEOUT);
    }
    tc_fence_before();
    __syncthreads();
    // a wait that gave up leaves the MMAs possibly in flight: wait once more (bounded)
    // before the columns are released
    if (!ok) mbar_wait(&mbar, 0);
    if (warp == 0) tmem_dealloc(tm, ncols);
}

// ---------------------------------------------------------------------------------------
// The surrogate MLP, 16 -> 64 -> 64 -> 7 with SiLU, in one packed FP32 parameter vector
// (gy_mlp_param_count floats, offsets below): weights input-major, y = x W + b.  Inputs and
// outputs are normalised per feature, x_n = (x - mean) / std, y = y_n std + mean.
constexpr int MLP_IN = 16, MLP_H = 64, MLP_OUT = 7, MLP_OUTP = 16;
constexpr int MP_W1 = 0;
constexpr int MP_B1 = MP_W1 + MLP_IN * MLP_H;
constexpr int MP_W2 = MP_B1 + MLP_H;
constexpr int MP_B2 = MP_W2 + MLP_H * MLP_H;
constexpr int MP_W3 = MP_B2 + MLP_H;
constexpr int MP_B3 = MP_W3 + MLP_H * MLP_OUT;
constexpr int MP_IN_MEAN = MP_B3 + MLP_OUT;
constexpr int MP_IN_STD = MP_IN_MEAN + MLP_IN;
constexpr int MP_OUT_MEAN = MP_IN_STD + MLP_IN;
constexpr int MP_OUT_STD = MP_OUT_MEAN + MLP_OUT;
constexpr int MP_COUNT = MP_OUT_STD + MLP_OUT;

__device__ __forceinline__ uint16_t bf16_rn(float x)
{
    return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }

// Shared-memory operands of one 128-row tile: the layer inputs (K-major, written per row by
// the row's thread) and the transposed weights B[n][k] = W[k][n], staged once per CTA.
struct MlpSmem {
    alignas(1024) unsigned char a1[128 * MLP_IN * 2];   // normalised inputs, K = 16
    alignas(1024) unsigned char a2[128 * MLP_H * 2];    // hidden activations, K = 64 (both layers)
    alignas(1024) unsigned char w1[MLP_H * MLP_IN * 2];
    alignas(1024) unsigned char w2[MLP_H * MLP_H * 2];
    alignas(1024) unsigned char w3[MLP_OUTP * MLP_H * 2];
    float b1[MLP_H], b2[MLP_H], b3[MLP_OUTP];
    float in_mean[MLP_IN], in_rstd[MLP_IN], out_mean[MLP_OUTP], out_std[MLP_OUTP];
    uint64_t mbar;
    uint32_t tbase;
};

__device__ void mlp_stage_params(MlpSmem &S, const float *prm)
{
    for (int e = threadIdx.x; e < MLP_H * MLP_IN; e += blockDim.x) {
        const int n = e / MLP_IN, k = e - n * MLP_IN;  // B1[n][k] = W1[k][n]
        *reinterpret_cast<uint16_t *>(S.w1 + tc_off(n, k, MLP_IN)) = bf16_rn(prm[MP_W1 + k * MLP_H + n]);
    }
    for (int e = threadIdx.x; e < MLP_H * MLP_H; e += blockDim.x) {
        const int n = e / MLP_H, k = e - n * MLP_H;
        *reinterpret_cast<uint16_t *>(S.w2 + tc_off(n, k, MLP_H)) = bf16_rn(prm[MP_W2 + k * MLP_H + n]);
    }
    for (int e = threadIdx.x; e < MLP_OUTP * MLP_H; e += blockDim.x) {
        const int n = e / MLP_H, k = e - n * MLP_H;
        const float w = n < MLP_OUT ? prm[MP_W3 + k * MLP_OUT + n] : 0.f;
        *reinterpret_cast<uint16_t *>(S.w3 + tc_off(n, k, MLP_H)) = bf16_rn(w);
    }
    for (int e = threadIdx.x; e < MLP_H; e += blockDim.x) {
        S.b1[e] = prm[MP_B1 + e];
        S.b2[e] = prm[MP_B2 + e];
    }
    for (int e = threadIdx.x; e < MLP_OUTP; e += blockDim.x) {
        S.b3[e] = e < MLP_OUT ? prm[MP_B3 + e] : 0.f;
        S.out_mean[e] = e < MLP_OUT ? prm[MP_OUT_MEAN + e] : 0.f;
        S.out_std[e] = e < MLP_OUT ? prm[MP_OUT_STD + e] : 0.f;
    }
    for (int e = threadIdx.x; e < MLP_IN; e += blockDim.x) {
        S.in_mean[e] = prm[MP_IN_MEAN + e];
        S.in_rstd[e] = 1.0f / prm[MP_IN_STD + e];
    }
}

// One layer: D[tmem cols 0..N) = A (128 x K, smem) * B^T (N x K, smem), issued by thread 0,
// waited for by every thread.  The caller has fenced and synchronised the A writes.
__device__ __forceinline__ bool mlp_layer(MlpSmem &S, const unsigned char *A, const unsigned char *B, int N, int K,
                                          uint32_t &phase)
{
    if (threadIdx.x == 0) {
        const uint32_t idesc = tc_idesc_bf16(128, N);
        const uint32_t sbo = (uint32_t)(K / 8) * 128;
        for (int j = 0; j < K / 16; j++)
            tc_mma(S.tbase, tc_sdesc(smem_u32(A) + 256 * j, 128, sbo), tc_sdesc(smem_u32(B) + 256 * j, 128, sbo),
                   idesc, j > 0);
        tc_commit(&S.mbar);
    }
    const bool ok = mbar_wait(&S.mbar, phase & 1);
    phase++;
    tc_fence_after();
    return ok;
}

// hidden layer epilogue: bias + SiLU of this thread's row, written as the next layer's input
__device__ __forceinline__ void mlp_hidden_out(MlpSmem &S, const float *bias, int row)
{
    const int warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < MLP_H; c += 16) {
        float v[16];
        tmem_ld16(tmem_at(S.tbase, 32 * warp, c), v);
#pragma unroll
        for (int i = 0; i < 16; i += 8) {
            uint4 pk;
            uint16_t h[8];
#pragma unroll
            for (int q = 0; q < 8; q++) h[q] = bf16_rn(silu(v[i + q] + bias[c + i + q]));
            pk.x = h[0] | ((uint32_t)h[1] << 16);
            pk.y = h[2] | ((uint32_t)h[3] << 16);
            pk.z = h[4] | ((uint32_t)h[5] << 16);
            pk.w = h[6] | ((uint32_t)h[7] << 16);
            *reinterpret_cast<uint4 *>(S.a2 + tc_off(row, c + i, MLP_H)) = pk;
        }
    }
}

// Forward pass of 128 normalised input rows already in S.a1 (fenced): returns the 7 raw
// outputs of this thread's row.  Every thread of the 128-thread CTA must call it.
__device__ bool mlp_forward_tile(MlpSmem &S, uint32_t &phase, float out[MLP_OUT])
{
    const int row = threadIdx.x, warp = row >> 5;
    bool ok = mlp_layer(S, S.a1, S.w1, MLP_H, MLP_IN, phase);
    mlp_hidden_out(S, S.b1, row);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    ok = mlp_layer(S, S.a2, S.w2, MLP_H, MLP_H, phase) && ok;
    mlp_hidden_out(S, S.b2, row);  // the layer-2 MMAs have completed: a2 can be rewritten
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    ok = mlp_layer(S, S.a2, S.w3, MLP_OUTP, MLP_H, phase) && ok;
    float v[16];
    tmem_ld16(tmem_at(S.tbase, 32 * warp, 0), v);
#pragma unroll
    for (int o = 0; o < MLP_OUT; o++) out[o] = (v[o] + S.b3[o]) * S.out_std[o] + S.out_mean[o];
    tc_fence_before();
    // every row's TMEM read is done before the next tile's first MMA; the verdict is made
    // CTA-uniform so that all threads leave a tile loop together
    ok = __syncthreads_and(ok) != 0;
    tc_fence_after();
    return ok;
}

// write one row of raw inputs, normalised, as bf16 into S.a1
__device__ __forceinline__ void mlp_put_input(MlpSmem &S, int row, const float x[MLP_IN])
{
#pragma unroll
    for (int i = 0; i < MLP_IN; i += 8) {
        uint16_t h[8];
#pragma unroll
        for (int q = 0; q < 8; q++) h[q] = bf16_rn((x[i + q] - S.in_mean[i + q]) * S.in_rstd[i + q]);
        uint4 pk;
        pk.x = h[0] | ((uint32_t)h[1] << 16);
        pk.y = h[2] | ((uint32_t)h[3] << 16);
        pk.z = h[4] | ((uint32_t)h[5] << 16);
        pk.w = h[6] | ((uint32_t)h[7] << 16);
        *reinterpret_cast<uint4 *>(S.a1 + tc_off(row, i, MLP_IN)) = pk;
    }
}

constexpr uint32_t MLP_TMEM_COLS = 64;

__device__ __forceinline__ void mlp_begin(MlpSmem &S, const float *prm)
{
    if ((threadIdx.x >> 5) == 0) tmem_alloc(&S.tbase, MLP_TMEM_COLS);
    if (threadIdx.x == 0) {
        mbar_init(&S.mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    mlp_stage_params(S, prm);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

__device__ __forceinline__ void mlp_end(MlpSmem &S)
{
    tc_fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tmem_dealloc(S.tbase, MLP_TMEM_COLS);
}

// Y[n x 7] = MLP(X[n x 16]), raw (un-normalised) FP32 rows; persistent 128-row tiles
__global__ void __launch_bounds__(128) k_mlp_forward(const float *prm, const float *X, long long n, float *Y,
                                                     int *status)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    MlpSmem &S = *reinterpret_cast<MlpSmem *>(smem_raw);
    mlp_begin(S, prm);
    uint32_t phase = 0;
    bool ok = true;
    const long long tiles = (n + 127) / 128;
    for (long long t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        const long long r = t * 128 + threadIdx.x;
        float x[MLP_IN];
#pragma unroll
        for (int i = 0; i < MLP_IN; i++) x[i] = r < n ? X[r * MLP_IN + i] : S.in_mean[i];
        mlp_put_input(S, threadIdx.x, x);
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        float y[MLP_OUT];
        ok = mlp_forward_tile(S, phase, y);
        if (r < n)
#pragma unroll
            for (int o = 0; o < MLP_OUT; o++) Y[r * MLP_OUT + o] = y[o];
    }
    if (!ok && threadIdx.x == 0 && status) atomicOr(status, ERR_TC_TIMEOUT);
    mlp_end(S);
}

}  // namespace gy

extern "C" gy_status gy_tc_gemm_bf16(const uint16_t *d_A, const uint16_t *d_B, float *d_C, int M, int N, int K,
                                     int *d_status, void *stream)
{
    using namespace gy;
    if (!d_A || !d_B || !d_C || M <= 0 || N < 16 || N > TC_GEMM_NMAX || N % 16 || K < 16 || K > TC_GEMM_KMAX ||
        K % 16)
        return GY_ERR_ARG;
    const size_t smem = (size_t)(128 + N) * K * 2;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_GEMM_SMEM) != cudaSuccess)
            return GY_ERR_CUDA;
        attr = true;
    }
    k_tc_gemm<<<(M + 127) / 128, 128, smem, static_cast<cudaStream_t>(stream)>>>(d_A, d_B, d_C, M, N, K, d_status);
    note_launch(1);
    return cudaPeekAtLastError() == cudaSuccess ? GY_OK : GY_ERR_CUDA;
}

extern "C" int64_t gy_mlp_param_count(void) { return gy::MP_COUNT; }

extern "C" gy_status gy_mlp_forward(const float *d_params, const float *d_X, int64_t n, float *d_Y, int *d_status,
                                    void *stream)
{
    using namespace gy;
    if (!d_params || n < 0 || (n > 0 && (!d_X || !d_Y))) return GY_ERR_ARG;
    if (n == 0) return GY_OK;
    const size_t smem = sizeof(MlpSmem) + 1024;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return GY_ERR_CUDA;
        attr = true;
    }
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (n + 127) / 128;
    const int grid = (int)std::min<long long>(tiles, (long long)sms * 4);
    k_mlp_forward<<<grid, 128, smem, static_cast<cudaStream_t>(stream)>>>(d_params, d_X, n, d_Y, d_status);
    note_launch(1);
    return cudaPeekAtLastError() == cudaSuccess ? GY_OK : GY_ERR_CUDA;
}
