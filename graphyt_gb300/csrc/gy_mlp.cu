// gy_mlp.cu -- BF16 tensor-core (tcgen05 + TMEM) kernels of the learned Drucker-Prager
// surrogate, and the plain GEMM they are checked against.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/graphyt_gpu.h"
#include "gy_kernels.cuh"
#include "gy_physics.cuh"
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
    // every row's TMEM read is done before the next tile's first MMA; the outcome is made
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

// ---------------------------------------------------------------------------------------
// Training.  One CTA trains on one 128-sample tile of the batch: forward (three MMAs, the
// pre-activations kept in TMEM), the MSE gradient, backward through the layers (two MMAs) and
// the weight gradients (three MMAs with K = 128 samples), added into the global gradient with
// atomics.  Operands of the weight-gradient MMAs are the transposed activations (K = samples),
// stored in one region as rows XT (16) | H2T (64) | H1T (64) | DZ1T (64) of 128 samples, so
// each of them is the first rows of a 128-row window starting at its first row; the rows past
// the valid ones feed only TMEM lanes that are never read.
constexpr int MLP_TR = 16 + 64 + 64 + 64;            // rows of the transposed region
constexpr int TR_XT = 0, TR_H2T = 16, TR_H1T = 80, TR_DZ1T = 144;
constexpr int MLP_TRAIN_PARAMS = MP_IN_MEAN;          // trainable: weights and biases
// TMEM columns of the training kernel
constexpr int TM_Z1 = 0, TM_Z2 = 64, TM_Y = 128, TM_DH = 192, TM_G3 = 256, TM_G2 = 320, TM_G1 = 384;
constexpr uint32_t MLP_TRAIN_TMEM_COLS = 512;

struct MlpTrainSmem {
    alignas(1024) unsigned char xn[128 * MLP_IN * 2];    // A of layer 1
    alignas(1024) unsigned char h[128 * MLP_H * 2];      // A of layer 2 (h1), layer 3 (h2), then dz2
    alignas(1024) unsigned char dy[128 * MLP_OUTP * 2];  // A of dH2 = dY W3^T
    alignas(1024) unsigned char tr[MLP_TR * 128 * 2];    // transposed activations, K = 128 samples
    alignas(1024) unsigned char dyt[MLP_OUTP * 128 * 2]; // B of dW3
    alignas(1024) unsigned char dz2t[MLP_H * 128 * 2];   // B of dW2
    alignas(1024) unsigned char w1t[MLP_H * MLP_IN * 2];
    alignas(1024) unsigned char w2t[MLP_H * MLP_H * 2];
    alignas(1024) unsigned char w3t[MLP_OUTP * MLP_H * 2];
    alignas(1024) unsigned char w3[MLP_H * MLP_OUTP * 2]; // B of dH2: B[i][o] = W3[i][o]
    alignas(1024) unsigned char w2[MLP_H * MLP_H * 2];    // B of dH1: B[i][o] = W2[i][o]
    float b1[MLP_H], b2[MLP_H], b3[MLP_OUTP];
    float gb1[MLP_H], gb2[MLP_H], gb3[MLP_OUTP];
    float in_mean[MLP_IN], in_rstd[MLP_IN], out_mean[MLP_OUT], out_rstd[MLP_OUT];
    float loss;
    uint64_t mbar;
    uint32_t tbase;
};

__device__ __forceinline__ void put_bf16(unsigned char *tile, int r, int k, int K, float v)
{
    *reinterpret_cast<uint16_t *>(tile + tc_off(r, k, K)) = bf16_rn(v);
}

// d/dz silu(z) = s (1 + z (1 - s)), s = sigmoid(z)
__device__ __forceinline__ float silu_grad(float z)
{
    const float sg = 1.0f / (1.0f + __expf(-z));
    return sg * (1.0f + z * (1.0f - sg));
}

// issue `count` MMAs over K (16 columns each) into TMEM column `col`
__device__ __forceinline__ void mma_k(uint32_t tbase, int col, const unsigned char *A, const unsigned char *B, int N,
                                      int K)
{
    const uint32_t idesc = tc_idesc_bf16(128, N);
    const uint32_t sbo = (uint32_t)(K / 8) * 128;
    for (int j = 0; j < K / 16; j++)
        tc_mma(tbase + (uint32_t)col, tc_sdesc(smem_u32(A) + 256 * j, 128, sbo),
               tc_sdesc(smem_u32(B) + 256 * j, 128, sbo), idesc, j > 0);
}

// all threads: wait for the MMAs committed as phase `ph` (a CTA-uniform outcome)
__device__ __forceinline__ bool mma_done(uint64_t *mbar, uint32_t &ph)
{
    const bool ok = __syncthreads_and(mbar_wait(mbar, ph & 1)) != 0;
    ph++;
    tc_fence_after();
    return ok;
}

// shared-memory writes of this phase visible to the tensor core, then a CTA barrier
__device__ __forceinline__ void smem_to_tc()
{
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
    // splitmix64 finaliser
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// rows: sampled from [0, n) by a hash of (seed, step, row) when sample != 0, else row r of
// the batch is data row r (gradient checks)
__global__ void __launch_bounds__(128) k_mlp_train_tile(const float *prm, const float *X, const float *T, long long n,
                                                        int sample, unsigned long long seed, const int *step_ctr,
                                                        float *grad, float *loss_acc, int batch, int *status)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    MlpTrainSmem &S = *reinterpret_cast<MlpTrainSmem *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tmem_alloc(&S.tbase, MLP_TRAIN_TMEM_COLS);
    if (tid == 0) {
        mbar_init(&S.mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        S.loss = 0.f;
    }
    // ---- weights and biases (BF16 operand tiles in both orientations), normalisation ----
    for (int e = tid; e < MLP_H * MLP_IN; e += 128) {
        const int i = e / MLP_H, o = e - i * MLP_H;  // W1[i][o]
        put_bf16(S.w1t, o, i, MLP_IN, prm[MP_W1 + e]);
    }
    for (int e = tid; e < MLP_H * MLP_H; e += 128) {
        const int i = e / MLP_H, o = e - i * MLP_H;  // W2[i][o]
        const float w = prm[MP_W2 + e];
        put_bf16(S.w2t, o, i, MLP_H, w);
        put_bf16(S.w2, i, o, MLP_H, w);
    }
    for (int e = tid; e < MLP_H * MLP_OUTP; e += 128) {
        const int i = e / MLP_OUTP, o = e - i * MLP_OUTP;
        const float w = o < MLP_OUT ? prm[MP_W3 + i * MLP_OUT + o] : 0.f;
        put_bf16(S.w3t, o, i, MLP_H, w);
        put_bf16(S.w3, i, o, MLP_OUTP, w);
    }
    for (int e = tid; e < MLP_H; e += 128) {
        S.b1[e] = prm[MP_B1 + e];
        S.b2[e] = prm[MP_B2 + e];
        S.gb1[e] = 0.f;
        S.gb2[e] = 0.f;
    }
    if (tid < MLP_OUTP) {
        S.b3[tid] = tid < MLP_OUT ? prm[MP_B3 + tid] : 0.f;
        S.gb3[tid] = 0.f;
    }
    if (tid < MLP_IN) {
        S.in_mean[tid] = prm[MP_IN_MEAN + tid];
        S.in_rstd[tid] = 1.0f / prm[MP_IN_STD + tid];
    }
    if (tid < MLP_OUT) {
        S.out_mean[tid] = prm[MP_OUT_MEAN + tid];
        S.out_rstd[tid] = 1.0f / prm[MP_OUT_STD + tid];
    }
    __syncthreads();
    // ---- this thread's sample ----
    const int s = tid;
    const long long grow = (long long)blockIdx.x * 128 + s;
    long long idx = grow;
    if (sample) idx = (long long)(mix64(seed ^ mix64((unsigned long long)(*step_ctr) * 0x100000001ull + (unsigned long long)grow)) %
                                  (unsigned long long)n);
    const bool live = idx < n;
    float tn[MLP_OUT];
#pragma unroll
    for (int k = 0; k < MLP_IN; k++) {
        const float xv = live ? (X[idx * MLP_IN + k] - S.in_mean[k]) * S.in_rstd[k] : 0.f;
        put_bf16(S.xn, s, k, MLP_IN, xv);
        put_bf16(S.tr, TR_XT + k, s, 128, xv);
    }
#pragma unroll
    for (int o = 0; o < MLP_OUT; o++) tn[o] = live ? (T[idx * MLP_OUT + o] - S.out_mean[o]) * S.out_rstd[o] : 0.f;
    smem_to_tc();
    const uint32_t tb = S.tbase;
    uint32_t ph = 0;
    bool ok = true;
    // ---- layer 1 ----
    if (tid == 0) { mma_k(tb, TM_Z1, S.xn, S.w1t, MLP_H, MLP_IN); tc_commit(&S.mbar); }
    ok = mma_done(&S.mbar, ph) && ok;
    for (int c = 0; c < MLP_H; c += 16) {
        float v[16];
        tmem_ld16(tmem_at(tb, 32 * warp, TM_Z1 + c), v);
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const float hv = silu(v[q] + S.b1[c + q]);
            put_bf16(S.h, s, c + q, MLP_H, hv);
            put_bf16(S.tr, TR_H1T + c + q, s, 128, hv);
        }
    }
    smem_to_tc();
    // ---- layer 2 ----
    if (tid == 0) { mma_k(tb, TM_Z2, S.h, S.w2t, MLP_H, MLP_H); tc_commit(&S.mbar); }
    ok = mma_done(&S.mbar, ph) && ok;
    for (int c = 0; c < MLP_H; c += 16) {
        float v[16];
        tmem_ld16(tmem_at(tb, 32 * warp, TM_Z2 + c), v);
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const float hv = silu(v[q] + S.b2[c + q]);
            put_bf16(S.h, s, c + q, MLP_H, hv);
            put_bf16(S.tr, TR_H2T + c + q, s, 128, hv);
        }
    }
    smem_to_tc();
    // ---- layer 3 and the loss gradient: L = sum (y - t)^2 / (batch * 7) ----
    if (tid == 0) { mma_k(tb, TM_Y, S.h, S.w3t, MLP_OUTP, MLP_H); tc_commit(&S.mbar); }
    ok = mma_done(&S.mbar, ph) && ok;
    {
        float v[16];
        tmem_ld16(tmem_at(tb, 32 * warp, TM_Y), v);
        float l2 = 0.f;
        const float gs = 2.0f / ((float)batch * (float)MLP_OUT);
#pragma unroll
        for (int o = 0; o < MLP_OUTP; o++) {
            float dyv = 0.f;
            if (o < MLP_OUT && live) {
                const float d = v[o] + S.b3[o] - tn[o];
                l2 += d * d;
                dyv = gs * d;
                atomicAdd(&S.gb3[o], dyv);
            }
            put_bf16(S.dy, s, o, MLP_OUTP, dyv);
            put_bf16(S.dyt, o, s, 128, dyv);
        }
        for (int off = 16; off > 0; off >>= 1) l2 += __shfl_xor_sync(0xffffffffu, l2, off);
        if ((tid & 31) == 0) atomicAdd(&S.loss, l2);
    }
    smem_to_tc();
    // ---- dH2 = dY W3^T ----
    if (tid == 0) { mma_k(tb, TM_DH, S.dy, S.w3, MLP_H, MLP_OUTP); tc_commit(&S.mbar); }
    ok = mma_done(&S.mbar, ph) && ok;
    for (int c = 0; c < MLP_H; c += 16) {
        float dh[16], z[16];
        tmem_ld16(tmem_at(tb, 32 * warp, TM_DH + c), dh);
        tmem_ld16(tmem_at(tb, 32 * warp, TM_Z2 + c), z);
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const float dz = live ? dh[q] * silu_grad(z[q] + S.b2[c + q]) : 0.f;
            atomicAdd(&S.gb2[c + q], dz);
            put_bf16(S.h, s, c + q, MLP_H, dz);       // layer 3 is done with h2
            put_bf16(S.dz2t, c + q, s, 128, dz);
        }
    }
    smem_to_tc();
    // ---- dH1 = dZ2 W2^T, dW3 = H2^T dY, dW2 = H1^T dZ2 ----
    if (tid == 0) {
        mma_k(tb, TM_DH, S.h, S.w2, MLP_H, MLP_H);
        mma_k(tb, TM_G3, S.tr + TR_H2T * 256, S.dyt, MLP_OUTP, 128);
        mma_k(tb, TM_G2, S.tr + TR_H1T * 256, S.dz2t, MLP_H, 128);
        tc_commit(&S.mbar);
    }
    ok = mma_done(&S.mbar, ph) && ok;
    for (int c = 0; c < MLP_H; c += 16) {
        float dh[16], z[16];
        tmem_ld16(tmem_at(tb, 32 * warp, TM_DH + c), dh);
        tmem_ld16(tmem_at(tb, 32 * warp, TM_Z1 + c), z);
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const float dz = live ? dh[q] * silu_grad(z[q] + S.b1[c + q]) : 0.f;
            atomicAdd(&S.gb1[c + q], dz);
            put_bf16(S.tr, TR_DZ1T + c + q, s, 128, dz);
        }
    }
    if (warp < 2) {  // TMEM lanes 0-63: rows i of dW3 and dW2
        const int i = tid;
        float g3[16];
        tmem_ld16(tmem_at(tb, 32 * warp, TM_G3), g3);
#pragma unroll
        for (int o = 0; o < MLP_OUT; o++) atomicAdd(&grad[MP_W3 + i * MLP_OUT + o], g3[o]);
        for (int c = 0; c < MLP_H; c += 16) {
            float g2[16];
            tmem_ld16(tmem_at(tb, 32 * warp, TM_G2 + c), g2);
#pragma unroll
            for (int q = 0; q < 16; q++) atomicAdd(&grad[MP_W2 + i * MLP_H + c + q], g2[q]);
        }
    }
    smem_to_tc();
    // ---- dW1 = X^T dZ1 ----
    if (tid == 0) { mma_k(tb, TM_G1, S.tr + TR_XT * 256, S.tr + TR_DZ1T * 256, MLP_H, 128); tc_commit(&S.mbar); }
    ok = mma_done(&S.mbar, ph) && ok;
    if (warp == 0) {  // TMEM lanes 0-15: rows k of dW1
        for (int c = 0; c < MLP_H; c += 16) {
            float g1[16];
            tmem_ld16(tmem_at(tb, 0, TM_G1 + c), g1);
            if (tid < MLP_IN)
#pragma unroll
                for (int q = 0; q < 16; q++) atomicAdd(&grad[MP_W1 + tid * MLP_H + c + q], g1[q]);
        }
    }
    __syncthreads();
    for (int e = tid; e < MLP_H; e += 128) {
        atomicAdd(&grad[MP_B1 + e], S.gb1[e]);
        atomicAdd(&grad[MP_B2 + e], S.gb2[e]);
    }
    if (tid < MLP_OUT) atomicAdd(&grad[MP_B3 + tid], S.gb3[tid]);
    if (tid == 0) atomicAdd(loss_acc, S.loss / ((float)batch * (float)MLP_OUT));
    if (!ok && tid == 0 && status) atomicOr(status, ERR_TC_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tb, MLP_TRAIN_TMEM_COLS);
}

// Adam on the trainable parameters, one CTA; the step counter advances at the end.  The
// step's loss moves from the accumulator to loss_last.
__global__ void __launch_bounds__(1024) k_mlp_adam(float *prm, float *grad, float *m, float *v, int *step_ctr, float lr,
                                                   float *loss_acc, float *loss_last)
{
    const int t = *step_ctr + 1;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.0f / (1.0f - powf(b1, (float)t)), c2 = 1.0f / (1.0f - powf(b2, (float)t));
    for (int p = threadIdx.x; p < MLP_TRAIN_PARAMS; p += blockDim.x) {
        const float g = grad[p];
        const float mm = b1 * m[p] + (1.0f - b1) * g;
        const float vv = b2 * v[p] + (1.0f - b2) * g * g;
        m[p] = mm;
        v[p] = vv;
        prm[p] -= lr * (mm * c1) / (sqrtf(vv * c2) + eps);
        grad[p] = 0.f;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *loss_last = *loss_acc;
        *loss_acc = 0.f;
        *step_ctr = t;
    }
}

// per-column sums and sums of squares of a row-major n x w FP32 matrix, into double acc[2w]
__global__ void k_colstats(const float *A, long long n, int w, double *acc)
{
    __shared__ double sm[2 * 32];
    for (int c = threadIdx.x; c < 2 * w; c += blockDim.x) sm[c] = 0.0;
    __syncthreads();
    double ls[32], lq[32];
    for (int c = 0; c < w; c++) { ls[c] = 0.0; lq[c] = 0.0; }
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x)
        for (int c = 0; c < w; c++) {
            const double x = A[r * w + c];
            ls[c] += x;
            lq[c] += x * x;
        }
    for (int c = 0; c < w; c++) {
        atomicAdd(&sm[c], ls[c]);
        atomicAdd(&sm[w + c], lq[c]);
    }
    __syncthreads();
    for (int c = threadIdx.x; c < 2 * w; c += blockDim.x) atomicAdd(&acc[c], sm[c]);
}

// ---------------------------------------------------------------------------------------
// The surrogate pass of a step: the particles G2P deferred (yielding Drucker-Prager particles,
// their stress still the previous step's) in tiles of 128.  Per particle the MLP predicts the
// return from the elastic trial stress -- stress = trial + predicted correction, plastic
// strain + predicted increment d -- and the prediction is kept when
//   * the yield function there is within tol x cohesion of zero (the exact mapping lands on
//     zero, ConstitutiveModels.cpp:321-344),
//   * d is not negative, and
//   * the predicted stress is, within tol x cohesion per component, the stress the flow rule
//     gives for the multiplier d / xi: the trial deviator scaled by 1 - G dl / sqrt(J2) and
//     the trial mean stress less K eta_bar dl (:397-416) -- a point of the yield surface that
//     is not the return of this trial state fails here;
// the plastic strain tensor then follows the flow direction of the trial deviator with that
// multiplier.  Otherwise the exact return mapping runs.  The Grady-Kipp update follows in
// both cases.
__global__ void __launch_bounds__(128) k_dp_surrogate(PView P, const float4 *pend, const unsigned int *pend_n,
                                                      unsigned int cap, const DevMaterial *mats, const float *prm,
                                                      const StepScalars *scp, const float *flaw, float tol,
                                                      unsigned long long *counts, int *status)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    MlpSmem &S = *reinterpret_cast<MlpSmem *>(smem_raw);
    mlp_begin(S, prm);
    const unsigned int cnt = min(*pend_n, cap);
    const float dt = scp->dt;
    uint32_t phase = 0;
    bool ok = true;
    unsigned int acc = 0, fb = 0;
    const unsigned int tiles = (cnt + 127u) / 128u;
    for (unsigned int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const unsigned int e = tile * 128u + threadIdx.x;
        const bool live = e < cnt;
        Constit c;
        long long slot = 0;
        float de[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        int mat = 0, pid = 0;
        if (live) {
            const float4 q0 = pend[2 * e], q1 = pend[2 * e + 1];
            slot = (long long)__float_as_int(q0.x);
            de[0] = q0.y; de[1] = q0.z; de[2] = q0.w; de[3] = q1.x; de[4] = q1.y; de[5] = q1.z;
#pragma unroll
            for (int k = 0; k < 6; k++) {
                c.s[k] = P.f(PF_S0 + k, slot);
                c.ep[k] = P.f(PF_EP0 + k, slot);
                c.r[k] = de[k] / dt;
                c.e[k] = 0.f;
            }
            c.eqps = P.f(PF_EQPS, slot);
            c.dmg = P.f(PF_DMG, slot);
            c.smax = P.f(PF_SMAX, slot);
            c.mass = P.f(PF_MASS, slot);
            c.rho = P.f(PF_RHO, slot);
            mat = info_mat((uint32_t)P.ii(PF_INFO, slot));
            pid = P.ii(PF_PID, slot);
        }
        const DevMaterial &M = mats[mat];
        float x[MLP_IN];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            x[k] = de[k];
            x[6 + k] = live ? c.s[k] : 0.f;
        }
        x[12] = live ? c.eqps : 0.f;
        x[13] = live ? c.dmg : 0.f;
        x[14] = M.cohesion;
        x[15] = M.phi_deg;
        if (!live) {
#pragma unroll
            for (int k = 0; k < MLP_IN; k++) x[k] = S.in_mean[k];
        }
        mlp_put_input(S, threadIdx.x, x);
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        float y[MLP_OUT];
        ok = mlp_forward_tile(S, phase, y);
        if (live) {
            float t[6];
            dp_trial_yields(c, M, dt, t);
            float sp[6];
#pragma unroll
            for (int k = 0; k < 6; k++) sp[k] = t[k] + y[k];
            const float deq = y[6];
            const float res = dp_residual(sp, c.eqps + deq, M);
            const float I1 = (1.0f / 3.0f) * (t[0] + t[1] + t[2]);
            const float sd[6] = {t[0] - I1, t[1] - I1, t[2] - I1, t[3], t[4], t[5]};
            const float J2 = 0.5f * (sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2] + 2.0f * sd[3] * sd[3] +
                                     2.0f * sd[4] * sd[4] + 2.0f * sd[5] * sd[5]);
            const float dL = deq / M.xi;
            const float fs = J2 > 0.f ? 1.0f - M.G * dL * rsqrtf(J2) : 1.0f, pm = I1 - M.K * M.eta_bar * dL;
            float flow_gap = 0.f;  // largest component distance to the flow-rule stress of dL
#pragma unroll
            for (int k = 0; k < 6; k++) flow_gap = fmaxf(flow_gap, fabsf(sp[k] - (fs * sd[k] + (k < 3 ? pm : 0.f))));
            if (ok && deq >= 0.f && fabsf(res) <= tol * M.cohesion && flow_gap <= tol * M.cohesion) {
                const float hj = J2 > 0.f ? 0.5f / J2 : 0.f;
#pragma unroll
                for (int k = 0; k < 6; k++) {
                    c.s[k] = sp[k];
                    c.ep[k] += dL * (hj * sd[k] + (k < 3 ? M.eta_bar / 3.0f : 0.f));
                }
                c.eqps += deq;
                acc++;
            } else {
                cm_drucker_prager(c, M, dt);
                fb++;
            }
            if (M.damage && M.damage_model == 1) dm_grady_kipp3(c, M, dt, flaw, pid);
#pragma unroll
            for (int k = 0; k < 6; k++) {
                P.f(PF_S0 + k, slot) = c.s[k];
                P.f(PF_EP0 + k, slot) = c.ep[k];
            }
            P.f(PF_EQPS, slot) = c.eqps;
            P.f(PF_DMG, slot) = c.dmg;
            P.f(PF_SMAX, slot) = c.smax;
        }
    }
    // counts of kept predictions and of fallbacks to the exact mapping
    for (int off = 16; off > 0; off >>= 1) {
        acc += __shfl_xor_sync(0xffffffffu, acc, off);
        fb += __shfl_xor_sync(0xffffffffu, fb, off);
    }
    if ((threadIdx.x & 31) == 0 && counts) {
        atomicAdd(&counts[0], (unsigned long long)acc);
        atomicAdd(&counts[1], (unsigned long long)fb);
    }
    if (!ok && threadIdx.x == 0 && status) atomicOr(status, ERR_TC_TIMEOUT);
    mlp_end(S);
}

void launch_dp_surrogate(const PView &P, const float4 *pend, const unsigned int *pend_n, unsigned int cap,
                         const DevMaterial *mats, const float *prm, const StepScalars *scp, const float *flaw, float tol,
                         unsigned long long *counts, int *status, cudaStream_t s)
{
    const size_t smem = sizeof(MlpSmem) + 1024;
    static int grid = 0;
    if (grid == 0) {
        cudaFuncSetAttribute(k_dp_surrogate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int dev = 0, sms = 1, b = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_dp_surrogate, 128, smem);
        // every resident CTA holds MLP_TMEM_COLS of the 512 tensor-memory columns
        b = std::max(1, std::min(b, (int)(512 / MLP_TMEM_COLS)));
        grid = sms * b;
    }
    k_dp_surrogate<<<grid, 128, smem, s>>>(P, pend, pend_n, cap, mats, prm, scp, flaw, tol, counts, status);
    note_launch(1);
}

// The give-up path of the bounded mbarrier wait: thread 0 initialises an mbarrier that nothing
// arrives at, every thread waits on it, and the block reports the wait that gave up in the
// status word -- the route every tensor-core wait of the library takes when its arrival is lost.
__global__ void k_tc_wait_check(int *status, unsigned long long *elapsed_ns)
{
    __shared__ uint64_t mbar;
    if (threadIdx.x == 0) mbar_init(&mbar, 1);
    __syncthreads();
    const unsigned long long t0 = clock_now_ns();
    const bool ok = __syncthreads_and(mbar_wait(&mbar, 0)) != 0;
    if (threadIdx.x == 0) {
        if (!ok) atomicOr(status, ERR_TC_TIMEOUT);
        *elapsed_ns = clock_now_ns() - t0;
    }
}

}  // namespace gy

extern "C" gy_status gy_tc_wait_check(int *d_status, unsigned long long *d_elapsed_ns, void *stream)
{
    using namespace gy;
    if (!d_status || !d_elapsed_ns) return GY_ERR_ARG;
    k_tc_wait_check<<<1, 64, 0, static_cast<cudaStream_t>(stream)>>>(d_status, d_elapsed_ns);
    note_launch(1);
    return cudaPeekAtLastError() == cudaSuccess ? GY_OK : GY_ERR_CUDA;
}

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

namespace {

size_t train_smem() { return sizeof(gy::MlpTrainSmem) + 1024; }

gy_status train_attr()
{
    static bool done = false;
    if (done) return GY_OK;
    if (cudaFuncSetAttribute(gy::k_mlp_train_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()) !=
        cudaSuccess)
        return GY_ERR_CUDA;
    done = true;
    return GY_OK;
}

}  // namespace

extern "C" gy_status gy_mlp_grad(const float *d_params, const float *d_X, const float *d_T, int64_t n, float *d_grad,
                                 float *d_loss, int *d_status, void *stream)
{
    using namespace gy;
    if (!d_params || !d_X || !d_T || !d_grad || !d_loss || n <= 0 || n % 128) return GY_ERR_ARG;
    if (train_attr() != GY_OK) return GY_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the step counter is read only when sampling; a zero from the status word's neighbour
    // is not needed: pass the loss word itself as an unused counter
    k_mlp_train_tile<<<(unsigned)(n / 128), 128, train_smem(), s>>>(d_params, d_X, d_T, n, 0, 0ull,
                                                                      reinterpret_cast<const int *>(d_loss), d_grad,
                                                                      d_loss, (int)n, d_status);
    note_launch(1);
    return cudaPeekAtLastError() == cudaSuccess ? GY_OK : GY_ERR_CUDA;
}

extern "C" gy_status gy_mlp_train(float *d_params, const float *d_X, const float *d_T, int64_t n, int steps, int batch,
                                  float lr, uint64_t seed, int init, float *loss_out, int *d_status, void *stream)
{
    using namespace gy;
    if (!d_params || !d_X || !d_T || n < 1 || steps < 0 || batch < 128 || batch % 128 || !(lr > 0.f))
        return GY_ERR_ARG;
    if (train_attr() != GY_OK) return GY_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int np = MP_COUNT;
    std::vector<float> host(np, 0.0f);
    if (cudaMemcpyAsync(host.data(), d_params, np * sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GY_ERR_CUDA;
    if (init) {
        // normalisation from the data (per-column mean and standard deviation; constant
        // columns keep a unit scale), weights uniform in +-sqrt(6 / (fan_in + fan_out)),
        // biases zero
        double *acc = nullptr;
        if (cudaMalloc(&acc, 2 * (MLP_IN + MLP_OUT) * sizeof(double)) != cudaSuccess) return GY_ERR_NOMEM;
        cudaMemsetAsync(acc, 0, 2 * (MLP_IN + MLP_OUT) * sizeof(double), s);
        const int g = (int)std::min<long long>((n + 255) / 256, 1024);
        k_colstats<<<g, 256, 0, s>>>(d_X, n, MLP_IN, acc);
        k_colstats<<<g, 256, 0, s>>>(d_T, n, MLP_OUT, acc + 2 * MLP_IN);
        note_launch(2);
        std::vector<double> a(2 * (MLP_IN + MLP_OUT));
        const cudaError_t e1 = cudaMemcpyAsync(a.data(), acc, a.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
        const cudaError_t e2 = cudaStreamSynchronize(s);
        cudaFree(acc);
        if (e1 != cudaSuccess || e2 != cudaSuccess) return GY_ERR_CUDA;
        auto fill = [&](const double *sum, int w, int mean_off, int std_off) {
            for (int c = 0; c < w; c++) {
                const double mu = sum[c] / (double)n;
                const double var = std::max(sum[w + c] / (double)n - mu * mu, 0.0);
                double sd = std::sqrt(var);
                if (!(sd > 1e-12 * std::max(1.0, std::fabs(mu)))) sd = 1.0;
                host[mean_off + c] = (float)mu;
                host[std_off + c] = (float)sd;
            }
        };
        fill(a.data(), MLP_IN, MP_IN_MEAN, MP_IN_STD);
        fill(a.data() + 2 * MLP_IN, MLP_OUT, MP_OUT_MEAN, MP_OUT_STD);
        unsigned long long st = seed * 0x9E3779B97F4A7C15ull + 1ull;
        auto uni = [&]() {  // uniform in [-1, 1)
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            return (double)(st >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
        };
        auto init_w = [&](int off, int fin, int fout) {
            const double b = std::sqrt(6.0 / (fin + fout));
            for (int k = 0; k < fin * fout; k++) host[off + k] = (float)(b * uni());
        };
        init_w(MP_W1, MLP_IN, MLP_H);
        init_w(MP_W2, MLP_H, MLP_H);
        init_w(MP_W3, MLP_H, MLP_OUT);
        for (int k = 0; k < MLP_H; k++) host[MP_B1 + k] = host[MP_B2 + k] = 0.f;
        for (int k = 0; k < MLP_OUT; k++) host[MP_B3 + k] = 0.f;
        if (cudaMemcpyAsync(d_params, host.data(), np * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return GY_ERR_CUDA;
    }
    if (steps == 0) return GY_OK;
    // the steps run on a private stream (a graph cannot be captured on the legacy default
    // stream), ordered after the caller's work and waited for before returning
    cudaStream_t ts = nullptr;
    cudaEvent_t ev = nullptr;
    if (cudaStreamCreateWithFlags(&ts, cudaStreamNonBlocking) != cudaSuccess) return GY_ERR_CUDA;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
        cudaStreamDestroy(ts);
        return GY_ERR_CUDA;
    }
    gy_status rc = GY_OK;
    if (cudaEventRecord(ev, s) != cudaSuccess || cudaStreamWaitEvent(ts, ev, 0) != cudaSuccess) rc = GY_ERR_CUDA;
    // optimizer state: gradient, two moments, step counter, loss words
    float *buf = nullptr;
    const size_t nf = 3 * (size_t)np + 8;
    if (rc == GY_OK && cudaMalloc(&buf, nf * sizeof(float)) != cudaSuccess) rc = GY_ERR_NOMEM;
    if (rc == GY_OK && cudaMemsetAsync(buf, 0, nf * sizeof(float), ts) != cudaSuccess) rc = GY_ERR_CUDA;
    float *grad = buf, *m1 = buf + np, *m2 = buf + 2 * np;
    int *ctr = reinterpret_cast<int *>(buf + 3 * np);
    float *loss_acc = buf + 3 * np + 1, *loss_last = buf + 3 * np + 2;
    // one step captured as a graph and replayed
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (rc == GY_OK && cudaStreamBeginCapture(ts, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = GY_ERR_CUDA;
    if (rc == GY_OK) {
        k_mlp_train_tile<<<(unsigned)(batch / 128), 128, train_smem(), ts>>>(d_params, d_X, d_T, n, 1, seed, ctr, grad,
                                                                               loss_acc, batch, d_status);
        k_mlp_adam<<<1, 1024, 0, ts>>>(d_params, grad, m1, m2, ctr, lr, loss_acc, loss_last);
        if (cudaStreamEndCapture(ts, &graph) != cudaSuccess) rc = GY_ERR_CUDA;
    }
    if (rc == GY_OK && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) rc = GY_ERR_CUDA;
    for (int k = 0; k < steps && rc == GY_OK; k++) {
        if (cudaGraphLaunch(exec, ts) != cudaSuccess) rc = GY_ERR_CUDA;
        note_launch(2);
    }
    float lh = 0.f;
    if (rc == GY_OK && (cudaMemcpyAsync(&lh, loss_last, sizeof(float), cudaMemcpyDeviceToHost, ts) != cudaSuccess ||
                        cudaStreamSynchronize(ts) != cudaSuccess))
        rc = GY_ERR_CUDA;
    if (rc != GY_OK) cudaStreamSynchronize(ts);
    if (loss_out) *loss_out = lh;
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (buf) cudaFree(buf);
    cudaEventDestroy(ev);
    cudaStreamDestroy(ts);
    return rc;
}
