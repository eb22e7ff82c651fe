// mlp.cu -- the charging network: a 6 -> 64 -> 64 -> 1 tanh MLP that maps a cell's charging
// inputs (log nH, log T, log zeta and three grain moments, see k_charge_features) to the start
// point of the Marchand Newton iteration, t = psi/psi0 - 1.
//
// The two hidden-layer GEMMs and the three GEMMs of the backward pass run on the 5th-generation
// tensor cores: BF16 operands staged in shared memory (K-major core-matrix layout, umma.cuh),
// FP32 accumulators in TMEM, one elected thread issuing tcgen05.mma, completion through an
// mbarrier, results read back with tcgen05.ld.  One CTA of 128 threads handles a tile of 128
// samples; thread t owns sample t (TMEM lane t) for the element-wise work.
//   forward:  z1 = x W1^T (M128 N64 K16)      h1 = tanh(z1 + b1)
//             z2 = h1 W2^T (M128 N64 K64)     h2 = tanh(z2 + b2)     y = h2 . w3 + b3  (FP32)
//   backward: dz2 = dy w3 (1 - h2^2)
//             dh1 = dz2 W2 (M128 N64 K64, B = W2^T packed)           dz1 = dh1 (1 - h1^2)
//             [dW2^T; .] = [h1^T; x^T; 0] dz2 (M128 N64 K128: rows 0-63)
//             [.; dW1^T; .] = [h1^T; x^T; 0] dz1 (M128 N64 K128: rows 64-79)
// Bias and output-layer gradients are reduced in shared memory; every CTA adds its gradients
// to the global FP32 gradient with atomics.  Master weights and Adam moments are FP32; the BF16
// copies the MMAs read are re-packed after every update.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/shark_gpu.h"
#include "mlp.h"
#include "umma.cuh"

namespace shark {
namespace mlp {

constexpr int F = SHARK_MLP_NFEAT, KIN = 16, H = 64, TILE = 128;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * KIN, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H;
constexpr int OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H, NPARAM = OFF_B3 + 1;
constexpr int OFF_XMU = NPARAM, OFF_XSD = OFF_XMU + F, OFF_TMU = OFF_XSD + F, OFF_TSD = OFF_TMU + 1;
constexpr int NBLOB = OFF_TSD + 1;
static_assert(NPARAM == SHARK_MLP_NPARAM && NBLOB == SHARK_MLP_NBLOB, "blob layout");

// packed BF16 operands (core-matrix layout): W1 (64 x 16) | W2 (64 x 64) | W2^T (64 x 64)
constexpr int PK_W1 = 0, PK_W2 = PK_W1 + H * KIN * 2, PK_W2T = PK_W2 + H * H * 2, PK_BYTES = PK_W2T + H * H * 2;

// shared memory of one tile (bytes)
constexpr int S_X = 0;                           // 128 x 16   A of layer 1
constexpr int S_W1 = S_X + TILE * KIN * 2;       //  64 x 16   B of layer 1
constexpr int S_H1 = S_W1 + H * KIN * 2;         // 128 x 64   A of layer 2
constexpr int S_W2 = S_H1 + TILE * H * 2;        //  64 x 64   B of layer 2
constexpr int S_FWD_END = S_W2 + H * H * 2;
constexpr int S_DZ2 = S_FWD_END;                 // 128 x 64   A of dh1
constexpr int S_W2T = S_DZ2 + TILE * H * 2;      //  64 x 64   B of dh1
constexpr int S_HT = S_W2T + H * H * 2;          // 128 x 128  A of the weight gradients
constexpr int S_DZ2T = S_HT + TILE * TILE * 2;   //  64 x 128  B of dW2
constexpr int S_DZ1T = S_DZ2T + H * TILE * 2;    //  64 x 128  B of dW1
constexpr int S_RED = S_DZ1T + H * TILE * 2;     // 128 x 65 FP32 reduction scratch
constexpr int S_TRAIN_END = S_RED + TILE * 65 * 4;

template <bool TRAIN> struct TmemCols { static constexpr uint32_t value = TRAIN ? 256u : 128u; };
constexpr uint32_t WAIT_LIMIT = 1u << 24;

__device__ __forceinline__ void put_bf16(uint8_t* base, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}

// column sums over the 128 samples of v[64] (one row per thread) -> atomically into g[0..63]
__device__ __forceinline__ void reduce_cols_to(float* red, const float* v, float* g) {
    const int t = threadIdx.x;
    __syncthreads();
    for (int j = 0; j < H; ++j) red[t * 65 + j] = v[j];
    __syncthreads();
    if (t < H) {
        float s = 0.0f;
        for (int r = 0; r < TILE; ++r) s += red[r * 65 + t];
        atomicAdd(&g[t], s);
    }
}

template <bool TRAIN>
__global__ void __launch_bounds__(TILE, 1) k_mlp(MlpArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t s_mbar;
    __shared__ uint32_t s_tmem;
    __shared__ float s_sum[2];
    const int t = threadIdx.x, warp = t >> 5;
    const int idx = blockIdx.x * TILE + t;
    const bool valid = idx < a.n;
    const long long sample = valid ? (a.index ? (long long)a.index[idx] : (long long)idx) : 0;
    const float* P = a.blob;

    if (warp == 0) umma::tmem_alloc(&s_tmem, TmemCols<TRAIN>::value);
    if (t == 0) {
        umma::mbar_init(&s_mbar, 1);
        s_sum[0] = s_sum[1] = 0.0f;
    }
    // packed weights -> shared memory
    {
        const int4* src = reinterpret_cast<const int4*>(a.packed);
        int4* w1 = reinterpret_cast<int4*>(sm + S_W1);
        int4* w2 = reinterpret_cast<int4*>(sm + S_W2);
        for (int i = t; i < H * KIN * 2 / 16; i += TILE) w1[i] = src[PK_W1 / 16 + i];
        for (int i = t; i < H * H * 2 / 16; i += TILE) w2[i] = src[PK_W2 / 16 + i];
        if (TRAIN) {
            int4* w2t = reinterpret_cast<int4*>(sm + S_W2T);
            for (int i = t; i < H * H * 2 / 16; i += TILE) w2t[i] = src[PK_W2T / 16 + i];
            // rows 80..127 of [h1^T; x^T; 0] stay zero
            int4* ht = reinterpret_cast<int4*>(sm + S_HT + 80 / 8 * (TILE * 16));
            for (int i = t; i < 48 * TILE * 2 / 16; i += TILE) ht[i] = make_int4(0, 0, 0, 0);
        }
    }
    // normalised features of this sample
    float xn[KIN];
#pragma unroll
    for (int i = 0; i < KIN; ++i) xn[i] = 0.0f;
    if (valid)
        for (int i = 0; i < F; ++i) xn[i] = (a.feat[sample * a.feat_stride + i] - P[OFF_XMU + i]) / P[OFF_XSD + i];
#pragma unroll
    for (int i = 0; i < KIN; ++i) {
        put_bf16(sm + S_X, umma::kmajor_offset(t, i, KIN), xn[i]);
        if (TRAIN) put_bf16(sm + S_HT, umma::kmajor_offset(64 + i, t, TILE), xn[i]);
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tm = s_tmem;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    const uint32_t sbase = umma::smem_addr(sm);
    bool ok = true;
    uint32_t phase = 0;

    // ---- layer 1: D[0:64) = x W1^T --------------------------------------------------------------
    if (t == 0) {
        umma::mma_bf16(tm + 0, umma::smem_desc(sbase + S_X, 128, KIN * 16), umma::smem_desc(sbase + S_W1, 128, KIN * 16),
                       umma::idesc_bf16(128, 64), 0u);
        umma::commit(&s_mbar);
    }
    ok = umma::mbar_wait(&s_mbar, phase, WAIT_LIMIT) && ok;
    phase ^= 1;
    umma::fence_after_sync();
    float h1[H];
#pragma unroll
    for (int c = 0; c < H; c += 16) umma::tmem_ld16(tm + lane_base + c, h1 + c);
#pragma unroll
    for (int j = 0; j < H; ++j) {
        h1[j] = tanhf(h1[j] + P[OFF_B1 + j]);
        put_bf16(sm + S_H1, umma::kmajor_offset(t, j, H), h1[j]);
        if (TRAIN) put_bf16(sm + S_HT, umma::kmajor_offset(j, t, TILE), h1[j]);
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();

    // ---- layer 2: D[64:128) = h1 W2^T -------------------------------------------------------------
    if (t == 0) {
        for (int kk = 0; kk < H / 16; ++kk)
            umma::mma_bf16(tm + 64, umma::smem_desc(sbase + S_H1 + kk * 256, 128, H * 16),
                           umma::smem_desc(sbase + S_W2 + kk * 256, 128, H * 16), umma::idesc_bf16(128, 64),
                           kk > 0 ? 1u : 0u);
        umma::commit(&s_mbar);
    }
    ok = umma::mbar_wait(&s_mbar, phase, WAIT_LIMIT) && ok;
    phase ^= 1;
    umma::fence_after_sync();
    float h2[H];
#pragma unroll
    for (int c = 0; c < H; c += 16) umma::tmem_ld16(tm + lane_base + 64 + c, h2 + c);
    float y = P[OFF_B3];
#pragma unroll
    for (int j = 0; j < H; ++j) {
        h2[j] = tanhf(h2[j] + P[OFF_B2 + j]);
        y += P[OFF_W3 + j] * h2[j];
    }

    if (!TRAIN) {
        if (valid && a.out) a.out[idx] = y * P[OFF_TSD] + P[OFF_TMU];
        if (valid && a.seed) {
            // start point psi = psi0 (1 + t) inside the reference's admissible range [psi0, 0):
            // an iterate below psi0 is clamped and flagged low-temperature (ionisation.f90:119-125),
            // so t > 0 starts from psi0 itself; psi >= 0 is no start (the kernel falls back to psi0)
            const double tt = fmin((double)(y * P[OFF_TSD] + P[OFF_TMU]), 0.0);
            const float ps = (float)(a.psi0 * (1.0 + tt));
            a.seed[sample] = ps < 0.0f ? ps : 0.0f;
        }
    } else {
        float* red = reinterpret_cast<float*>(sm + S_RED);
        const float yn = valid ? (a.target[sample * a.feat_stride + F] - P[OFF_TMU]) / P[OFF_TSD] : 0.0f;
        const float err = valid ? y - yn : 0.0f;
        const float dy = 2.0f * err * a.inv_n;
        float dz[H];
#pragma unroll
        for (int j = 0; j < H; ++j) {
            dz[j] = dy * P[OFF_W3 + j] * (1.0f - h2[j] * h2[j]);
            put_bf16(sm + S_DZ2, umma::kmajor_offset(t, j, H), dz[j]);
            put_bf16(sm + S_DZ2T, umma::kmajor_offset(j, t, TILE), dz[j]);
        }
        umma::fence_proxy_async();
        // output-layer and bias gradients
        atomicAdd(&s_sum[0], dy);
        atomicAdd(&s_sum[1], err * err);
        reduce_cols_to(red, dz, a.grad + OFF_B2);
#pragma unroll
        for (int j = 0; j < H; ++j) h2[j] *= dy;
        reduce_cols_to(red, h2, a.grad + OFF_W3);
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        if (t == 0) {
            atomicAdd(&a.grad[OFF_B3], s_sum[0]);
            atomicAdd(a.loss, s_sum[1]);
            // dh1 = dz2 W2 -> D[0:64)
            for (int kk = 0; kk < H / 16; ++kk)
                umma::mma_bf16(tm + 0, umma::smem_desc(sbase + S_DZ2 + kk * 256, 128, H * 16),
                               umma::smem_desc(sbase + S_W2T + kk * 256, 128, H * 16), umma::idesc_bf16(128, 64),
                               kk > 0 ? 1u : 0u);
            // [h1^T; x^T; 0] dz2 -> D[128:192): rows 0-63 = dW2^T
            for (int kk = 0; kk < TILE / 16; ++kk)
                umma::mma_bf16(tm + 128, umma::smem_desc(sbase + S_HT + kk * 256, 128, TILE * 16),
                               umma::smem_desc(sbase + S_DZ2T + kk * 256, 128, TILE * 16), umma::idesc_bf16(128, 64),
                               kk > 0 ? 1u : 0u);
            umma::commit(&s_mbar);
        }
        ok = umma::mbar_wait(&s_mbar, phase, WAIT_LIMIT) && ok;
        phase ^= 1;
        umma::fence_after_sync();
        float d[H];
#pragma unroll
        for (int c = 0; c < H; c += 16) umma::tmem_ld16(tm + lane_base + c, d + c);
#pragma unroll
        for (int i = 0; i < H; ++i) {
            d[i] = d[i] * (1.0f - h1[i] * h1[i]);   // dz1
            put_bf16(sm + S_DZ1T, umma::kmajor_offset(i, t, TILE), d[i]);
        }
        umma::fence_proxy_async();
        float g[H];
#pragma unroll
        for (int c = 0; c < H; c += 16) umma::tmem_ld16(tm + lane_base + 128 + c, g + c);
        if (t < H)   // row t of dW2^T: dW2[j][t]
            for (int j = 0; j < H; ++j) atomicAdd(&a.grad[OFF_W2 + j * H + t], g[j]);
        reduce_cols_to(red, d, a.grad + OFF_B1);
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        if (t == 0) {
            // [h1^T; x^T; 0] dz1 -> D[192:256): rows 64-79 = dW1^T
            for (int kk = 0; kk < TILE / 16; ++kk)
                umma::mma_bf16(tm + 192, umma::smem_desc(sbase + S_HT + kk * 256, 128, TILE * 16),
                               umma::smem_desc(sbase + S_DZ1T + kk * 256, 128, TILE * 16), umma::idesc_bf16(128, 64),
                               kk > 0 ? 1u : 0u);
            umma::commit(&s_mbar);
        }
        ok = umma::mbar_wait(&s_mbar, phase, WAIT_LIMIT) && ok;
        phase ^= 1;
        umma::fence_after_sync();
#pragma unroll
        for (int c = 0; c < H; c += 16) umma::tmem_ld16(tm + lane_base + 192 + c, g + c);
        if (t >= 64 && t < 64 + KIN) {
            const int i = t - 64;   // row 64 + i of the product: dW1[j][i]
            if (i < F)
                for (int j = 0; j < H; ++j) atomicAdd(&a.grad[OFF_W1 + j * KIN + i], g[j]);
        }
    }
    if (!ok && a.err) atomicOr(a.err, 1u);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after_sync();
        umma::tmem_dealloc(tm, TmemCols<TRAIN>::value);
    }
}

// Adam on the FP32 master weights (W1 columns >= F stay zero), then the BF16 packs.
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1t, float b2t) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    if (p < OFF_B1 && (p % KIN) >= F) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gi = g[p];
    const float mi = b1 * m[p] + (1.0f - b1) * gi;
    const float vi = b2 * v[p] + (1.0f - b2) * gi * gi;
    m[p] = mi;
    v[p] = vi;
    w[p] -= lr * (mi / (1.0f - b1t)) / (sqrtf(vi / (1.0f - b2t)) + eps);
}

__global__ void k_pack(const float* __restrict__ w, uint8_t* __restrict__ pk) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < H * KIN) {                       // W1 as B: row j (output), K = input i
        const int j = e / KIN, i = e % KIN;
        put_bf16(pk + PK_W1, umma::kmajor_offset(j, i, KIN), w[OFF_W1 + e]);
    }
    if (e < H * H) {
        const int j = e / H, i = e % H;      // W2[j][i]: row j (output), K = input i
        put_bf16(pk + PK_W2, umma::kmajor_offset(j, i, H), w[OFF_W2 + e]);
        put_bf16(pk + PK_W2T, umma::kmajor_offset(i, j, H), w[OFF_W2 + e]);   // W2^T: row i, K = j
    }
}

}  // namespace mlp

// ---- host launchers (mlp.h) -----------------------------------------------------------------
size_t mlp_packed_bytes() { return mlp::PK_BYTES; }

cudaError_t mlp_pack(const float* blob, uint8_t* packed, cudaStream_t st) {
    mlp::k_pack<<<(mlp::H * mlp::H + 255) / 256, 256, 0, st>>>(blob, packed);
    return cudaGetLastError();
}

cudaError_t mlp_forward(const MlpArgs& a, cudaStream_t st) {
    const int smem = mlp::S_FWD_END;
    cudaError_t e = cudaFuncSetAttribute(mlp::k_mlp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    if (a.n <= 0) return cudaSuccess;
    mlp::k_mlp<false><<<(a.n + mlp::TILE - 1) / mlp::TILE, mlp::TILE, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t mlp_backward(const MlpArgs& a, cudaStream_t st) {
    const int smem = mlp::S_TRAIN_END;
    cudaError_t e = cudaFuncSetAttribute(mlp::k_mlp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    if (a.n <= 0) return cudaSuccess;
    mlp::k_mlp<true><<<(a.n + mlp::TILE - 1) / mlp::TILE, mlp::TILE, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t mlp_adam(float* blob, const float* grad, float* m, float* v, float lr, int step, cudaStream_t st) {
    const float b1t = powf(0.9f, (float)step), b2t = powf(0.999f, (float)step);
    mlp::k_adam<<<(mlp::NPARAM + 255) / 256, 256, 0, st>>>(blob, grad, m, v, lr, b1t, b2t);
    return cudaGetLastError();
}

}  // namespace shark
