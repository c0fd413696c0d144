// Radial MLP surrogate of the Table pair potential (EvaluatorPairTable,
// hoomd/md/EvaluatorPairTable.h): training kernels (FP32, one thread per sample, then batch
// reductions and Adam) and two inference paths on the BF16 tensor cores with FP32 accumulation:
// tcgen05 tiles of 128 pairs with the accumulators in tensor memory (k_mlp_forces_tc, the
// default, at the end of this file) and warp-level mma.sync m16n8k16 tiles of 16 pairs
// (k_mlp_forces, k_eval).
//
// mma.sync tile: the 16 pairs of a tile are the 16 rows of the A operand. Layer 1 multiplies the
// 32 radial features (and, for the derivative, their r-derivatives) by W1r^T; its FP32
// accumulator starts from the per-type-pair offset C[p] = W1e E[p] + b1. The accumulator
// fragment of one layer (rows g and g+8, columns 2t and 2t+1 of each 8-column tile) is exactly the
// A-operand fragment of the next layer's 16-column k-step, so the activations stay in registers
// from the radial features to the energy. The derivative dU/dr is carried forward beside the
// value (dz = W dh), which doubles the products and needs no transposed weights.
#include <cstdint>

#include <cuda_bf16.h>

#include "gb_device.cuh"
#include "gb_host.h"

namespace gb
{
namespace
{
constexpr int EMB = 16, RBF = 32, HID = 64;
constexpr int O_W1E = 0, O_W1R = 1024, O_B1 = 3072, O_W2 = 3136, O_B2 = 7232, O_W3 = 7296,
              O_B3 = 7360, O_E = 7424;

// per-sample training scratch row (floats)
constexpr int S_GZ2 = 0, S_H1 = 64, S_GDZ2 = 128, S_DH1 = 192, S_GZ1 = 256, S_GDZ1 = 320,
              S_H2 = 384, S_DH2 = 448, S_PHI = 512, S_DPHI = 544, S_E = 576, S_GU = 592,
              S_GD = 593, S_LOSS = 594, SW = 596;

// inference block (bytes): mma.sync fragments of W1r and W2, b2, w3, b3, the tcgen05 operand
// images of W1r and W2 (K-major core-matrix layout), then C[p] per type pair
constexpr size_t I_FW1 = 0, I_FW2 = 4096, I_B2 = 12288, I_W3 = 12544, I_B3 = 12800,
                 I_TW1 = 12816, I_TW2 = 16912, I_C = 25104;

// Byte offset of element (row, k) of a K-major tcgen05 operand with K columns in the
// no-swizzle layout: core matrices of 8 rows x 16 bytes, K-adjacent core matrices 128 bytes
// apart (the descriptor's leading-dimension offset), row groups K / 8 * 128 bytes apart (its
// stride-dimension offset).
__host__ __device__ constexpr uint32_t tc_off(int row, int k, int K)
    {
    return (uint32_t)((row >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
    }

__host__ __device__ inline size_t param_count(uint32_t n_pairs)
    {
    return (size_t)O_E + (size_t)EMB * n_pairs;
    }

__device__ __forceinline__ float q_bf16(float x)
    {
    return __bfloat162float(__float2bfloat16_rn(x));
    }

// activation rounding model: 0 none, 1 bfloat16, 2 bfloat16 + bfloat16 remainder
__device__ __forceinline__ float q_act(float x, int quant)
    {
    if (quant == 0)
        return x;
    const float hi = q_bf16(x);
    return quant == 1 ? hi : hi + q_bf16(x - hi);
    }

__device__ __forceinline__ float q_w(float x, int quant)
    {
    return quant ? q_bf16(x) : x;
    }

struct Silu
    {
    float f, d1, d2;
    };

// silu(z) = z s(z), s = logistic; first and second derivatives
__device__ __forceinline__ Silu silu3(float z)
    {
    const float s = 1.0f / (1.0f + expf(-z));
    Silu o;
    o.f = z * s;
    o.d1 = s * (1.0f + z * (1.0f - s));
    o.d2 = s * (1.0f - s) * (2.0f + z * (1.0f - 2.0f * s));
    return o;
    }

// ------------------------------------------------------------------------------------------------
// training
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128)
    k_train_sample(const float* __restrict__ th, uint32_t n_pairs, float r_min, float r_cut,
                   const uint32_t* __restrict__ pair, const float* __restrict__ rr,
                   const float* __restrict__ Ut, const float* __restrict__ Ft, uint32_t B,
                   float lam, int quant, float* __restrict__ grad, float* __restrict__ S)
    {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B)
        return;
    float* row = S + (size_t)s * SW;
    const uint32_t p = min(pair[s], n_pairs - 1);
    const float r = rr[s];
    const float h = (r_cut - r_min) / (float)(RBF - 1);
    const float gamma = 1.0f / (2.0f * h * h);
    float phi[RBF], dphi[RBF];
    for (int k = 0; k < RBF; k++)
        {
        const float d = r - (r_min + (float)k * h);
        const float e = expf(-gamma * d * d);
        phi[k] = q_act(e, quant);
        dphi[k] = q_act(-2.0f * gamma * d * e, quant);
        row[S_PHI + k] = phi[k];
        row[S_DPHI + k] = dphi[k];
        }
    float emb[EMB];
    for (int m = 0; m < EMB; m++)
        {
        emb[m] = q_w(th[O_E + (size_t)p * EMB + m], quant);
        row[S_E + m] = emb[m];
        }
    float dz1[HID], s1[HID], t1[HID], h1[HID], dh1[HID];
    for (int n = 0; n < HID; n++)
        {
        float a = th[O_B1 + n], da = 0.0f;
        for (int m = 0; m < EMB; m++)
            a += q_w(th[O_W1E + n * EMB + m], quant) * emb[m];
        for (int k = 0; k < RBF; k++)
            {
            const float w = q_w(th[O_W1R + n * RBF + k], quant);
            a += w * phi[k];
            da += w * dphi[k];
            }
        const Silu sl = silu3(a);
        dz1[n] = da;
        s1[n] = sl.d1;
        t1[n] = sl.d2;
        h1[n] = q_act(sl.f, quant);
        dh1[n] = q_act(sl.d1 * da, quant);
        row[S_H1 + n] = h1[n];
        row[S_DH1 + n] = dh1[n];
        }
    float dz2[HID], s2[HID], t2[HID];
    float U = th[O_B3], dU = 0.0f;
    for (int n = 0; n < HID; n++)
        {
        float a = th[O_B2 + n], da = 0.0f;
        for (int k = 0; k < HID; k++)
            {
            const float w = q_w(th[O_W2 + n * HID + k], quant);
            a += w * h1[k];
            da += w * dh1[k];
            }
        const Silu sl = silu3(a);
        dz2[n] = da;
        s2[n] = sl.d1;
        t2[n] = sl.d2;
        const float w3 = q_w(th[O_W3 + n], quant);
        U += w3 * sl.f;
        dU += w3 * (sl.d1 * da);
        row[S_H2 + n] = sl.f;
        row[S_DH2 + n] = sl.d1 * da;
        }
    const float eU = U - Ut[s], eD = dU + Ft[s];
    const float gU = 2.0f * lam * eU / (float)B, gD = 2.0f * eD / (float)B;
    row[S_GU] = gU;
    row[S_GD] = gD;
    row[S_LOSS] = eD * eD + lam * eU * eU;
    float gz2[HID], gdz2[HID];
    for (int n = 0; n < HID; n++)
        {
        const float w3 = q_w(th[O_W3 + n], quant);
        const float g_h2 = gU * w3, g_dh2 = gD * w3;
        gdz2[n] = g_dh2 * s2[n];
        gz2[n] = g_h2 * s2[n] + g_dh2 * t2[n] * dz2[n];
        row[S_GZ2 + n] = gz2[n];
        row[S_GDZ2 + n] = gdz2[n];
        }
    float gz1[HID];
    for (int k = 0; k < HID; k++)
        {
        float g_h1 = 0.0f, g_dh1 = 0.0f;
        for (int n = 0; n < HID; n++)
            {
            const float w = q_w(th[O_W2 + n * HID + k], quant);
            g_h1 += w * gz2[n];
            g_dh1 += w * gdz2[n];
            }
        const float gd = g_dh1 * s1[k];
        gz1[k] = g_h1 * s1[k] + g_dh1 * t1[k] * dz1[k];
        row[S_GZ1 + k] = gz1[k];
        row[S_GDZ1 + k] = gd;
        }
    for (int m = 0; m < EMB; m++)
        {
        float g = 0.0f;
        for (int n = 0; n < HID; n++)
            g += q_w(th[O_W1E + n * EMB + m], quant) * gz1[n];
        atomicAdd(grad + O_E + (size_t)p * EMB + m, g);
        }
    }

// out[a * nb + b] = sum_s X[s][xo + a] Y[s][yo + b] (+ X[s][x2o + a] Y[s][y2o + b] when x2o >= 0);
// yo < 0 makes Y the constant 1 (bias sums). Fixed summation order.
__global__ void k_outer(float* __restrict__ out, const float* __restrict__ S, uint32_t B, int xo,
                        int yo, int x2o, int y2o, int na, int nb)
    {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= na * nb)
        return;
    const int a = o / nb, b = o % nb;
    float acc = 0.0f;
    for (uint32_t s = 0; s < B; s++)
        {
        const float* row = S + (size_t)s * SW;
        const float y = yo >= 0 ? row[yo + b] : 1.0f;
        acc += row[xo + a] * y;
        if (x2o >= 0)
            acc += row[x2o + a] * row[y2o + b];
        }
    out[o] = acc;
    }

__global__ void k_loss_sum(const float* __restrict__ S, uint32_t B, double* out)
    {
    __shared__ double sm[32];
    double acc = 0.0;
    for (uint32_t s = threadIdx.x; s < B; s += blockDim.x)
        acc += (double)S[(size_t)s * SW + S_LOSS];
    acc = warp_sum(acc);
    if (threadIdx.x % 32 == 0)
        sm[threadIdx.x / 32] = acc;
    __syncthreads();
    if (threadIdx.x < 32)
        {
        acc = threadIdx.x < blockDim.x / 32 ? sm[threadIdx.x] : 0.0;
        acc = warp_sum(acc);
        if (threadIdx.x == 0)
            *out = acc / (double)B;
        }
    }

__global__ void k_adam(float* __restrict__ th, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
    {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        th[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        }
    }

// ------------------------------------------------------------------------------------------------
// inference
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
    {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
    }

// remainder after rounding to bfloat16 (the low half of a two-term representation)
__device__ __forceinline__ float bf16_rem(float x)
    {
    return x - q_bf16(x);
    }

__global__ void k_prepare(const float* __restrict__ th, uint32_t n_pairs, unsigned char* inf)
    {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t* fw1 = reinterpret_cast<uint32_t*>(inf + I_FW1);
    uint32_t* fw2 = reinterpret_cast<uint32_t*>(inf + I_FW2);
    float* b2 = reinterpret_cast<float*>(inf + I_B2);
    float* w3 = reinterpret_cast<float*>(inf + I_W3);
    float* C = reinterpret_cast<float*>(inf + I_C);
    // operand fragments: B[k][n] = W[n][k]; lane (g, t) holds (k = 2t, 2t+1; n = g) and
    // (k = 2t+8, 2t+9; n = g) of each 16 x 8 tile
    if (tid < 2 * 8 * 32)
        {
        const uint32_t lane = tid % 32, j = (tid / 32) % 8, kk = tid / 256;
        const uint32_t g = lane >> 2, t = lane & 3, n = 8 * j + g, k = 16 * kk + 2 * t;
        const float* W = th + O_W1R + n * RBF;
        fw1[2 * tid] = pack_bf16(W[k], W[k + 1]);
        fw1[2 * tid + 1] = pack_bf16(W[k + 8], W[k + 9]);
        }
    if (tid < 4 * 8 * 32)
        {
        const uint32_t lane = tid % 32, j = (tid / 32) % 8, kk = tid / 256;
        const uint32_t g = lane >> 2, t = lane & 3, n = 8 * j + g, k = 16 * kk + 2 * t;
        const float* W = th + O_W2 + n * HID;
        fw2[2 * tid] = pack_bf16(W[k], W[k + 1]);
        fw2[2 * tid + 1] = pack_bf16(W[k + 8], W[k + 9]);
        }
    if (tid < HID)
        {
        b2[tid] = th[O_B2 + tid];
        w3[tid] = q_bf16(th[O_W3 + tid]);
        }
    // tcgen05 B operands: B[k][n] = W[n][k], stored as the K-major N x K matrix W
    if (tid < HID * RBF)
        {
        const uint32_t n = tid / RBF, k = tid % RBF;
        *reinterpret_cast<__nv_bfloat16*>(inf + I_TW1 + tc_off((int)n, (int)k, RBF))
            = __float2bfloat16_rn(th[O_W1R + n * RBF + k]);
        }
    if (tid < HID * HID)
        {
        const uint32_t n = tid / HID, k = tid % HID;
        *reinterpret_cast<__nv_bfloat16*>(inf + I_TW2 + tc_off((int)n, (int)k, HID))
            = __float2bfloat16_rn(th[O_W2 + n * HID + k]);
        }
    if (tid == 0)
        *reinterpret_cast<float*>(inf + I_B3) = th[O_B3];
    for (uint32_t o = tid; o < n_pairs * HID; o += gridDim.x * blockDim.x)
        {
        const uint32_t p = o / HID, n = o % HID;
        float a = th[O_B1 + n];
        for (int m = 0; m < EMB; m++)
            a += q_bf16(th[O_W1E + n * EMB + m]) * q_bf16(th[O_E + (size_t)p * EMB + m]);
        C[o] = a;
        }
    }

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint2 b)
    {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                 "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
    }

struct MlpSmem
    {
    uint2 fw1[2 * 8 * 32];
    uint2 fw2[4 * 8 * 32];
    float b2[HID];
    float w3[HID];
    float b3;
    };

__device__ void load_smem(MlpSmem& sm, const unsigned char* inf)
    {
    const uint2* f1 = reinterpret_cast<const uint2*>(inf + I_FW1);
    const uint2* f2 = reinterpret_cast<const uint2*>(inf + I_FW2);
    for (int k = threadIdx.x; k < 2 * 8 * 32; k += blockDim.x)
        sm.fw1[k] = f1[k];
    for (int k = threadIdx.x; k < 4 * 8 * 32; k += blockDim.x)
        sm.fw2[k] = f2[k];
    for (int k = threadIdx.x; k < HID; k += blockDim.x)
        {
        sm.b2[k] = reinterpret_cast<const float*>(inf + I_B2)[k];
        sm.w3[k] = reinterpret_cast<const float*>(inf + I_W3)[k];
        }
    if (threadIdx.x == 0)
        sm.b3 = *reinterpret_cast<const float*>(inf + I_B3);
    __syncthreads();
    }

__device__ __forceinline__ float logistic(float z)
    {
    return __fdividef(1.0f, 1.0f + __expf(-z));
    }

// One tile of 16 pairs. Lane (g, t) supplies rows g (p0, r0) and g + 8 (p1, r1); all four lanes
// of a row group receive U and dU/dr of both rows.
template<bool SPLIT>
__device__ __forceinline__ void mlp_tile(const MlpSmem& sm, const float* __restrict__ C,
                                         uint32_t p0, uint32_t p1, float r0, float r1,
                                         float r_min, float h, float gamma, float& U0, float& U1,
                                         float& D0, float& D1)
    {
    const uint32_t lane = threadIdx.x % 32, t = lane & 3;
    float acc[8][4], dacc[8][4];
    const float* C0 = C + (size_t)p0 * HID;
    const float* C1 = C + (size_t)p1 * HID;
#pragma unroll
    for (int j = 0; j < 8; j++)
        {
        const float2 c0 = __ldg(reinterpret_cast<const float2*>(C0 + 8 * j + 2 * t));
        const float2 c1 = __ldg(reinterpret_cast<const float2*>(C1 + 8 * j + 2 * t));
        acc[j][0] = c0.x;
        acc[j][1] = c0.y;
        acc[j][2] = c1.x;
        acc[j][3] = c1.y;
        dacc[j][0] = dacc[j][1] = dacc[j][2] = dacc[j][3] = 0.0f;
        }
    // layer 1: radial features of both rows at columns 16kk + 2t + {0, 1, 8, 9}
#pragma unroll
    for (int kk = 0; kk < 2; kk++)
        {
        float ph[2][4], dph[2][4];
#pragma unroll
        for (int q = 0; q < 4; q++)
            {
            const int col = 16 * kk + 2 * t + (q & 1) + (q >> 1) * 8;
            const float mu = r_min + (float)col * h;
            const float d0 = r0 - mu, d1 = r1 - mu;
            const float e0 = __expf(-gamma * d0 * d0), e1 = __expf(-gamma * d1 * d1);
            ph[0][q] = e0;
            ph[1][q] = e1;
            dph[0][q] = -2.0f * gamma * d0 * e0;
            dph[1][q] = -2.0f * gamma * d1 * e1;
            }
        uint32_t a[4], da[4];
        a[0] = pack_bf16(ph[0][0], ph[0][1]);
        a[1] = pack_bf16(ph[1][0], ph[1][1]);
        a[2] = pack_bf16(ph[0][2], ph[0][3]);
        a[3] = pack_bf16(ph[1][2], ph[1][3]);
        da[0] = pack_bf16(dph[0][0], dph[0][1]);
        da[1] = pack_bf16(dph[1][0], dph[1][1]);
        da[2] = pack_bf16(dph[0][2], dph[0][3]);
        da[3] = pack_bf16(dph[1][2], dph[1][3]);
#pragma unroll
        for (int j = 0; j < 8; j++)
            {
            const uint2 b = sm.fw1[(kk * 8 + j) * 32 + lane];
            mma16816(acc[j], a, b);
            mma16816(dacc[j], da, b);
            }
        if (SPLIT)
            {
            a[0] = pack_bf16(bf16_rem(ph[0][0]), bf16_rem(ph[0][1]));
            a[1] = pack_bf16(bf16_rem(ph[1][0]), bf16_rem(ph[1][1]));
            a[2] = pack_bf16(bf16_rem(ph[0][2]), bf16_rem(ph[0][3]));
            a[3] = pack_bf16(bf16_rem(ph[1][2]), bf16_rem(ph[1][3]));
            da[0] = pack_bf16(bf16_rem(dph[0][0]), bf16_rem(dph[0][1]));
            da[1] = pack_bf16(bf16_rem(dph[1][0]), bf16_rem(dph[1][1]));
            da[2] = pack_bf16(bf16_rem(dph[0][2]), bf16_rem(dph[0][3]));
            da[3] = pack_bf16(bf16_rem(dph[1][2]), bf16_rem(dph[1][3]));
#pragma unroll
            for (int j = 0; j < 8; j++)
                {
                const uint2 b = sm.fw1[(kk * 8 + j) * 32 + lane];
                mma16816(acc[j], a, b);
                mma16816(dacc[j], da, b);
                }
            }
        }
    // silu and its derivative; the accumulators become the next layer's A fragments
    uint32_t a2[4][4], da2[4][4], a2l[4][4], da2l[4][4];
#pragma unroll
    for (int j = 0; j < 8; j++)
        {
        float hv[4], dv[4];
#pragma unroll
        for (int e = 0; e < 4; e++)
            {
            const float z = acc[j][e];
            const float s = logistic(z);
            hv[e] = z * s;
            dv[e] = s * (1.0f + z * (1.0f - s)) * dacc[j][e];
            }
        const int kk = j >> 1, hi = (j & 1) * 2;
        a2[kk][hi] = pack_bf16(hv[0], hv[1]);
        a2[kk][hi + 1] = pack_bf16(hv[2], hv[3]);
        da2[kk][hi] = pack_bf16(dv[0], dv[1]);
        da2[kk][hi + 1] = pack_bf16(dv[2], dv[3]);
        if (SPLIT)
            {
            a2l[kk][hi] = pack_bf16(bf16_rem(hv[0]), bf16_rem(hv[1]));
            a2l[kk][hi + 1] = pack_bf16(bf16_rem(hv[2]), bf16_rem(hv[3]));
            da2l[kk][hi] = pack_bf16(bf16_rem(dv[0]), bf16_rem(dv[1]));
            da2l[kk][hi + 1] = pack_bf16(bf16_rem(dv[2]), bf16_rem(dv[3]));
            }
        }
    // layer 2
#pragma unroll
    for (int j = 0; j < 8; j++)
        {
        const float2 bb = *reinterpret_cast<const float2*>(sm.b2 + 8 * j + 2 * t);
        acc[j][0] = bb.x;
        acc[j][1] = bb.y;
        acc[j][2] = bb.x;
        acc[j][3] = bb.y;
        dacc[j][0] = dacc[j][1] = dacc[j][2] = dacc[j][3] = 0.0f;
        }
#pragma unroll
    for (int kk = 0; kk < 4; kk++)
#pragma unroll
        for (int j = 0; j < 8; j++)
            {
            const uint2 b = sm.fw2[(kk * 8 + j) * 32 + lane];
            mma16816(acc[j], a2[kk], b);
            mma16816(dacc[j], da2[kk], b);
            if (SPLIT)
                {
                mma16816(acc[j], a2l[kk], b);
                mma16816(dacc[j], da2l[kk], b);
                }
            }
    // output layer: U = w3 . silu(z2) + b3, dU = w3 . silu'(z2) dz2
    float u0 = 0.f, u1 = 0.f, g0 = 0.f, g1 = 0.f;
#pragma unroll
    for (int j = 0; j < 8; j++)
        {
        const float2 w = *reinterpret_cast<const float2*>(sm.w3 + 8 * j + 2 * t);
#pragma unroll
        for (int e = 0; e < 4; e++)
            {
            const float z = acc[j][e];
            const float s = logistic(z);
            const float hv = z * s;
            const float dv = s * (1.0f + z * (1.0f - s)) * dacc[j][e];
            const float we = (e & 1) ? w.y : w.x;
            if (e < 2)
                {
                u0 += we * hv;
                g0 += we * dv;
                }
            else
                {
                u1 += we * hv;
                g1 += we * dv;
                }
            }
        }
#pragma unroll
    for (int o = 1; o < 4; o <<= 1)
        {
        u0 += __shfl_xor_sync(0xffffffffu, u0, o);
        u1 += __shfl_xor_sync(0xffffffffu, u1, o);
        g0 += __shfl_xor_sync(0xffffffffu, g0, o);
        g1 += __shfl_xor_sync(0xffffffffu, g1, o);
        }
    U0 = u0 + sm.b3;
    U1 = u1 + sm.b3;
    D0 = g0;
    D1 = g1;
    }

template<bool SPLIT>
__global__ void __launch_bounds__(128)
    k_eval(const unsigned char* __restrict__ inf, uint32_t n_pairs, float r_min, float r_cut,
           const uint32_t* __restrict__ pair, const float* __restrict__ rr, uint32_t n,
           float* __restrict__ U, float* __restrict__ dU)
    {
    __shared__ MlpSmem sm;
    load_smem(sm, inf);
    const float* C = reinterpret_cast<const float*>(inf + I_C);
    const float h = (r_cut - r_min) / (float)(RBF - 1);
    const float gamma = 1.0f / (2.0f * h * h);
    const uint32_t lane = threadIdx.x % 32, g = lane >> 2;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t tile = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; tile * 16 < n;
         tile += warps)
        {
        const uint32_t s0 = tile * 16 + g, s1 = s0 + 8;
        const bool v0 = s0 < n, v1 = s1 < n;
        const uint32_t p0 = v0 ? min(pair[s0], n_pairs - 1) : 0u;
        const uint32_t p1 = v1 ? min(pair[s1], n_pairs - 1) : 0u;
        const float r0 = v0 ? rr[s0] : r_min, r1 = v1 ? rr[s1] : r_min;
        float U0, U1, D0, D1;
        mlp_tile<SPLIT>(sm, C, p0, p1, r0, r1, r_min, h, gamma, U0, U1, D0, D1);
        if ((lane & 3) == 0)
            {
            if (v0)
                {
                U[s0] = U0;
                dU[s0] = D0;
                }
            if (v1)
                {
                U[s1] = U1;
                dU[s1] = D1;
                }
            }
        }
    }

// Pair list: for each particle i, its neighbours j > i with r_min^2 <= r^2 < r_cut^2, stored
// contiguously (a warp counts its particles' pairs, claims one range, and each lane writes its
// own pairs at its prefix offset).
__device__ __forceinline__ float pair_rsq(const float4& pi, const float4& pj, const gb_box& box)
    {
    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    min_image(box, dx, dy, dz);
    return dx * dx + dy * dy + dz * dz;
    }

__global__ void __launch_bounds__(256)
    k_pair_list(const float4* __restrict__ pos, unsigned int N, gb_box box,
                const unsigned int* __restrict__ n_neigh, const uint4* __restrict__ nl4,
                uint64_t stride, float rminsq, float rcutsq, uint2* __restrict__ pairs,
                unsigned int* __restrict__ count)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned int lane = threadIdx.x % 32;
    const bool active = i < N;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    unsigned int nn = 0;
    if (active)
        {
        pi = pos[i];
        nn = n_neigh[i];
        }
    auto visit = [&](auto&& hit) {
        for (unsigned int b = 0; b < (nn + 3) / 4; b++)
            {
            const uint4 q = nl4[(uint64_t)b * stride + i];
            const unsigned int js[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int e = 0; e < 4; e++)
                if (4 * b + e < nn && js[e] > i)
                    {
                    const float rsq = pair_rsq(pi, pos[js[e]], box);
                    if (rsq >= rminsq && rsq < rcutsq)
                        hit(js[e]);
                    }
            }
    };
    unsigned int c = 0;
    if (active)
        visit([&](unsigned int) { c++; });
    unsigned int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
        {
        const unsigned int v = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o)
            incl += v;
        }
    unsigned int base = 0;
    if (lane == 31)
        base = atomicAdd(count, incl);
    base = __shfl_sync(0xffffffffu, base, 31);
    unsigned int w = base + incl - c;
    if (active)
        visit([&](unsigned int j) { pairs[w++] = make_uint2(i, j); });
    }

template<bool SPLIT>
__global__ void __launch_bounds__(128)
    k_mlp_forces(const unsigned char* __restrict__ inf, const float4* __restrict__ pos,
                 gb_box box, unsigned int ntypes, uint32_t n_pairs, float r_min, float r_cut,
                 const uint2* __restrict__ pairs, const unsigned int* __restrict__ count,
                 float4* __restrict__ force)
    {
    __shared__ MlpSmem sm;
    __shared__ float4 s_f[4][16];
    __shared__ unsigned int s_i[4][16];
    load_smem(sm, inf);
    const unsigned int n = *count;
    const float* C = reinterpret_cast<const float*>(inf + I_C);
    const float h = (r_cut - r_min) / (float)(RBF - 1);
    const float gamma = 1.0f / (2.0f * h * h);
    const uint32_t lane = threadIdx.x % 32, g = lane >> 2, t = lane & 3, wib = threadIdx.x / 32;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t tile = blockIdx.x * (blockDim.x / 32) + wib; tile * 16 < n; tile += warps)
        {
        // geometry of rows g and g + 8
        float3 dv[2];
        float r[2];
        uint32_t p[2], ii[2], jj[2];
        bool v[2];
#pragma unroll
        for (int k = 0; k < 2; k++)
            {
            const uint32_t s = tile * 16 + g + 8 * k;
            v[k] = s < n;
            const uint2 pr = v[k] ? pairs[s] : make_uint2(0u, 0u);
            ii[k] = pr.x;
            jj[k] = pr.y;
            const float4 pi = pos[pr.x], pj = pos[pr.y];
            float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            min_image(box, dx, dy, dz);
            dv[k] = make_float3(dx, dy, dz);
            r[k] = v[k] ? sqrtf(dx * dx + dy * dy + dz * dz) : r_min;
            const unsigned int ta = __float_as_uint(pi.w), tb = __float_as_uint(pj.w);
            const unsigned int a = min(ta, tb), b = max(ta, tb);
            p[k] = v[k] ? min(a * ntypes - a * (a - 1) / 2 + (b - a), n_pairs - 1) : 0u;
            }
        float U0, U1, D0, D1;
        mlp_tile<SPLIT>(sm, C, p[0], p[1], r[0], r[1], r_min, h, gamma, U0, U1, D0, D1);
        // lane t = k of each row group owns row g + 8k: force on i, reaction on j
        if (t < 2)
            {
            const int k = t;
            const float U = k ? U1 : U0, D = k ? D1 : D0;
            const float fd = v[k] ? -D / r[k] : 0.0f;
            const float4 f = make_float4(fd * dv[k].x, fd * dv[k].y, fd * dv[k].z,
                                         v[k] ? 0.5f * U : 0.0f);
            s_f[wib][g + 8 * k] = f;
            s_i[wib][g + 8 * k] = v[k] ? ii[k] : 0xffffffffu;
            if (v[k])
                atomicAdd(force + jj[k], make_float4(-f.x, -f.y, -f.z, f.w));
            }
        __syncwarp();
        // rows of one particle i are consecutive: one atomic per run of equal i
        if (lane < 16)
            {
            const unsigned int me = s_i[wib][lane];
            const bool head = me != 0xffffffffu && (lane == 0 || s_i[wib][lane - 1] != me);
            if (head)
                {
                float4 acc = s_f[wib][lane];
                for (uint32_t q = lane + 1; q < 16 && s_i[wib][q] == me; q++)
                    {
                    const float4 o = s_f[wib][q];
                    acc.x += o.x;
                    acc.y += o.y;
                    acc.z += o.z;
                    acc.w += o.w;
                    }
                atomicAdd(force + me, acc);
                }
            }
        __syncwarp();
        }
    }

// ------------------------------------------------------------------------------------------------
// tcgen05 inference: tiles of 128 pairs, one pair per TMEM lane
// ------------------------------------------------------------------------------------------------
// A CTA of 256 threads walks tiles of 128 pairs. Rows (pairs) are the M = 128 lanes of the
// tensor memory; warp w serves lanes 32 (w % 4) .. + 31 and hidden units 32 (w / 4) .. + 31, so
// two threads share a row. Per tile: the radial features (value and r-derivative, each as a
// bfloat16 high part and its bfloat16 remainder) go to shared memory as K-major operands; one
// thread issues the layer-1 products (M = 128, N = 64, K = 32 in two K = 16 steps, high and low
// parts accumulated into the same FP32 accumulator) into tensor memory and commits them to an
// mbarrier; after the wait every thread reads its row's accumulators with tcgen05.ld, adds C[p],
// applies SiLU and its derivative and writes the layer-2 operands (K = 64) over the layer-1 ones;
// the layer-2 products go to the other two accumulators; the output layer, the radial derivative
// and the forces follow in registers, and each pair adds its force to both particles with float4
// atomics. C[p] is loaded before the layer-1 products and the next tile's pair one tile ahead.
// Tensor memory: 4 accumulators x 64 FP32 columns = 256 columns per CTA, two CTAs per SM. Every wait on the mbarrier is bounded; a wait that runs out records an error
// and all threads leave the tile loop together, free the tensor memory and return.
constexpr int TC_THREADS = 256;
constexpr uint32_t TC_OP = 0;                        // operands: 4 x (128 x 64) bf16 = 64 KB
constexpr uint32_t TC_W1 = 65536;                    // W1r image, 64 x 32 bf16
constexpr uint32_t TC_W2 = TC_W1 + 4096;             // W2 image, 64 x 64 bf16
constexpr uint32_t TC_B2 = TC_W2 + 8192;             // b2, w3 (64 floats each)
constexpr uint32_t TC_W3 = TC_B2 + 256;
constexpr uint32_t TC_PART = TC_W3 + 256;            // 128 x float2: second-half partial sums
constexpr uint32_t TC_MISC = TC_PART + 1024;         // mbarrier, tensor-memory base, b3
constexpr uint32_t TC_SMEM = TC_MISC + 64;
constexpr uint32_t TC_TMEM_COLS = 256;
// instruction descriptor (kind::f16): FP32 accumulator, BF16 A and B, both K-major,
// N = 64 (N >> 3 at bit 17), M = 128 (M >> 4 at bit 24)
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17)
                              | ((128u >> 4) << 24);
constexpr uint32_t TC_WAIT_LIMIT = 1u << 24;

__device__ __forceinline__ uint32_t smem_addr(const void* p)
    {
    return (uint32_t)__cvta_generic_to_shared(p);
    }

// shared-memory matrix descriptor of a K-major operand with K columns (no swizzle)
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, int K)
    {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16)
           | ((uint64_t)(((uint32_t)K / 8u * 128u) >> 4) << 32) | ((uint64_t)1 << 46);
    }

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc)
    {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                 ::"r"(tmem_d), "l"(a), "l"(b), "r"(TC_IDESC), "r"(acc));
    }

__device__ __forceinline__ void tc_commit(uint64_t* mbar)
    {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(smem_addr(mbar)));
    }

// bounded wait for the mbarrier phase with the given parity; true when it completed
__device__ __forceinline__ bool tc_wait(uint64_t* mbar, uint32_t parity)
    {
    uint32_t done = 0;
    for (uint32_t it = 0; it < TC_WAIT_LIMIT && !done; it++)
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     "selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(smem_addr(mbar)), "r"(parity));
    return done != 0;
    }

// 32 consecutive FP32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32])
    {
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
                 "%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,"
                 "%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                   "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),
                   "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                   "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                   "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int c = 0; c < 32; c++)
        v[c] = __uint_as_float(r[c]);
    }

// eight values as a 16-byte row of a core matrix: the high bfloat16 parts, or the remainders
__device__ __forceinline__ uint4 bf16x8(const float* v, bool remainder)
    {
    float x[8];
#pragma unroll
    for (int e = 0; e < 8; e++)
        x[e] = remainder ? bf16_rem(v[e]) : v[e];
    return make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]),
                      pack_bf16(x[6], x[7]));
    }

template<bool SPLIT>
__global__ void __launch_bounds__(TC_THREADS, 2)
    k_mlp_forces_tc(const unsigned char* __restrict__ inf, const float4* __restrict__ pos,
                    gb_box box, unsigned int ntypes, uint32_t n_pairs, float r_min, float r_cut,
                    const uint2* __restrict__ pairs, const unsigned int* __restrict__ count,
                    float4* __restrict__ force, uint32_t* __restrict__ err)
    {
    extern __shared__ __align__(1024) unsigned char sm[];
    const uint32_t tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const uint32_t quarter = warp & 3u, half = warp >> 2;
    const uint32_t row = 32u * quarter + lane;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + TC_MISC);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + TC_MISC + 8);
    float* b3s = reinterpret_cast<float*>(sm + TC_MISC + 12);
    const float* b2 = reinterpret_cast<const float*>(sm + TC_B2);
    const float* w3 = reinterpret_cast<const float*>(sm + TC_W3);
    float2* part = reinterpret_cast<float2*>(sm + TC_PART);

    // weights and biases into shared memory
    {
    const uint4* src1 = reinterpret_cast<const uint4*>(inf + I_TW1);
    const uint4* src2 = reinterpret_cast<const uint4*>(inf + I_TW2);
    uint4* dst1 = reinterpret_cast<uint4*>(sm + TC_W1);
    uint4* dst2 = reinterpret_cast<uint4*>(sm + TC_W2);
    for (uint32_t k = tid; k < 4096 / 16; k += TC_THREADS)
        dst1[k] = src1[k];
    for (uint32_t k = tid; k < 8192 / 16; k += TC_THREADS)
        dst2[k] = src2[k];
    if (tid < HID)
        {
        reinterpret_cast<float*>(sm + TC_B2)[tid] = reinterpret_cast<const float*>(inf + I_B2)[tid];
        reinterpret_cast<float*>(sm + TC_W3)[tid] = reinterpret_cast<const float*>(inf + I_W3)[tid];
        }
    if (tid == 0)
        {
        *b3s = *reinterpret_cast<const float*>(inf + I_B3);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
        }
    if (warp == 0)
        {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_addr(tmem_slot)), "r"(TC_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
        }
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    }
    const uint32_t tmem = *tmem_slot;
    const uint32_t t_lane = tmem + ((32u * quarter) << 16);
    const uint32_t op = smem_addr(sm + TC_OP), w1a = smem_addr(sm + TC_W1),
                   w2a = smem_addr(sm + TC_W2);
    const float* C = reinterpret_cast<const float*>(inf + I_C);
    const float hstep = (r_cut - r_min) / (float)(RBF - 1);
    const float gamma = 1.0f / (2.0f * hstep * hstep);
    const unsigned int n = *count;
    uint32_t parity = 0;
    // the pair of this thread's row in the next tile is loaded one tile ahead
    uint2 pr_next = make_uint2(0u, 0u);
    if (blockIdx.x * 128u + row < n)
        pr_next = pairs[blockIdx.x * 128u + row];

    for (uint32_t tile = blockIdx.x; tile * 128u < n; tile += gridDim.x)
        {
        // geometry of this thread's row (both threads of a row compute it)
        const uint32_t s = tile * 128u + row;
        const bool v = s < n;
        const uint2 pr = v ? pr_next : make_uint2(0u, 0u);
        const float4 pi = pos[pr.x], pj = pos[pr.y];
        float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        min_image(box, dx, dy, dz);
        const float r = v ? sqrtf(dx * dx + dy * dy + dz * dz) : r_min;
        uint32_t p;
        {
        const unsigned int ta = __float_as_uint(pi.w), tb = __float_as_uint(pj.w);
        const unsigned int a = min(ta, tb), b = max(ta, tb);
        p = v ? min(a * ntypes - a * (a - 1) / 2 + (b - a), n_pairs - 1) : 0u;
        }
        // this row's first-layer offsets, in flight while the layer-1 products run
        float4 cv[8];
        {
        const float4* Cp = reinterpret_cast<const float4*>(C + (size_t)p * HID + 32 * half);
#pragma unroll
        for (int q = 0; q < 8; q++)
            cv[q] = __ldg(Cp + q);
        }
        // layer-1 operands: features 16 half .. 16 half + 15 of this row
        {
        float ph[16], dph[16];
#pragma unroll
        for (int q = 0; q < 16; q++)
            {
            const int k = 16 * (int)half + q;
            const float mu = r_min + (float)k * hstep;
            const float d = r - mu;
            const float e = __expf(-gamma * d * d);
            ph[q] = e;
            dph[q] = -2.0f * gamma * d * e;
            }
#pragma unroll
        for (int g = 0; g < 2; g++)
            {
            const uint32_t off = tc_off((int)row, 16 * (int)half + 8 * g, RBF);
            *reinterpret_cast<uint4*>(sm + TC_OP + 0 * 8192 + off) = bf16x8(ph + 8 * g, false);
            *reinterpret_cast<uint4*>(sm + TC_OP + 2 * 8192 + off) = bf16x8(dph + 8 * g, false);
            if (SPLIT)
                {
                *reinterpret_cast<uint4*>(sm + TC_OP + 1 * 8192 + off) = bf16x8(ph + 8 * g, true);
                *reinterpret_cast<uint4*>(sm + TC_OP + 3 * 8192 + off) = bf16x8(dph + 8 * g, true);
                }
            }
        }
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (tid == 0)
            {
#pragma unroll
            for (int k = 0; k < RBF / 16; k++)
                {
                const uint64_t bw = tc_desc(w1a + 256u * k, RBF);
                tc_mma(tmem + 0, tc_desc(op + 0 * 8192 + 256u * k, RBF), bw, k > 0);
                tc_mma(tmem + 64, tc_desc(op + 2 * 8192 + 256u * k, RBF), bw, k > 0);
                if (SPLIT)
                    {
                    tc_mma(tmem + 0, tc_desc(op + 1 * 8192 + 256u * k, RBF), bw, 1u);
                    tc_mma(tmem + 64, tc_desc(op + 3 * 8192 + 256u * k, RBF), bw, 1u);
                    }
                }
            tc_commit(mbar);
            }
        if (!__syncthreads_and(tc_wait(mbar, parity)))
            {
            if (tid == 0)
                atomicExch(err, 1u);
            break;
            }
        parity ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;");
        // layer 1 epilogue: hidden units 32 half .. 32 half + 31 of this row
        {
        float z[32], dzv[32];
        tc_ld32(t_lane + 0 + 32u * half, z);
        tc_ld32(t_lane + 64 + 32u * half, dzv);
#pragma unroll
        for (int q = 0; q < 8; q++)
            {
            const float4 c = cv[q];
            z[4 * q] += c.x;
            z[4 * q + 1] += c.y;
            z[4 * q + 2] += c.z;
            z[4 * q + 3] += c.w;
            }
#pragma unroll
        for (int c = 0; c < 32; c++)
            {
            const float sg = logistic(z[c]);
            const float hv = z[c] * sg;
            dzv[c] = sg * (1.0f + z[c] * (1.0f - sg)) * dzv[c];
            z[c] = hv;
            }
#pragma unroll
        for (int g = 0; g < 4; g++)
            {
            const uint32_t off = tc_off((int)row, 32 * (int)half + 8 * g, HID);
            *reinterpret_cast<uint4*>(sm + TC_OP + 0 * 16384 + off) = bf16x8(z + 8 * g, false);
            *reinterpret_cast<uint4*>(sm + TC_OP + 2 * 16384 + off) = bf16x8(dzv + 8 * g, false);
            if (SPLIT)
                {
                *reinterpret_cast<uint4*>(sm + TC_OP + 1 * 16384 + off) = bf16x8(z + 8 * g, true);
                *reinterpret_cast<uint4*>(sm + TC_OP + 3 * 16384 + off)
                    = bf16x8(dzv + 8 * g, true);
                }
            }
        }
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (tid == 0)
            {
#pragma unroll
            for (int k = 0; k < HID / 16; k++)
                {
                const uint64_t bw = tc_desc(w2a + 256u * k, HID);
                tc_mma(tmem + 128, tc_desc(op + 0 * 16384 + 256u * k, HID), bw, k > 0);
                tc_mma(tmem + 192, tc_desc(op + 2 * 16384 + 256u * k, HID), bw, k > 0);
                if (SPLIT)
                    {
                    tc_mma(tmem + 128, tc_desc(op + 1 * 16384 + 256u * k, HID), bw, 1u);
                    tc_mma(tmem + 192, tc_desc(op + 3 * 16384 + 256u * k, HID), bw, 1u);
                    }
                }
            tc_commit(mbar);
            }
        if (!__syncthreads_and(tc_wait(mbar, parity)))
            {
            if (tid == 0)
                atomicExch(err, 1u);
            break;
            }
        parity ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;");
        {
        const uint32_t sn = (tile + gridDim.x) * 128u + row;
        if (sn < n)
            pr_next = pairs[sn];
        }
        // layer 2 epilogue and the output layer: U = w3 . silu(z2) + b3, dU = w3 . silu'(z2) dz2
        float u = 0.0f, du = 0.0f;
        {
        float z[32], dzv[32];
        tc_ld32(t_lane + 128 + 32u * half, z);
        tc_ld32(t_lane + 192 + 32u * half, dzv);
#pragma unroll
        for (int c = 0; c < 32; c++)
            {
            const int k = 32 * (int)half + c;
            const float zz = z[c] + b2[k];
            const float sg = logistic(zz);
            u += w3[k] * (zz * sg);
            du += w3[k] * (sg * (1.0f + zz * (1.0f - sg)) * dzv[c]);
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        if (half == 1)
            part[row] = make_float2(u, du);
        __syncthreads();
        if (half == 0 && v)
            {
            const float2 o = part[row];
            const float U = u + o.x + *b3s, D = du + o.y;
            const float fd = -D / r;
            const float4 f = make_float4(fd * dx, fd * dy, fd * dz, 0.5f * U);
            atomicAdd(force + pr.x, f);
            atomicAdd(force + pr.y, make_float4(-f.x, -f.y, -f.z, f.w));
            }
        }
    // every thread has finished its tensor-memory loads (or left the loop together)
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                     ::"r"(tmem), "r"(TC_TMEM_COLS));
    }
} // namespace
} // namespace gb

using namespace gb;

extern "C"
    {
    size_t gb_mlp_param_count(uint32_t n_pairs)
        {
        return param_count(n_pairs);
        }

    size_t gb_mlp_train_scratch_bytes(uint32_t batch)
        {
        return (size_t)batch * SW * sizeof(float);
        }

    int gb_mlp_loss_grad(const float* d_theta, uint32_t n_pairs, float r_min, float r_cut,
                         const uint32_t* d_pair, const float* d_r, const float* d_U,
                         const float* d_F, uint32_t batch, float lam, int quant, float* d_grad,
                         double* d_loss, void* d_scratch, void* stream)
        {
        GB_REQUIRE(d_theta && d_pair && d_r && d_U && d_F && d_grad && d_loss && d_scratch,
                   "gb_mlp_loss_grad: null argument");
        GB_REQUIRE(n_pairs > 0 && batch > 0, "gb_mlp_loss_grad: empty batch or no type pairs");
        GB_REQUIRE(r_cut > r_min, "gb_mlp_loss_grad: r_cut must exceed r_min");
        GB_REQUIRE(quant >= 0 && quant <= 2, "gb_mlp_loss_grad: quant must be 0, 1 or 2");
        cudaStream_t s = (cudaStream_t)stream;
        float* S = static_cast<float*>(d_scratch);
        if (cudaMemsetAsync(d_grad, 0, param_count(n_pairs) * sizeof(float), s) != cudaSuccess)
            return fail(GB_ERR_CUDA, "gb_mlp_loss_grad: memset");
        k_train_sample<<<div_up(batch, 128), 128, 0, s>>>(d_theta, n_pairs, r_min, r_cut, d_pair,
                                                          d_r, d_U, d_F, batch, lam, quant,
                                                          d_grad, S);
        auto outer = [&](int off, int xo, int yo, int x2o, int y2o, int na, int nb) {
            k_outer<<<div_up(na * nb, 128), 128, 0, s>>>(d_grad + off, S, batch, xo, yo, x2o,
                                                         y2o, na, nb);
        };
        outer(O_W1E, S_GZ1, S_E, -1, -1, HID, EMB);
        outer(O_W1R, S_GZ1, S_PHI, S_GDZ1, S_DPHI, HID, RBF);
        outer(O_B1, S_GZ1, -1, -1, -1, HID, 1);
        outer(O_W2, S_GZ2, S_H1, S_GDZ2, S_DH1, HID, HID);
        outer(O_B2, S_GZ2, -1, -1, -1, HID, 1);
        outer(O_W3, S_GU, S_H2, S_GD, S_DH2, 1, HID);
        outer(O_B3, S_GU, -1, -1, -1, 1, 1);
        k_loss_sum<<<1, 256, 0, s>>>(S, batch, d_loss);
        return check_launch("gb_mlp_loss_grad");
        }

    int gb_mlp_adam(float* d_theta, const float* d_grad, float* d_m, float* d_v, size_t n,
                    float lr, float beta1, float beta2, float eps, uint32_t step, void* stream)
        {
        GB_REQUIRE(d_theta && d_grad && d_m && d_v && step > 0, "gb_mlp_adam: bad argument");
        const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
        k_adam<<<div_up(n, 256) < 1024 ? div_up(n, 256) : 1024, 256, 0, (cudaStream_t)stream>>>(
            d_theta, d_grad, d_m, d_v, n, lr, beta1, beta2, eps, c1, c2);
        return check_launch("gb_mlp_adam");
        }

    size_t gb_mlp_infer_bytes(uint32_t n_pairs)
        {
        return I_C + (size_t)n_pairs * HID * sizeof(float);
        }

    int gb_mlp_prepare(const float* d_theta, uint32_t n_pairs, void* d_infer, void* stream)
        {
        GB_REQUIRE(d_theta && d_infer && n_pairs > 0, "gb_mlp_prepare: bad argument");
        const unsigned int work = n_pairs * HID > HID * HID ? n_pairs * HID : HID * HID;
        k_prepare<<<div_up(work, 256), 256, 0, (cudaStream_t)stream>>>(
            d_theta, n_pairs, static_cast<unsigned char*>(d_infer));
        return check_launch("gb_mlp_prepare");
        }

    int gb_mlp_eval(const void* d_infer, uint32_t n_pairs, float r_min, float r_cut,
                    int act_split, const uint32_t* d_pair, const float* d_r, uint32_t n,
                    float* d_U, float* d_dU, void* stream)
        {
        GB_REQUIRE(d_infer && d_pair && d_r && d_U && d_dU && n_pairs > 0,
                   "gb_mlp_eval: null argument");
        if (n == 0)
            return GB_OK;
        const unsigned int grid = div_up(div_up(n, 16), 4);
        const unsigned char* inf = static_cast<const unsigned char*>(d_infer);
        if (act_split)
            k_eval<true><<<grid, 128, 0, (cudaStream_t)stream>>>(inf, n_pairs, r_min, r_cut,
                                                                 d_pair, d_r, n, d_U, d_dU);
        else
            k_eval<false><<<grid, 128, 0, (cudaStream_t)stream>>>(inf, n_pairs, r_min, r_cut,
                                                                  d_pair, d_r, n, d_U, d_dU);
        return check_launch("gb_mlp_eval");
        }

    size_t gb_mlp_forces_scratch_bytes(unsigned int N, unsigned int Nmax)
        {
        // pair count word, then one (i, j) pair per full-list slot at most
        return 256 + (size_t)N * Nmax * sizeof(uint2);
        }

    int gb_mlp_forces(const gb_mlp_force_args* a, void* stream)
        {
        GB_REQUIRE(a && a->d_force && a->d_pos && a->d_n_neigh && a->d_nlist && a->d_infer
                       && a->d_scratch,
                   "gb_mlp_forces: null argument");
        GB_REQUIRE(a->ntypes > 0 && a->r_cut > a->r_min && a->r_min >= 0.0f,
                   "gb_mlp_forces: bad types or radii");
        GB_REQUIRE(a->stride >= a->N && a->stride % 32 == 0, "gb_mlp_forces: bad stride");
        cudaStream_t s = (cudaStream_t)stream;
        const uint32_t n_pairs = a->ntypes * (a->ntypes + 1) / 2;
        unsigned char* sc = static_cast<unsigned char*>(a->d_scratch);
        unsigned int* count = reinterpret_cast<unsigned int*>(sc);
        uint2* pairs = reinterpret_cast<uint2*>(sc + 256);
        // count word, then the tensor-core path's error word
        if (cudaMemsetAsync(count, 0, 2 * sizeof(unsigned int), s) != cudaSuccess
            || cudaMemsetAsync(a->d_force, 0, (size_t)a->N * 16, s) != cudaSuccess)
            return fail(GB_ERR_CUDA, "gb_mlp_forces: memset");
        if (a->N == 0)
            return GB_OK;
        const float4* pos = reinterpret_cast<const float4*>(a->d_pos);
        k_pair_list<<<div_up(a->N, 256), 256, 0, s>>>(
            pos, a->N, a->box, a->d_n_neigh, reinterpret_cast<const uint4*>(a->d_nlist),
            a->stride, a->r_min * a->r_min, a->r_cut * a->r_cut, pairs, count);
        const unsigned char* inf = static_cast<const unsigned char*>(a->d_infer);
        float4* force = reinterpret_cast<float4*>(a->d_force);
        if (a->mma_sync == 0)
            {
            // tcgen05 tiles: two CTAs per SM (256 tensor-memory columns each)
            static int sms = 0;
            if (sms == 0)
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
            auto kern = a->act_split ? k_mlp_forces_tc<true> : k_mlp_forces_tc<false>;
            static bool attr = false;
            if (!attr)
                {
                cudaFuncSetAttribute(k_mlp_forces_tc<true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
                cudaFuncSetAttribute(k_mlp_forces_tc<false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
                attr = true;
                }
            kern<<<2u * (unsigned)sms, TC_THREADS, TC_SMEM, s>>>(
                inf, pos, a->box, a->ntypes, n_pairs, a->r_min, a->r_cut, pairs, count, force,
                count + 1);
            return check_launch("gb_mlp_forces (tcgen05)");
            }
        const unsigned int grid = 152u * 16u;
        if (a->act_split)
            k_mlp_forces<true><<<grid, 128, 0, s>>>(inf, pos, a->box, a->ntypes, n_pairs,
                                                    a->r_min, a->r_cut, pairs, count, force);
        else
            k_mlp_forces<false><<<grid, 128, 0, s>>>(inf, pos, a->box, a->ntypes, n_pairs,
                                                     a->r_min, a->r_cut, pairs, count, force);
        return check_launch("gb_mlp_forces");
        }
    }
