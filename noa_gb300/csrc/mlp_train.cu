/*
 * Learned DCS surrogate: training-data preparation, forward / backward / Adam
 * kernels and the C ABI of the model object (include/noa_dcs.h,
 * noa_dcs_mlp_*).  No counterpart in the reference.
 *
 * Training runs on the 5th-generation tensor cores (tcgen05.mma, operands in
 * shared memory, FP32 accumulator in TMEM; tcgen05.cuh) in BF16 with FP32
 * accumulation: the 128 x 128 products of the two hidden layers, their input
 * gradients and their weight gradients.  The first layer (4 inputs) and
 * the output layer (1 output) are FP32 on the CUDA cores.  In the forward
 * products both the hidden activations and the weights enter as a BF16 hi +
 * lo pair (x = hi + lo, 16 significant bits), as three products
 * A_hi W_hi + A_lo W_hi + A_hi W_lo with FP32 accumulation; the weight pairs
 * are refreshed from the FP32 master copy after every Adam step, so training
 * sees the numerics of inference.  Gradients flow in single BF16.
 *
 * Loss: mean squared error of the normalised residual (mlp.cuh).
 */
#include "dcs_fp64.cuh"
#include "dcs_launch.h"
#include "mlp.cuh"
#include "tcgen05.cuh"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <initializer_list>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

using namespace noa_mlp;

namespace {

constexpr int NPARAM_PAD = (NPARAM + 3) & ~3;  // parameter-sized buffers, padded to 16 bytes
constexpr int G_THREADS = 256;
constexpr int G_TMEM_COLS = 128;  // the 128 x 128 FP32 accumulator
using noa_tc::MAT_BYTES;

enum { G_FWD = 0, G_DX = 1, G_DW = 2 };

// Dynamic shared memory of a mode: FWD stages A hi / lo and W hi / lo, the
// gradient modes one A and one B operand; 1 KB of alignment slack.
template <int MODE>
constexpr size_t gemm_smem() {
    return (MODE == G_FWD ? 4u : 2u) * MAT_BYTES + 1024u;
}

struct GemmArgs {
    const float *A;         // FWD: layer input H [M][128]; DX, DW: dZ [M][128]
    const float *B;         // DW: H_prev [M][128]
    const __nv_bfloat16 *W; // FWD, DX: weights [128 out][128 in] (hi); FWD also reads lo at W + 2*128*128
    const float *bias;      // FWD
    const float *zprev;     // DX: pre-activation of the previous layer [M][128]
    float *outZ;            // FWD: Z; DX: dZ_prev
    float *outH;            // FWD: H = silu(Z)
    float *dW;              // DW: [128 out][128 in], accumulated
    float *db;              // DW: [128], accumulated
    unsigned int *status;   // set to NOA_DCS_ERROR_TIMEOUT if an mbarrier wait expires
    int M;
};

// 8 FP32 values -> 8 BF16 (hi), and the rounding residues as 8 BF16 (lo).
__device__ __forceinline__ void split8(const float (&v)[8], uint4 &hi, uint4 &lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const __nv_bfloat162 ph = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
        const float2 back = __bfloat1622float2(ph);
        const __nv_bfloat162 pl = __floats2bfloat162_rn(v[2 * i] - back.x, v[2 * i + 1] - back.y);
        h[i] = *reinterpret_cast<const uint32_t *>(&ph);
        l[i] = *reinterpret_cast<const uint32_t *>(&pl);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// One CTA per 128-row tile, on the 5th-generation tensor cores:
//   FWD: Z = A W^T + b with A and W as BF16 hi + lo pairs (three products
//        A_hi W_hi + A_lo W_hi + A_hi W_lo), H = silu(Z)
//   DX : dZ_prev = (dZ W) * silu'(z_prev)          (B operand = W^T)
//   DW : dW += dZ^T H_prev over this tile's samples  (M = out, N = in, K = samples)
// The operands are staged as BF16 in shared memory in the canonical K-major
// layout (tcgen05.cuh): item e covers row r = e % 128 and the 8 K-consecutive
// elements k0 .. k0 + 7, k0 = 8 (e / 128), one 16-byte store per item (a warp
// stores 32 rows of one K-block: conflict-free).  Where the product needs a
// transposed operand (DX's W^T, DW's dZ^T and H_prev^T) the 8 elements come
// from 8 source rows at column r, which across a warp are coalesced reads.
// One thread issues the MMAs into a 128-column TMEM accumulator and commits
// to an mbarrier; every thread waits (bounded), then warp w reads TMEM lanes
// 32 (w % 4) .. + 31 (rows) and columns 64 (w / 4) .. + 63 for the epilogue.
template <int MODE>
__global__ void __launch_bounds__(G_THREADS, 1) mlp_gemm_kernel(const GemmArgs g) {
    using namespace noa_tc;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *sm = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
    unsigned char *sA = sm, *sB = sm + MAT_BYTES;
    unsigned char *sAl = sm + 2 * MAT_BYTES, *sBl = sm + 3 * MAT_BYTES;  // FWD only
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) unsigned long long mbar;
    const int row0 = blockIdx.x * H;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0)
        tmem_alloc(smem_u32(&tmem_slot), G_TMEM_COLS);
    if (tid == 0) {
        mbar_init(smem_u32(&mbar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }

    // stage the operands
    for (int e = tid; e < H * H / 8; e += G_THREADS) {
        const int r = e % H, k0 = (e / H) * 8;
        const uint32_t o = canon_off(r, k0);
        float v[8];
        if (MODE == G_DW) {
            // A(r = out, k = sample) = dZ[k][r]; B(r = in, k = sample) = H_prev[k][r]
            float w[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const bool in = row0 + k0 + j < g.M;
                v[j] = in ? g.A[(size_t)(row0 + k0 + j) * H + r] : 0.f;
                w[j] = in ? g.B[(size_t)(row0 + k0 + j) * H + r] : 0.f;
            }
            uint4 hi, lo;
            split8(v, hi, lo);
            *reinterpret_cast<uint4 *>(sA + o) = hi;
            split8(w, hi, lo);
            *reinterpret_cast<uint4 *>(sB + o) = hi;
        } else {
            // A(r = sample, k) = A[r][k]
            if (row0 + r < g.M) {
                const float4 *src = reinterpret_cast<const float4 *>(g.A + (size_t)(row0 + r) * H + k0);
                const float4 x = src[0], y = src[1];
                v[0] = x.x, v[1] = x.y, v[2] = x.z, v[3] = x.w, v[4] = y.x, v[5] = y.y, v[6] = y.z, v[7] = y.w;
            } else {
#pragma unroll
                for (int j = 0; j < 8; j++)
                    v[j] = 0.f;
            }
            uint4 hi, lo;
            split8(v, hi, lo);
            *reinterpret_cast<uint4 *>(sA + o) = hi;
            if (MODE == G_FWD) {
                *reinterpret_cast<uint4 *>(sAl + o) = lo;
                // B(r = out, k = in) = W[r][k], hi and lo
                *reinterpret_cast<uint4 *>(sB + o) = *reinterpret_cast<const uint4 *>(g.W + r * H + k0);
                *reinterpret_cast<uint4 *>(sBl + o) = *reinterpret_cast<const uint4 *>(g.W + 2 * H * H + r * H + k0);
            } else {
                // DX: B(r = in, k = out) = W[k][r]
                uint32_t b[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const __nv_bfloat162 t = __halves2bfloat162(g.W[(k0 + 2 * j) * H + r], g.W[(k0 + 2 * j + 1) * H + r]);
                    b[j] = *reinterpret_cast<const uint32_t *>(&t);
                }
                *reinterpret_cast<uint4 *>(sB + o) = make_uint4(b[0], b[1], b[2], b[3]);
            }
        }
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t acc = tmem_slot;
    const uint32_t mb = smem_u32(&mbar);

    if (tid == 0) {
        const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB), al0 = smem_u32(sAl), bl0 = smem_u32(sBl);
#pragma unroll
        for (int ks = 0; ks < 8; ks++) {
            const uint32_t o = ks * 256;  // 16 K-elements = two core matrices
            const uint64_t a = make_desc(a0 + o), b = make_desc(b0 + o);
            mma_ss(acc, a, b, ks > 0);
            if (MODE == G_FWD) {
                mma_ss(acc, make_desc(al0 + o), b, 1);
                mma_ss(acc, a, make_desc(bl0 + o), 1);
            }
        }
        mma_commit(mb);
    }
    const bool ok = mbar_wait(mb, 0);
    fence_after();

    if (ok) {
        const int row = (warp & 3) * 32 + lane;
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
#pragma unroll 1
        for (int half = 0; half < 2; half++) {
            const int c0 = (warp >> 2) * 64 + half * 32;
            float v[32];
            tmem_ld32(acc + lane_base + (uint32_t)c0, v);
            if (MODE == G_DW) {
                // row = out index, column = in index; 16-byte vector atomics
                // (the weight blocks of G start 16-byte aligned)
#pragma unroll
                for (int j = 0; j < 32; j += 4)
                    atomicAdd(reinterpret_cast<float4 *>(&g.dW[row * H + c0 + j]),
                              make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]));
            } else if (row0 + row < g.M) {
                const size_t o = (size_t)(row0 + row) * H + c0;
                if (MODE == G_FWD) {
#pragma unroll
                    for (int j = 0; j < 32; j += 4) {
                        float4 z, h;
                        z.x = v[j] + g.bias[c0 + j];
                        z.y = v[j + 1] + g.bias[c0 + j + 1];
                        z.z = v[j + 2] + g.bias[c0 + j + 2];
                        z.w = v[j + 3] + g.bias[c0 + j + 3];
                        h.x = silu(z.x), h.y = silu(z.y), h.z = silu(z.z), h.w = silu(z.w);
                        *reinterpret_cast<float4 *>(g.outZ + o + j) = z;
                        *reinterpret_cast<float4 *>(g.outH + o + j) = h;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 32; j += 4) {
                        const float4 zp = *reinterpret_cast<const float4 *>(g.zprev + o + j);
                        float4 d;
                        d.x = v[j] * dsilu(zp.x), d.y = v[j + 1] * dsilu(zp.y);
                        d.z = v[j + 2] * dsilu(zp.z), d.w = v[j + 3] * dsilu(zp.w);
                        *reinterpret_cast<float4 *>(g.outZ + o + j) = d;
                    }
                }
            }
        }
    } else {
        if (lane == 0)
            atomicMax(g.status, (unsigned int)NOA_DCS_ERROR_TIMEOUT);
        mbar_wait(mb, 0);  // one more bounded wait before the TMEM it writes is freed
    }
    if (MODE == G_DW && tid < H) {
        float s = 0.f;
        for (int k = 0; k < H && row0 + k < g.M; k++)
            s += g.A[(size_t)(row0 + k) * H + tid];
        atomicAdd(&g.db[tid], s);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        tmem_dealloc(acc, G_TMEM_COLS);
}

// Layer 1 (FP32): Z1 = X W1^T + b1, H1 = silu(Z1).
__global__ void mlp_fwd1_kernel(const float *__restrict__ X, const float *__restrict__ P, float *Z1, float *H1,
                                int M) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < M * H; e += gridDim.x * blockDim.x) {
        const int s = e / H, j = e % H;
        float z = P[OFF_B1 + j];
#pragma unroll
        for (int i = 0; i < IN; i++)
            z = fmaf(P[OFF_W1 + j * IN + i], X[s * IN + i], z);
        Z1[e] = z;
        H1[e] = silu(z);
    }
}

// Output layer (FP32) and the loss gradient: pred = Wo h3 + bo,
// loss = mean (pred - t)^2 over the batch of M samples (scaled by inv_batch);
// dZ3 = dpred Wo * silu'(z3); dWo, dbo accumulated per CTA.  128 samples per CTA.
__global__ void __launch_bounds__(128) mlp_out_kernel(const float *__restrict__ H3, const float *__restrict__ Z3,
                                                      const float *__restrict__ T, const float *__restrict__ P,
                                                      float *dZ3, float *G, float *loss, int M, float inv_batch,
                                                      float *pred_out) {
    __shared__ float sd[128];
    const int s = blockIdx.x * 128 + threadIdx.x;
    const int ns = min(128, M - (int)blockIdx.x * 128);  // samples of this CTA
    float dp = 0.f;
    if (s < M) {
        // four partial sums: the row's loads are independent and overlap
        float y4[4] = {P[OFF_BO], 0.f, 0.f, 0.f};
#pragma unroll 8
        for (int k = 0; k < H; k++)
            y4[k & 3] = fmaf(P[OFF_WO + k], H3[(size_t)s * H + k], y4[k & 3]);
        const float y = (y4[0] + y4[1]) + (y4[2] + y4[3]);
        if (pred_out)
            pred_out[s] = y;
        if (T) {
            const float d = y - T[s];
            dp = 2.f * d * inv_batch;
            atomicAdd(loss, d * d * inv_batch);
        }
    }
    sd[threadIdx.x] = dp;
    __syncthreads();
    if (!T)
        return;
    if (s < M) {
#pragma unroll 8
        for (int k = 0; k < H; k++)
            dZ3[(size_t)s * H + k] = dp * P[OFF_WO + k] * dsilu(Z3[(size_t)s * H + k]);
    }
    // dWo[k] = sum_s dp_s h3[s][k], thread k (coalesced across threads)
    const int k = threadIdx.x;
    float g4[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
    for (int i = 0; i < ns; i++)
        g4[i & 3] = fmaf(sd[i], H3[(size_t)(blockIdx.x * 128 + i) * H + k], g4[i & 3]);
    const float g = (g4[0] + g4[1]) + (g4[2] + g4[3]);
    atomicAdd(&G[OFF_WO + k], g);
    if (k == 0) {
        float b = 0.f;
        for (int i = 0; i < 128; i++)
            b += sd[i];
        atomicAdd(&G[OFF_BO], b);
    }
}

// Layer-1 gradients: dW1[j][i] += sum_s dZ1[s][j] X[s][i], db1 += sum dZ1.  128 samples per CTA.
__global__ void __launch_bounds__(128) mlp_bwd1_kernel(const float *__restrict__ dZ1, const float *__restrict__ X,
                                                       float *G, int M) {
    const int j = threadIdx.x;
    const int ns = min(128, M - (int)blockIdx.x * 128);  // samples of this CTA
    float gw[IN] = {0.f, 0.f, 0.f, 0.f}, gb = 0.f;
    // bounds hoisted out of the loop so that the unrolled loads overlap
#pragma unroll 8
    for (int i = 0; i < ns; i++) {
        const int s = blockIdx.x * 128 + i;
        const float d = dZ1[(size_t)s * H + j];
        const float4 x = reinterpret_cast<const float4 *>(X)[s];
        gb += d;
        gw[0] = fmaf(d, x.x, gw[0]);
        gw[1] = fmaf(d, x.y, gw[1]);
        gw[2] = fmaf(d, x.z, gw[2]);
        gw[3] = fmaf(d, x.w, gw[3]);
    }
#pragma unroll
    for (int c = 0; c < IN; c++)
        atomicAdd(&G[OFF_W1 + j * IN + c], gw[c]);
    atomicAdd(&G[OFF_B1 + j], gb);
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters; refreshes the BF16
// copies of W2, W3 used by the tensor-core products.
__global__ void mlp_adam_kernel(float *P, const float *G, float *Mm, float *V, __nv_bfloat16 *Wb, float lr,
                                float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPARAM; i += gridDim.x * blockDim.x) {
        const float g = G[i];
        const float m = b1 * Mm[i] + (1.f - b1) * g;
        const float v = b2 * V[i] + (1.f - b2) * g * g;
        Mm[i] = m;
        V[i] = v;
        const float p = P[i] - lr * (m * c1) / (sqrtf(v * c2) + eps);
        P[i] = p;
        int w = -1;
        if (i >= OFF_W2 && i < OFF_W2 + H * H)
            w = i - OFF_W2;
        else if (i >= OFF_W3 && i < OFF_W3 + H * H)
            w = H * H + i - OFF_W3;
        if (w >= 0) {
            const __nv_bfloat16 hi = __float2bfloat16_rn(p);
            Wb[w] = hi;
            Wb[2 * H * H + w] = __float2bfloat16_rn(p - __bfloat162float(hi));
        }
    }
}

// BF16 hi / lo pairs of W2, W3: Wb[0 .. 2HH) hi (W2 then W3), Wb[2HH .. 4HH) lo.
__global__ void mlp_round_weights_kernel(const float *P, __nv_bfloat16 *Wb) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * H * H; i += gridDim.x * blockDim.x) {
        const float p = i < H * H ? P[OFF_W2 + i] : P[OFF_W3 + i - H * H];
        const __nv_bfloat16 hi = __float2bfloat16_rn(p);
        Wb[i] = hi;
        Wb[2 * H * H + i] = __float2bfloat16_rn(p - __bfloat162float(hi));
    }
}

// Gathers a batch: Xb[i] = X[perm[i]], Tb[i] = T[perm[i]].
__global__ void mlp_gather_kernel(const float *X, const float *T, const int32_t *perm, float *Xb, float *Tb, int M) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        const int s = perm[i];
#pragma unroll
        for (int c = 0; c < IN; c++)
            Xb[i * IN + c] = X[(size_t)s * IN + c];
        if (T)
            Tb[i] = T[s];
    }
}

// Training data: raw features and the residual target from the FP64 plain
// kernels (dcs_fp64.cuh).  state: 1 = open pair with DCS > 0 (a training
// sample), 0 = closed by the kinematic bounds, 2 = open by the bounds but with
// DCS = 0 (every screening term clamped) or no finite baseline -- cells that
// hold such pairs must not be answered by the network.
template <int PROC>
__global__ void mlp_prepare_kernel(const double *K, const double *q, const uint8_t *elem, int64_t n,
                                   const noa_dcs_consts *consts, const float *logA, float *Xraw, float *R,
                                   uint8_t *valid) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const noa_dcs_consts &c = consts[elem[i]];
        double base;
        const bool open = baseline<PROC>(K[i], q[i], c, base);
        bool ok = open;
        double d = 0.;
        if (ok) {
            d = PROC == NOA_DCS_PAIR_PRODUCTION ? noa_dcs::pprod_fp64(K[i], q[i], c) : noa_dcs::photo_fp64(K[i], q[i], c);
            ok = d > 0. && isfinite(base);
        }
        const double nu = q[i] / (K[i] + c.mass);
        Xraw[i * IN + 0] = (float)log(K[i]);
        Xraw[i * IN + 1] = (float)log(nu);
        Xraw[i * IN + 2] = (float)c.Zd * 0.01f;
        Xraw[i * IN + 3] = logA[elem[i]];
        R[i] = ok ? (float)(log(d) - base) : 0.f;
        valid[i] = ok ? 1 : (open ? 2 : 0);
    }
}

} // namespace

struct noa_dcs_mlp {
    int process = 0;
    int batch = 0;
    float *P = nullptr, *G = nullptr, *Mm = nullptr, *V = nullptr;
    __nv_bfloat16 *Wb = nullptr;
    float *Xb = nullptr, *Tb = nullptr;
    float *Z1 = nullptr, *H1 = nullptr, *Z2 = nullptr, *H2 = nullptr, *Z3 = nullptr, *H3 = nullptr;
    float *D3 = nullptr, *D2 = nullptr, *D1 = nullptr;
    float *loss = nullptr;
    unsigned int *status = nullptr;  // device word, see take_status
    int64_t step = 0;
    float norm[2 * IN + 2] = {};
};

namespace {

thread_local char g_merr[256] = "";

int mfail(int st, const char *msg, cudaError_t e = cudaSuccess) {
    if (e != cudaSuccess)
        snprintf(g_merr, sizeof g_merr, "%s: %s", msg, cudaGetErrorString(e));
    else
        snprintf(g_merr, sizeof g_merr, "%s", msg);
    return st;
}

// Raises the three GEMM kernels' dynamic shared-memory limits once per device
// (called when a model is created).
cudaError_t set_gemm_smem() {
    static std::atomic<bool> done[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev >= 0 && dev < 64 && done[dev].load())
        return cudaSuccess;
    e = cudaFuncSetAttribute(mlp_gemm_kernel<G_FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)gemm_smem<G_FWD>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mlp_gemm_kernel<G_DX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)gemm_smem<G_DX>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mlp_gemm_kernel<G_DW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)gemm_smem<G_DW>());
    if (e == cudaSuccess && dev >= 0 && dev < 64)
        done[dev].store(true);
    return e;
}

// Status word of the tensor-core kernels: NOA_DCS_ERROR_TIMEOUT after an
// expired mbarrier wait.  Read (and cleared) after the work of a call;
// synchronises the stream.
int take_status(noa_dcs_mlp *m, cudaStream_t s);

// Forward over M <= batch rows already in m->Xb; prediction to pred if given.
cudaError_t forward(noa_dcs_mlp *m, int M, float *pred, cudaStream_t s) {
    const int tiles = (M + H - 1) / H;
    mlp_fwd1_kernel<<<(M * H + 255) / 256, 256, 0, s>>>(m->Xb, m->P, m->Z1, m->H1, M);
    GemmArgs g{};
    g.M = M;
    g.status = m->status;
    g.A = m->H1;
    g.W = m->Wb;
    g.bias = m->P + OFF_B2;
    g.outZ = m->Z2;
    g.outH = m->H2;
    mlp_gemm_kernel<G_FWD><<<tiles, G_THREADS, gemm_smem<G_FWD>(), s>>>(g);
    g.A = m->H2;
    g.W = m->Wb + H * H;
    g.bias = m->P + OFF_B3;
    g.outZ = m->Z3;
    g.outH = m->H3;
    mlp_gemm_kernel<G_FWD><<<tiles, G_THREADS, gemm_smem<G_FWD>(), s>>>(g);
    if (pred)
        mlp_out_kernel<<<tiles, 128, 0, s>>>(m->H3, m->Z3, nullptr, m->P, nullptr, nullptr, nullptr, M, 0.f, pred);
    return cudaGetLastError();
}

// Loss and gradient of one batch of M rows in Xb / Tb into m->G (zeroed first).
cudaError_t backward(noa_dcs_mlp *m, int M, cudaStream_t s) {
    const int tiles = (M + H - 1) / H;
    cudaError_t e = cudaMemsetAsync(m->G, 0, sizeof(float) * NPARAM, s);
    if (e != cudaSuccess)
        return e;
    if ((e = forward(m, M, nullptr, s)) != cudaSuccess)
        return e;
    mlp_out_kernel<<<tiles, 128, 0, s>>>(m->H3, m->Z3, m->Tb, m->P, m->D3, m->G, m->loss, M, 1.f / (float)M,
                                         nullptr);
    GemmArgs g{};
    g.M = M;
    g.status = m->status;
    // layer 3: dW3 = dZ3^T H2, dZ2 = (dZ3 W3) silu'(Z2)
    g.A = m->D3;
    g.B = m->H2;
    g.dW = m->G + OFF_W3;
    g.db = m->G + OFF_B3;
    mlp_gemm_kernel<G_DW><<<tiles, G_THREADS, gemm_smem<G_DW>(), s>>>(g);
    g.W = m->Wb + H * H;
    g.zprev = m->Z2;
    g.outZ = m->D2;
    mlp_gemm_kernel<G_DX><<<tiles, G_THREADS, gemm_smem<G_DX>(), s>>>(g);
    // layer 2: dW2 = dZ2^T H1, dZ1 = (dZ2 W2) silu'(Z1)
    g.A = m->D2;
    g.B = m->H1;
    g.dW = m->G + OFF_W2;
    g.db = m->G + OFF_B2;
    mlp_gemm_kernel<G_DW><<<tiles, G_THREADS, gemm_smem<G_DW>(), s>>>(g);
    g.W = m->Wb;
    g.zprev = m->Z1;
    g.outZ = m->D1;
    mlp_gemm_kernel<G_DX><<<tiles, G_THREADS, gemm_smem<G_DX>(), s>>>(g);
    mlp_bwd1_kernel<<<tiles, 128, 0, s>>>(m->D1, m->Xb, m->G, M);
    return cudaGetLastError();
}

// Every buffer must be device (or managed) memory of the current device before
// it reaches a kernel; nullptr passes (optional arguments are checked by the
// callers).
bool device_ok(std::initializer_list<const void *> ptrs) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return false;
    for (const void *p : ptrs) {
        if (!p)
            continue;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (!(a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev)))
            return false;
    }
    return true;
}

int take_status(noa_dcs_mlp *m, cudaStream_t s) {
    unsigned int st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, m->status, sizeof st, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return mfail(NOA_DCS_ERROR_CUDA, "status read", e);
    if (st) {
        cudaMemsetAsync(m->status, 0, sizeof st, s);
        return mfail((int)st, "a tensor-core wait expired (mbarrier); the results of this call are invalid");
    }
    return NOA_DCS_SUCCESS;
}

} // namespace

extern "C" {

int noa_dcs_mlp_create(noa_dcs_mlp **out, int process, int batch) {
    g_merr[0] = '\0';
    if (!out)
        return mfail(NOA_DCS_ERROR_INVALID_VALUE, "NULL model pointer");
    *out = nullptr;
    if (process != NOA_DCS_PAIR_PRODUCTION && process != NOA_DCS_PHOTONUCLEAR)
        return mfail(NOA_DCS_ERROR_NOT_SUPPORTED, "the surrogate covers pair production and photonuclear");
    if (batch < 128 || batch > (1 << 20) || batch % 128)
        return mfail(NOA_DCS_ERROR_INVALID_VALUE, "batch must be a multiple of 128 in [128, 2^20]");
    cudaError_t e = set_gemm_smem();
    if (e != cudaSuccess)
        return mfail(NOA_DCS_ERROR_CUDA, "cudaFuncSetAttribute", e);
    noa_dcs_mlp *m = new (std::nothrow) noa_dcs_mlp();
    if (!m)
        return mfail(NOA_DCS_ERROR_INVALID_VALUE, "out of host memory");
    m->process = process;
    m->batch = batch;
    const size_t act = sizeof(float) * (size_t)batch * H;
    float **acts[] = {&m->Z1, &m->H1, &m->Z2, &m->H2, &m->Z3, &m->H3, &m->D3, &m->D2, &m->D1};
    e = cudaSuccess;
    for (float **a : acts)
        if (e == cudaSuccess)
            e = cudaMalloc((void **)a, act);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&m->P, sizeof(float) * NPARAM_PAD * 4);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&m->Wb, sizeof(__nv_bfloat16) * 4 * H * H);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&m->Xb, sizeof(float) * (size_t)batch * (IN + 1) + 2 * sizeof(float));
    if (e != cudaSuccess) {
        for (float **a : acts)
            cudaFree(*a);
        cudaFree(m->P);
        cudaFree(m->Wb);
        cudaFree(m->Xb);
        delete m;
        return mfail(NOA_DCS_ERROR_CUDA, "model allocation", e);
    }
    m->G = m->P + NPARAM_PAD;  // each block 16-byte aligned (vector atomics on G)
    m->Mm = m->G + NPARAM_PAD;
    m->V = m->Mm + NPARAM_PAD;
    m->Tb = m->Xb + (size_t)batch * IN;
    m->loss = m->Tb + batch;
    m->status = reinterpret_cast<unsigned int *>(m->loss + 1);
    cudaMemset(m->P, 0, sizeof(float) * NPARAM_PAD * 4);
    cudaMemset(m->status, 0, sizeof(unsigned int));
    cudaMemset(m->Wb, 0, sizeof(__nv_bfloat16) * 4 * H * H);
    *out = m;
    return NOA_DCS_SUCCESS;
}

int noa_dcs_mlp_set_params(noa_dcs_mlp *m, const float *params, const float *adam_m, const float *adam_v,
                           int64_t step, const float *norm) {
    if (!m || !params || !norm)
        return mfail(NOA_DCS_ERROR_INVALID_VALUE, "NULL argument");
    cudaError_t e = cudaMemcpy(m->P, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = adam_m ? cudaMemcpy(m->Mm, adam_m, sizeof(float) * NPARAM, cudaMemcpyHostToDevice)
                   : cudaMemset(m->Mm, 0, sizeof(float) * NPARAM);
    if (e == cudaSuccess)
        e = adam_v ? cudaMemcpy(m->V, adam_v, sizeof(float) * NPARAM, cudaMemcpyHostToDevice)
                   : cudaMemset(m->V, 0, sizeof(float) * NPARAM);
    if (e != cudaSuccess)
        return mfail(NOA_DCS_ERROR_CUDA, "cudaMemcpy(params)", e);
    mlp_round_weights_kernel<<<64, 256>>>(m->P, m->Wb);
    if ((e = cudaDeviceSynchronize()) != cudaSuccess)
        return mfail(NOA_DCS_ERROR_CUDA, "round weights", e);
    m->step = step;
    std::memcpy(m->norm, norm, sizeof m->norm);
    return NOA_DCS_SUCCESS;
}

int noa_dcs_mlp_get_params(noa_dcs_mlp *m, float *params, float *adam_m, float *adam_v, int64_t *step) {
    if (!m || !params)
        return mfail(NOA_DCS_ERROR_INVALID_VALUE, "NULL argument");
    cudaError_t e = cudaMemcpy(params, m->P, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && adam_m)
        e = cudaMemcpy(adam_m, m->Mm, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && adam_v)
        e = cudaMemcpy(adam_v, m->V, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return mfail(NOA_DCS_ERROR_CUDA, "cudaMemcpy(params)", e);
    if (step)
        *step = m->step;
    return NOA_DCS_SUCCESS;
}

int noa_dcs_mlp_prepare(int process, const double *K, const double *q, const uint8_t *elem, int64_t n,
                        const noa_dcs_element *elements, int n_elements, double mass, float *Xraw, float *R,
                        uint8_t *valid, void *stream) {
    g_merr[0] = '\0';
    if (process != NOA_DCS_PAIR_PRODUCTION && process != NOA_DCS_PHOTONUCLEAR)
        return mfail(NOA_DCS_ERROR_NOT_SUPPORTED, "the surrogate covers pair production and photonuclear");
    if (n < 0 || n_elements < 1 || n_elements > 16 || !elements)
        return mfail(NOA_DCS_ERROR_INVALID_VALUE, "bad sizes");
    if (n == 0)
        return NOA_DCS_SUCCESS;
    if (!K || !q || !elem || !Xraw || !R || !valid || !device_ok({K, q, elem, Xraw, R, valid}))
        return mfail(NOA_DCS_ERROR_NOT_DEVICE_MEMORY, "K, q, elem, Xraw, R and valid must be device memory");
    noa_dcs_consts hc[16];
    float hlogA[16];
    for (int i = 0; i < n_elements; i++) {
        noa_dcs_fill_consts(&hc[i], elements[i].A, elements[i].I, elements[i].Z, mass);
        hlogA[i] = (float)std::log(elements[i].A);
    }
    // The element table (up to 16 constant sets) is staged through a small
    // device buffer that lives until this call's work is done (synchronised
    // below); data preparation is off the evaluation path.
    noa_dcs_consts *dc = nullptr;
    float *dl = nullptr;
    cudaError_t e = cudaMalloc((void **)&dc, sizeof hc + sizeof hlogA);
    if (e != cudaSuccess)
        return mfail(NOA_DCS_ERROR_CUDA, "cudaMalloc(element table)", e);
    dl = reinterpret_cast<float *>(dc + 16);
    cudaStream_t s = (cudaStream_t)stream;
    e = cudaMemcpyAsync(dc, hc, sizeof hc, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dl, hlogA, sizeof hlogA, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        const int64_t blocks = (n + 255) / 256;
        const int grid = (int)(blocks < 152 * 16 ? blocks : 152 * 16);
        if (process == NOA_DCS_PAIR_PRODUCTION)
            mlp_prepare_kernel<NOA_DCS_PAIR_PRODUCTION><<<grid, 256, 0, s>>>(K, q, elem, n, dc, dl, Xraw, R, valid);
        else
            mlp_prepare_kernel<NOA_DCS_PHOTONUCLEAR><<<grid, 256, 0, s>>>(K, q, elem, n, dc, dl, Xraw, R, valid);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    cudaFree(dc);
    if (e != cudaSuccess)
        return mfail(NOA_DCS_ERROR_CUDA, "prepare", e);
    return NOA_DCS_SUCCESS;
}

int noa_dcs_mlp_train(noa_dcs_mlp *m, const float *X, const float *T, int64_t n, const int32_t *perm,
                      int64_t n_steps, float lr, float lr_final, float *losses, void *stream) {
    g_merr[0] = '\0';
    if (!m || !X || !T || !perm || n < m->batch || n_steps < 0)
        return mfail(NOA_DCS_ERROR_INVALID_VALUE, "bad training arguments (n must be at least one batch)");
    if (!device_ok({X, T, perm, losses}))
        return mfail(NOA_DCS_ERROR_NOT_DEVICE_MEMORY, "X, T, perm and losses must be device memory");
    cudaStream_t s = (cudaStream_t)stream;
    const int B = m->batch;
    const int64_t batches = n / B;
    cudaError_t e = cudaSuccess;
    for (int64_t i = 0; i < n_steps && e == cudaSuccess; i++) {
        const int64_t b = (m->step) % batches;
        mlp_gather_kernel<<<(B + 255) / 256, 256, 0, s>>>(X, T, perm + b * B, m->Xb, m->Tb, B);
        cudaMemsetAsync(m->loss, 0, sizeof(float), s);
        if ((e = backward(m, B, s)) != cudaSuccess)
            break;
        // cosine decay from lr to lr_final over the n_steps of this call
        const double frac = n_steps > 1 ? (double)i / (double)(n_steps - 1) : 0.;
        const float lr_i = (float)(lr_final + 0.5 * (lr - lr_final) * (1. + std::cos(M_PI * frac)));
        m->step++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f / (1.f - std::pow(b1, (float)m->step));
        const float c2 = 1.f / (1.f - std::pow(b2, (float)m->step));
        mlp_adam_kernel<<<(NPARAM + 255) / 256, 256, 0, s>>>(m->P, m->G, m->Mm, m->V, m->Wb, lr_i, b1, b2, 1e-8f,
                                                             c1, c2);
        if (losses)
            cudaMemcpyAsync(losses + i, m->loss, sizeof(float), cudaMemcpyDeviceToDevice, s);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess)
        return mfail(NOA_DCS_ERROR_CUDA, "training step", e);
    return take_status(m, s);
}

int noa_dcs_mlp_predict(noa_dcs_mlp *m, const float *X, float *out, int64_t n, void *stream) {
    g_merr[0] = '\0';
    if (!m || (n > 0 && (!X || !out)) || n < 0)
        return mfail(NOA_DCS_ERROR_INVALID_VALUE, "bad arguments");
    if (n > 0 && !device_ok({X, out}))
        return mfail(NOA_DCS_ERROR_NOT_DEVICE_MEMORY, "X and out must be device memory");
    cudaStream_t s = (cudaStream_t)stream;
    for (int64_t off = 0; off < n; off += m->batch) {
        const int M = (int)((n - off) < m->batch ? (n - off) : m->batch);
        cudaMemcpyAsync(m->Xb, X + off * IN, sizeof(float) * IN * M, cudaMemcpyDeviceToDevice, s);
        const cudaError_t e = forward(m, M, out + off, s);
        if (e != cudaSuccess)
            return mfail(NOA_DCS_ERROR_CUDA, "forward", e);
    }
    return n > 0 ? take_status(m, s) : NOA_DCS_SUCCESS;
}

int noa_dcs_mlp_gradient(noa_dcs_mlp *m, const float *X, const float *T, int n, float *grad, float *loss,
                         void *stream) {
    g_merr[0] = '\0';
    if (!m || !X || !T || !grad || n < 1 || n > m->batch)
        return mfail(NOA_DCS_ERROR_INVALID_VALUE, "bad arguments (1 <= n <= batch)");
    if (!device_ok({X, T, grad, loss}))
        return mfail(NOA_DCS_ERROR_NOT_DEVICE_MEMORY, "X, T, grad and loss must be device memory");
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemcpyAsync(m->Xb, X, sizeof(float) * IN * n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(m->Tb, T, sizeof(float) * n, cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(m->loss, 0, sizeof(float), s);
    cudaError_t e = backward(m, n, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(grad, m->G, sizeof(float) * NPARAM, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && loss)
        e = cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess)
        return mfail(NOA_DCS_ERROR_CUDA, "gradient", e);
    return take_status(m, s);
}

int noa_dcs_mlp_destroy(noa_dcs_mlp *m) {
    if (!m)
        return NOA_DCS_SUCCESS;
    float *acts[] = {m->Z1, m->H1, m->Z2, m->H2, m->Z3, m->H3, m->D3, m->D2, m->D1};
    for (float *a : acts)
        cudaFree(a);
    cudaFree(m->P);
    cudaFree(m->Wb);
    cudaFree(m->Xb);
    delete m;
    return NOA_DCS_SUCCESS;
}

const char *noa_dcs_mlp_last_error(void) { return g_merr; }

// Internal accessor for the inference translation unit (mlp_infer.cu).
int noa_dcs_mlp_handles(noa_dcs_mlp *m, int *process, const float **P, const void **Wb, const float **norm) {
    if (!m)
        return 1;
    *process = m->process;
    *P = m->P;
    *Wb = m->Wb;
    *norm = m->norm;
    return 0;
}

} // extern "C"
