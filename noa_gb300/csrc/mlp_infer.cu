/*
 * Learned DCS surrogate, inference (noa_dcs_mlp_infer): four kernels on the
 * caller's stream.
 *
 *  1. classify: per pair, the kinematic bounds decided as the FP64 kernels
 *     decide them (closed -> 0); for the open pairs, compacted in shared
 *     memory, the normalised features and the trust-grid cell.  Pairs inside
 *     the trained domain whose cell passed the held-out error check go to the
 *     network list; the others to the fallback list (both in the model's
 *     scratch, positions from block-wide scans).
 *     Then netprep: the float baseline of mlp.cuh for each listed pair,
 *     densely over the list.
 *  2. network (tcgen05): a persistent CTA of four warpgroups keeps two tiles
 *     of 128 listed pairs in flight, two warpgroups each, so that the tensor
 *     core works on one tile while the CUDA cores run the other's SiLU
 *     epilogue.  Row r of a tile is TMEM lane r; a thread owns one row and 64
 *     of its 128 hidden units.  Layer 1 (4 -> 128) and the output layer run in
 *     FP32 on the CUDA cores; the two 128 x 128 layers run on the
 *     5th-generation tensor cores.  The activations are written to TMEM
 *     (tcgen05.st) as BF16 hi / lo, two per 32-bit column, and are the A
 *     operand of tcgen05.mma.cta_group::1.kind::f16 (M = N = 128, K = 16);
 *     W2 and W3 (hi / lo, resident in shared memory in the canonical
 *     no-swizzle K-major layout for the whole launch) are the B operands.
 *     One thread per tile issues the three products A_hi W_hi + A_lo W_hi +
 *     A_hi W_lo, accumulating in FP32 in TMEM, and commits to the tile's
 *     mbarrier; the epilogue reads the accumulator with tcgen05.ld, adds the
 *     bias and applies SiLU.  TMEM per tile: accumulator 128 columns, A hi 64,
 *     A lo 64 (512 for the two).
 *     DCS = exp(baseline + residual), in float (1e-6 relative).
 *  3. fallback: the FP32C evaluation (dcs_fp32c.cuh) of the fallback list,
 *     with FP64 (dcs_fp64.cuh) for pairs above its tolerance (pair
 *     production: after a second FP32 pass with the float-float screening
 *     log).
 *
 * Every mbarrier wait is bounded; on expiry the kernel records
 * NOA_DCS_ERROR_TIMEOUT in the model's status word, gives the MMAs still in
 * flight one more bounded wait, frees its TMEM and returns.
 */
#include "dcs_fp32c.cuh"
#include "dcs_fp64.cuh"
#include "dcs_launch.h"
#include "mlp.cuh"
#include "tcgen05.cuh"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

using namespace noa_mlp;

namespace {

constexpr int NT = 512;                   // threads of the network kernel: 4 warpgroups
constexpr int SLOTS = 2;                  // tiles in flight per CTA, two warpgroups each
constexpr int TILE = 128;                 // rows (pairs) per tile = TMEM lanes
constexpr int TMEM_COLS = 512;            // per slot: accumulator 128 + A hi 64 + A lo 64 columns
constexpr int MAT = H * H * 2;            // bytes of one 128 x 128 BF16 operand
constexpr int SMEM_NET = 4 * MAT + 1024;  // W2 hi/lo, W3 hi/lo, alignment slack
constexpr int MAX_EL = 16;

struct InferParams {
    const double *K;
    const double *q;
    double *out;
    int n_seg;
    int pad_;
    int64_t seg_begin[MAX_EL + 1];
    noa_dcs_consts consts[MAX_EL];
    float logA[MAX_EL];
    float Zf[MAX_EL];
    Norm norm;
    const uint8_t *trust;  // [n_seg][64][64]
    float logk_lo, logk_scale, lognu_lo, lognu_scale;  // cell = floor((log - lo) * scale)
    // lists
    int32_t *net_idx;
    float *net_base;
    float4 *net_feat;
    int32_t *fb_idx;
    uint8_t *fb_seg;
    uint8_t *net_seg;
    unsigned long long *counters;  // [0] network, [1] fallback, [2] status
    float tol;
};

__device__ __forceinline__ void append(unsigned long long *counter, bool flag, int &slot) {
    const unsigned m = __ballot_sync(0xffffffffu, flag);
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (m && lane == __ffs(m) - 1)
        base = atomicAdd(counter, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, __ffs(m ? m : 1u) - 1);
    slot = flag ? (int)(base + __popc(m & ((1u << lane) - 1u))) : -1;
}

// Classify, in tiles of CL_TILE pairs, in two phases.
//  1. Bounds: each thread decides the kinematic bounds of CL_ITEMS pairs as
//     the FP64 kernels decide them (open_fast), writes 0 for a closed pair,
//     and each warp compacts its open pairs (index, segment, K, q) into its
//     own shared-memory queue (warp ballots: no block-wide barrier).
//  2. Features, densely over each warp's queue: log K, log(q / (K + m)) (fast float
//     logs; the network's inputs need ~1e-6), the trust-grid cell (by
//     multiplication with the grid scale, as the host's cell assignment) and
//     its trust bit; trusted pairs go to the network list, the others to the
//     fallback list, with list positions from a block-wide scan and one
//     atomicAdd per list per tile.
// Only open pairs (20% for photonuclear, 54% for pair production on the
// benchmark law) pay for features.
constexpr int CL_THREADS = 256, CL_ITEMS = 4, CL_TILE = CL_THREADS * CL_ITEMS;

// Exclusive block-wide scan of two counts (256 threads); returns this
// thread's offsets and writes the totals to *tot_a, *tot_b (shared).
__device__ __forceinline__ void block_scan2(int ca, int cb, int &oa, int &ob, int *wa, int *wb, int *tot_a,
                                            int *tot_b) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int sa = ca, sb = cb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int ya = __shfl_up_sync(0xffffffffu, sa, o), yb = __shfl_up_sync(0xffffffffu, sb, o);
        if (lane >= o) {
            sa += ya;
            sb += yb;
        }
    }
    if (lane == 31) {
        wa[warp] = sa;
        wb[warp] = sb;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int ta = 0, tb = 0;
        for (int w = 0; w < CL_THREADS / 32; w++) {
            const int x = wa[w], y = wb[w];
            wa[w] = ta;
            wb[w] = tb;
            ta += x;
            tb += y;
        }
        *tot_a = ta;
        *tot_b = tb;
    }
    __syncthreads();
    oa = wa[warp] + sa - ca;
    ob = wb[warp] + sb - cb;
}

template <int PROC>
__global__ void __launch_bounds__(CL_THREADS) classify_kernel(const __grid_constant__ InferParams p) {
    __shared__ int warp_a[CL_THREADS / 32], warp_b[CL_THREADS / 32];
    __shared__ int tot_a, tot_b;
    __shared__ unsigned long long base_n, base_f;
    // per-warp queues of the open pairs: warp w owns entries [128 w, 128 w + 128)
    __shared__ double qK[CL_TILE], qq[CL_TILE];
    __shared__ int32_t qi[CL_TILE];
    __shared__ uint8_t qs[CL_TILE];
    __shared__ float4 s_feat[CL_TILE];
    const int64_t n = p.seg_begin[p.n_seg];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int qbase = warp * 32 * CL_ITEMS;
    const unsigned lt = (1u << lane) - 1u;
    int seg_at = 0;  // segment of this thread's last pair
    for (int64_t tile = (int64_t)blockIdx.x * CL_TILE; tile < n; tile += (int64_t)gridDim.x * CL_TILE) {
        // phase 1: bounds; closed pairs get 0, open pairs join the warp's queue.
        // The tile's K and q are all requested before the first decision
        // (memory latency, not arithmetic, bounds this phase).
        double Kv[CL_ITEMS], qv[CL_ITEMS];
#pragma unroll
        for (int j = 0; j < CL_ITEMS; j++) {
            const int64_t i = tile + j * CL_THREADS + threadIdx.x;
            Kv[j] = i < n ? p.K[i] : 0.;
            qv[j] = i < n ? p.q[i] : 0.;
        }
        int n_open = 0;  // warp-uniform
#pragma unroll
        for (int j = 0; j < CL_ITEMS; j++) {
            const int64_t i = tile + j * CL_THREADS + threadIdx.x;
            bool open = false;
            int seg = seg_at;
            if (i < n) {
                while (seg + 1 < p.n_seg && i >= p.seg_begin[seg + 1])  // a thread's pairs come in order
                    seg++;
                seg_at = seg;
                open = open_fast<PROC>(Kv[j], qv[j], p.consts[seg]);
                if (!open)
                    p.out[i] = 0.;
            }
            const unsigned m = __ballot_sync(0xffffffffu, open);
            if (open) {
                const int at = qbase + n_open + __popc(m & lt);
                qi[at] = (int32_t)i;
                qs[at] = (uint8_t)seg;
                qK[at] = Kv[j];
                qq[at] = qv[j];
            }
            n_open += __popc(m);
        }
        __syncwarp();
        // phase 2: features, cell and trust of the warp's queued pairs
        unsigned net_mask = 0, fb_mask = 0;
#pragma unroll
        for (int j = 0; j < CL_ITEMS; j++) {
            const int e = j * 32 + lane;
            if (e < n_open) {
                const int at = qbase + e;
                const int seg = qs[at];
                const float Kf = fpconv::f32_normal(qK[at]), qf = fpconv::f32_normal(qq[at]);  // NaN: no cell
                const float lk = __logf(Kf), ln = __logf(__fdividef(qf, Kf + p.consts[seg].mass_h));
                const float fk = floorf((lk - p.logk_lo) * p.logk_scale);
                const float fn = floorf((ln - p.lognu_lo) * p.lognu_scale);
                const bool in_grid = fk >= 0.f && fk < 64.f && fn >= 0.f && fn < 64.f;
                const bool trusted = in_grid && p.trust[(seg * 64 + (int)fk) * 64 + (int)fn] != 0;
                float4 f;
                f.x = (lk - p.norm.in_shift[0]) * p.norm.in_scale[0];
                f.y = (ln - p.norm.in_shift[1]) * p.norm.in_scale[1];
                f.z = (p.Zf[seg] * 0.01f - p.norm.in_shift[2]) * p.norm.in_scale[2];
                f.w = (p.logA[seg] - p.norm.in_shift[3]) * p.norm.in_scale[3];
                s_feat[at] = f;
                net_mask |= (unsigned)trusted << j;
                fb_mask |= (unsigned)!trusted << j;
            }
        }
        // list positions: one block-wide scan and one atomicAdd per list per tile
        int pn, pf;
        block_scan2(__popc(net_mask), __popc(fb_mask), pn, pf, warp_a, warp_b, &tot_a, &tot_b);
        if (threadIdx.x == 0) {
            base_n = tot_a ? atomicAdd(&p.counters[0], (unsigned long long)tot_a) : 0ull;
            base_f = tot_b ? atomicAdd(&p.counters[1], (unsigned long long)tot_b) : 0ull;
        }
        __syncthreads();
        unsigned long long wn = base_n + (unsigned long long)pn, wf = base_f + (unsigned long long)pf;
#pragma unroll
        for (int j = 0; j < CL_ITEMS; j++) {
            const int at = qbase + j * 32 + lane;
            if (net_mask & (1u << j)) {
                p.net_idx[wn] = qi[at];
                p.net_feat[wn] = s_feat[at];
                p.net_seg[wn] = qs[at];
                wn++;
            }
            if (fb_mask & (1u << j)) {
                p.fb_idx[wf] = qi[at];
                p.fb_seg[wf] = qs[at];
                wf++;
            }
        }
        // The next tile rewrites this warp's queue; its scan's first barrier
        // comes after every thread has used this tile's bases.
        __syncwarp();
    }
}

// Baselines of the network list, computed densely over the list (in the
// classify kernel only the trusted lanes would need them, and the others
// would wait).  A pair whose baseline float cannot form moves to the
// fallback list; its network row is computed but not written (index -1).
template <int PROC>
__global__ void __launch_bounds__(256) netprep_kernel(const __grid_constant__ InferParams p) {
    const unsigned long long cnt = p.counters[0];
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < cnt;
         base += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long e = base + threadIdx.x;
        bool to_fb = false;
        int32_t i = 0;
        uint8_t sg = 0;
        if (e < cnt) {
            i = p.net_idx[e];
            sg = p.net_seg[e];
            float bf;
            if (baseline_value<PROC>(p.K[i], p.q[i], p.consts[sg], bf) && isfinite(bf)) {
                p.net_base[e] = bf;
            } else {
                p.net_idx[e] = -1;
                to_fb = true;
            }
        }
        int s_fb;
        append(&p.counters[1], to_fb, s_fb);
        if (to_fb) {
            p.fb_idx[s_fb] = i;
            p.fb_seg[s_fb] = sg;
        }
    }
}

// Appends (index, segment) of the lanes with `push` to a shared-memory queue
// (warp-aggregated).
__device__ __forceinline__ void push_index(bool push, int32_t i, uint8_t sg, int32_t *q, uint8_t *qs, int *qn) {
    const unsigned m = __ballot_sync(0xffffffffu, push);
    if (m) {
        const int lane = threadIdx.x & 31;
        int at = 0;
        if (lane == 0)
            at = atomicAdd(qn, __popc(m));
        at = __shfl_sync(0xffffffffu, at, 0);
        if (push) {
            const int pos = at + __popc(m & ((1u << lane) - 1u));
            q[pos] = i;
            qs[pos] = sg;
        }
    }
}

// FP32C evaluation of the fallback list; pairs above the tolerance go to a
// shared-memory redo queue that full warps drain in FP64, so the FP64 work is
// proportional to the redo fraction (as in dcs_fp32c.cu).
// Four CTAs per SM (at most 64 registers; pair production spills 24 bytes
// and runs 2.7% faster than at three CTAs).
template <int PROC>
__global__ void __launch_bounds__(256, 4) fallback_kernel(const __grid_constant__ InferParams p) {
    // pair production: redo pairs are evaluated again with the float-float
    // screening log, and the few it still rejects go to a third queue (FP64)
    constexpr bool fine = PROC == NOA_DCS_PAIR_PRODUCTION;
    __shared__ int32_t rq[512], xq[fine ? 512 : 1];
    __shared__ uint8_t rs[512], xs[fine ? 512 : 1];
    __shared__ int rn, xn;
    if (threadIdx.x == 0) {
        rn = 0;
        xn = 0;
    }
    __syncthreads();
    const unsigned long long cnt = p.counters[1];
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < cnt;
         base += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long e = base + threadIdx.x;
        bool redo = false;
        int32_t i = 0;
        uint8_t sg = 0;
        if (e < cnt) {
            i = p.fb_idx[e];
            sg = p.fb_seg[e];
            const noa_dcs_consts &c = p.consts[sg];
            float est;
            // classify_kernel listed only pairs that the exact bounds leave open
            const double v = PROC == NOA_DCS_PAIR_PRODUCTION ? noa_dcs::pprod_fp32c<false>(p.K[i], p.q[i], c, est)
                                                             : noa_dcs::photo_fp32c<false>(p.K[i], p.q[i], c, est);
            redo = !(est <= p.tol);
            if (!redo)
                p.out[i] = v;
        }
        push_index(redo, i, sg, rq, rs, &rn);
        __syncthreads();
        const bool last = base + (unsigned long long)gridDim.x * blockDim.x >= cnt;
        // one call site each for the redo evaluation and the FP64 one
        for (;;) {
            bool did = false;
            const int n = rn;
            if (n >= (last ? 1 : 256)) {
                const int take = n < 256 ? n : 256;
                bool again = false;
                int32_t j = 0;
                uint8_t sj = 0;
                if ((int)threadIdx.x < take) {
                    const int k = n - take + threadIdx.x;
                    j = rq[k];
                    sj = rs[k];
                    const noa_dcs_consts &c = p.consts[sj];
                    if (fine) {
                        float est;
                        const double v = noa_dcs::pprod_fp32c<false, true>(p.K[j], p.q[j], c, est);
                        again = !(est <= p.tol);
                        if (!again)
                            p.out[j] = v;
                    } else {
                        p.out[j] = noa_dcs::photo_fp64_ol(p.K[j], p.q[j], c);
                    }
                }
                if (fine)
                    push_index(again, j, sj, xq, xs, &xn);
                __syncthreads();
                if (threadIdx.x == 0)
                    rn = n - take;
                __syncthreads();
                did = true;
            }
            if (fine) {
                const int nx = xn;
                if (nx >= 256 || (last && rn == 0 && nx > 0)) {
                    const int take = nx < 256 ? nx : 256;
                    if ((int)threadIdx.x < take) {
                        const int k = nx - take + threadIdx.x;
                        const int32_t j = xq[k];
                        p.out[j] = noa_dcs::pprod_fp64_ol(p.K[j], p.q[j], p.consts[xs[k]]);
                    }
                    __syncthreads();
                    if (threadIdx.x == 0)
                        xn = nx - take;
                    __syncthreads();
                    did = true;
                }
            }
            if (!did)
                break;
        }
    }
}

// ---------------------------------------------------------------- tcgen05 helpers (tcgen05.cuh)
using noa_tc::canon_off;
using noa_tc::fence_after;
using noa_tc::fence_async_smem;
using noa_tc::fence_before;
using noa_tc::make_desc;
using noa_tc::mbar_wait;
using noa_tc::mma_commit;
using noa_tc::smem_u32;
using noa_tc::tmem_ld32;
using noa_tc::tmem_st16;

// Packs 32 activations (consecutive hidden units, even unit in the low half)
// as BF16 hi / lo pairs: 16 + 16 32-bit TMEM columns.
__device__ __forceinline__ void pack32(const float (&h)[32], uint32_t (&hi)[16], uint32_t (&lo)[16]) {
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const __nv_bfloat16 a = __float2bfloat16_rn(h[2 * i]), b = __float2bfloat16_rn(h[2 * i + 1]);
        const __nv_bfloat162 ph = __halves2bfloat162(a, b);
        const __nv_bfloat162 pl = __halves2bfloat162(__float2bfloat16_rn(h[2 * i] - __bfloat162float(a)),
                                                     __float2bfloat16_rn(h[2 * i + 1] - __bfloat162float(b)));
        hi[i] = *reinterpret_cast<const uint32_t *>(&ph);
        lo[i] = *reinterpret_cast<const uint32_t *>(&pl);
    }
}

// Issues the 8 K-steps x 3 products of one 128 x 128 layer, A (hi / lo) from
// TMEM, and commits to the mbarrier.  One thread.
__device__ __forceinline__ void issue_layer_ts(uint32_t acc, uint32_t a_hi, uint32_t a_lo, uint32_t w_hi,
                                               uint32_t w_lo, uint32_t mbar) {
    fence_after();
#pragma unroll
    for (int ks = 0; ks < 8; ks++) {
        const uint32_t o = ks * 256;  // B: two core matrices along K per step
        const uint32_t c = ks * 8;    // A: 16 BF16 = 8 TMEM columns per step
        noa_tc::mma_ts(acc, a_hi + c, make_desc(w_hi + o), ks > 0);
        noa_tc::mma_ts(acc, a_lo + c, make_desc(w_hi + o), 1);
        noa_tc::mma_ts(acc, a_hi + c, make_desc(w_lo + o), 1);
    }
    mma_commit(mbar);
}

__device__ __forceinline__ void slot_sync(int slot) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + slot), "r"(NT / SLOTS) : "memory");
}

template <int PROC>
__global__ void __launch_bounds__(NT, 1) network_kernel(const __grid_constant__ InferParams p, const float *P,
                                                        const __nv_bfloat16 *Wb) {
    extern __shared__ unsigned char smem_raw[];
    // 1024-byte aligned operand area
    unsigned char *sm = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
    unsigned char *W2h = sm, *W2l = sm + MAT, *W3h = sm + 2 * MAT, *W3l = sm + 3 * MAT;
    __shared__ __align__(16) float sW1[H * IN];
    __shared__ float sb1[H], sb2[H], sb3[H], sWo[H];
    __shared__ float spart[SLOTS][TILE];
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) unsigned long long mbar[SLOTS];
    __shared__ int s_abort[SLOTS];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // two tiles in flight: slot s = warpgroups 2s, 2s+1; a thread owns row
    // `row` (its TMEM lane) and the 64 hidden units [64 half, 64 half + 64)
    const int slot = warp / 8, wis = warp % 8, half = wis / 4;
    const int row = (warp % 4) * 32 + lane;
    const unsigned long long cnt = p.counters[0];

    // weights to shared memory (canonical layout): 8 consecutive k of a row are 16 contiguous bytes
    for (int e = tid; e < H * H / 8; e += NT) {
        const int r = e / (H / 8), k = (e % (H / 8)) * 8;
        const uint32_t o = canon_off(r, k);
        const uint4 *src = reinterpret_cast<const uint4 *>(Wb) + e;
        *reinterpret_cast<uint4 *>(W2h + o) = src[0];
        *reinterpret_cast<uint4 *>(W3h + o) = src[H * H / 8];
        *reinterpret_cast<uint4 *>(W2l + o) = src[2 * H * H / 8];
        *reinterpret_cast<uint4 *>(W3l + o) = src[3 * H * H / 8];
    }
    for (int e = tid; e < H * IN; e += NT)
        sW1[e] = P[OFF_W1 + e];
    if (tid < H) {
        sb1[tid] = P[OFF_B1 + tid];
        sb2[tid] = P[OFF_B2 + tid];
        sb3[tid] = P[OFF_B3 + tid];
        sWo[tid] = P[OFF_WO + tid];
    }
    const float bo = P[OFF_BO];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid < SLOTS) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[tid])));
        s_abort[tid] = 0;
    }
    if (tid == 0)
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    // TMEM columns of this slot: accumulator [0, 128), A hi [128, 192), A lo [192, 256)
    const uint32_t tbase = tmem_slot + (uint32_t)(slot * 256);
    const uint32_t acc = tbase, a_hi = tbase + 128, a_lo = tbase + 192;
    const uint32_t lane_base = (uint32_t)((warp % 4) * 32) << 16;  // this warp's TMEM lane quarter
    const uint32_t mb = smem_u32(&mbar[slot]);
    const bool issuer = wis == 0 && lane == 0;
    uint32_t phase = 0;
    bool pending = false;  // an MMA batch of this slot not yet waited for

    const long long tiles = (long long)((cnt + TILE - 1) / TILE);
    const long long stride = (long long)gridDim.x * SLOTS;
    auto load_feat = [&](long long t) {
        const long long e = t * TILE + row;
        return (t < tiles && e < (long long)cnt) ? p.net_feat[e] : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    float4 f = load_feat((long long)blockIdx.x * SLOTS + slot);
    for (long long t = (long long)blockIdx.x * SLOTS + slot; t < tiles; t += stride) {
        const long long e = t * TILE + row;
        const bool valid = e < (long long)cnt;
        int32_t oi = -1;
        float obase = 0.f;
        if (half == 0 && valid) {
            oi = p.net_idx[e];
            obase = p.net_base[e];
        }
        const float4 f_next = load_feat(t + stride);
        // layer 1 (FP32): 64 hidden units of this row, written to TMEM as A
#pragma unroll 1
        for (int g = 0; g < 2; g++) {
            const int k0 = half * 64 + g * 32;
            float h[32];
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const float4 w = reinterpret_cast<const float4 *>(sW1)[k0 + j];
                float z = sb1[k0 + j];
                z = fmaf(w.x, f.x, z);
                z = fmaf(w.y, f.y, z);
                z = fmaf(w.z, f.z, z);
                z = fmaf(w.w, f.w, z);
                h[j] = silu(z);
            }
            uint32_t rh[16], rl[16];
            pack32(h, rh, rl);
            tmem_st16(a_hi + lane_base + (uint32_t)(k0 / 2), rh);
            tmem_st16(a_lo + lane_base + (uint32_t)(k0 / 2), rl);
        }
        f = f_next;
        // layers 2 and 3 on the tensor cores; the other slot's tile uses the
        // CUDA cores meanwhile
        float y = 0.f;
#pragma unroll 1
        for (int layer = 0; layer < 2; layer++) {
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            fence_before();
            slot_sync(slot);
            if (issuer)
                issue_layer_ts(acc, a_hi, a_lo, smem_u32(layer ? W3h : W2h), smem_u32(layer ? W3l : W2l), mb);
            pending = true;
            const bool ok = mbar_wait(mb, phase);
            if (!ok)
                s_abort[slot] = 1;
            fence_after();
            slot_sync(slot);
            if (s_abort[slot])
                break;
            phase ^= 1u;
            pending = false;
            const float *bias = layer ? sb3 : sb2;
#pragma unroll 1
            for (int g = 0; g < 2; g++) {
                const int c0 = half * 64 + g * 32;
                float v[32];
                tmem_ld32(acc + lane_base + (uint32_t)c0, v);
                if (layer == 0) {
                    float h[32];
#pragma unroll
                    for (int j = 0; j < 32; j++)
                        h[j] = silu(v[j] + bias[c0 + j]);
                    uint32_t rh[16], rl[16];
                    pack32(h, rh, rl);
                    tmem_st16(a_hi + lane_base + (uint32_t)(c0 / 2), rh);
                    tmem_st16(a_lo + lane_base + (uint32_t)(c0 / 2), rl);
                } else {
#pragma unroll
                    for (int j = 0; j < 32; j++)
                        y = fmaf(sWo[c0 + j], silu(v[j] + bias[c0 + j]), y);
                }
            }
        }
        if (s_abort[slot])
            break;
        // output: sum the two column halves, DCS = exp(baseline + residual)
        if (half == 1)
            spart[slot][row] = y;
        slot_sync(slot);
        if (half == 0 && valid) {
            const float yy = y + spart[slot][row] + bo;
            const float r = p.norm.out_shift + yy / p.norm.out_scale;
            if (oi >= 0)
                p.out[oi] = fpconv::f64(expf(obase + r));
        }
    }
    // after an expired wait, give the slot's MMAs in flight one more bounded
    // wait before the TMEM they write is freed
    if (pending && s_abort[slot])
        mbar_wait(mb, phase);
    if (tid < SLOTS && s_abort[tid])
        atomicMax(&p.counters[2], (unsigned long long)NOA_DCS_ERROR_TIMEOUT);
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_slot), "r"(TMEM_COLS));
}

} // namespace

// ---------------------------------------------------------------- C ABI
struct noa_dcs_mlp;  // defined in mlp_train.cu
extern "C" int noa_dcs_mlp_handles(noa_dcs_mlp *m, int *process, const float **P, const void **Wb,
                                   const float **norm);

namespace {

struct InferScratch {
    int device = -1;
    int64_t cap = 0;
    void *buf = nullptr;
};
InferScratch g_scratch;  // grown on demand; one per process, guarded by g_scratch_mu
std::mutex g_scratch_mu;
thread_local char g_ierr[256] = "";

// A buffer must be device (or managed) memory of the current device before it
// reaches a kernel.
bool on_device(const void *ptr, int device) {
    if (!ptr)
        return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == device);
}

int ifail(int st, const char *msg, cudaError_t e = cudaSuccess) {
    if (e != cudaSuccess)
        snprintf(g_ierr, sizeof g_ierr, "%s: %s", msg, cudaGetErrorString(e));
    else
        snprintf(g_ierr, sizeof g_ierr, "%s", msg);
    return st;
}

} // namespace

extern "C" int noa_dcs_mlp_infer(noa_dcs_mlp *model, const uint8_t *trust, int n_seg, const noa_dcs_element *elements,
                                 const int64_t *counts, double mass, double *result, const double *K, const double *q,
                                 float tolerance, unsigned long long *stats, void *stream) {
    g_ierr[0] = '\0';
    int process = 0;
    const float *P = nullptr, *norm = nullptr;
    const void *Wb = nullptr;
    if (!model || noa_dcs_mlp_handles(model, &process, &P, &Wb, &norm))
        return ifail(NOA_DCS_ERROR_INVALID_VALUE, "invalid model");
    if (n_seg < 1 || n_seg > MAX_EL || !elements || !counts || !trust)
        return ifail(NOA_DCS_ERROR_INVALID_VALUE, "segments must number 1..16, with a trust grid");
    if (!(tolerance > 0.f && tolerance < 1.f))
        return ifail(NOA_DCS_ERROR_INVALID_VALUE, "fallback tolerance must lie in (0, 1)");
    InferParams p;
    memset(&p, 0, sizeof p);
    p.K = K;
    p.q = q;
    p.out = result;
    p.n_seg = n_seg;
    for (int s = 0; s < n_seg; s++) {
        if (counts[s] < 0)
            return ifail(NOA_DCS_ERROR_INVALID_VALUE, "negative count");
        p.seg_begin[s + 1] = p.seg_begin[s] + counts[s];
        noa_dcs_fill_consts(&p.consts[s], elements[s].A, elements[s].I, elements[s].Z, mass);
        p.logA[s] = (float)log(elements[s].A);
        p.Zf[s] = (float)elements[s].Z;
    }
    const int64_t n = p.seg_begin[n_seg];
    if (n >= (1LL << 31))
        return ifail(NOA_DCS_ERROR_INVALID_VALUE, "at most 2^31 - 1 pairs per call");
    if (n == 0)
        return NOA_DCS_SUCCESS;
    memcpy(&p.norm, norm, sizeof p.norm);
    p.trust = trust;
    // the trust grid's cells: 64 x 64 over log K in [log 1e-3, log 1e6] and
    // log(q / (K + m)) in [log 1e-7, 0], the host's cell assignment
    // (surrogate.cells) in the same float arithmetic
    p.logk_lo = (float)log(1e-3);
    p.logk_scale = (float)(64.0 / (log(1e6) - log(1e-3)));
    p.lognu_lo = (float)log(1e-7);
    p.lognu_scale = (float)(64.0 / (0.0 - log(1e-7)));
    p.tol = tolerance;
    // scratch: counters, then the two lists
    int dev = 0;
    cudaGetDevice(&dev);
    if (!on_device(K, dev) || !on_device(q, dev) || !on_device(result, dev) || !on_device(trust, dev))
        return ifail(NOA_DCS_ERROR_NOT_DEVICE_MEMORY, "K, q, result and the trust grid must be device memory");
    // one call at a time owns the scratch (calls from several host threads serialise here)
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    const size_t per = sizeof(int32_t) + sizeof(float) + sizeof(float4) + 1 + sizeof(int32_t) + 1;
    if (g_scratch.device != dev || g_scratch.cap < n) {
        if (g_scratch.buf)
            cudaFree(g_scratch.buf);
        g_scratch.buf = nullptr;
        const cudaError_t e = cudaMalloc(&g_scratch.buf, 64 + per * (size_t)n + 64);
        if (e != cudaSuccess) {
            g_scratch.cap = 0;
            return ifail(NOA_DCS_ERROR_CUDA, "cudaMalloc(inference lists)", e);
        }
        g_scratch.cap = n;
        g_scratch.device = dev;
    }
    unsigned char *b = static_cast<unsigned char *>(g_scratch.buf);
    p.counters = reinterpret_cast<unsigned long long *>(b);
    p.net_feat = reinterpret_cast<float4 *>(b + 64);
    p.net_idx = reinterpret_cast<int32_t *>(p.net_feat + n);
    p.net_base = reinterpret_cast<float *>(p.net_idx + n);
    p.fb_idx = reinterpret_cast<int32_t *>(p.net_base + n);
    p.net_seg = reinterpret_cast<uint8_t *>(p.fb_idx + n);
    p.fb_seg = p.net_seg + n;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(p.counters, 0, 64, s);
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t blocks = (n + 255) / 256;
    const int cgrid = (int)(blocks < sms * 8 ? blocks : sms * 8);
    const int64_t ctiles = (n + CL_THREADS * CL_ITEMS - 1) / (CL_THREADS * CL_ITEMS);
    const int clgrid = (int)(ctiles < sms * 8 ? ctiles : sms * 8);
    if (e == cudaSuccess) {
        if (process == NOA_DCS_PAIR_PRODUCTION)
            classify_kernel<NOA_DCS_PAIR_PRODUCTION><<<clgrid, CL_THREADS, 0, s>>>(p);
        else
            classify_kernel<NOA_DCS_PHOTONUCLEAR><<<clgrid, CL_THREADS, 0, s>>>(p);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        if (process == NOA_DCS_PAIR_PRODUCTION)
            netprep_kernel<NOA_DCS_PAIR_PRODUCTION><<<cgrid, 256, 0, s>>>(p);
        else
            netprep_kernel<NOA_DCS_PHOTONUCLEAR><<<cgrid, 256, 0, s>>>(p);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        auto k = process == NOA_DCS_PAIR_PRODUCTION ? network_kernel<NOA_DCS_PAIR_PRODUCTION>
                                                    : network_kernel<NOA_DCS_PHOTONUCLEAR>;
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_NET);
        if (e == cudaSuccess) {
            k<<<sms, NT, SMEM_NET, s>>>(p, P, static_cast<const __nv_bfloat16 *>(Wb));
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) {
        if (process == NOA_DCS_PAIR_PRODUCTION)
            fallback_kernel<NOA_DCS_PAIR_PRODUCTION><<<sms * 8, 256, 0, s>>>(p);
        else
            fallback_kernel<NOA_DCS_PHOTONUCLEAR><<<sms * 8, 256, 0, s>>>(p);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && stats)
        e = cudaMemcpyAsync(stats, p.counters, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess)
        return ifail(NOA_DCS_ERROR_CUDA, "inference launch", e);
    return NOA_DCS_SUCCESS;
}

extern "C" const char *noa_dcs_mlp_infer_last_error(void) { return g_ierr; }
