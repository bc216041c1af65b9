/*
 * Host side of the batched multi-element engine: the plan object of the
 * C ABI (include/noa_dcs.h, noa_dcs_batch_plan_*), its tile-shape autotuner
 * and CUDA-graph capture.
 *
 * A plan fixes the process, the precision, the particle mass and the list of
 * segments (element, count).  It owns the engine's global scratch (one tile
 * counter, allocated at creation, so that execution itself never allocates)
 * and, once captured, a graph made of the counter memset and the kernel
 * launch.  Plans are not thread-safe; use one per host thread.
 */
#include "dcs_batched.cuh"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>

using noa_dcs::BatchParams;

struct noa_dcs_batch_plan {
    int device = 0;
    int process = 0;
    int precision = 0;
    int sms = 1;
    BatchParams params;
    int threads = 256;
    int items = 4;
    int ctas_per_sm = 2;
    cudaStream_t capture_stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    const void *graph_K = nullptr, *graph_q = nullptr;
    void *graph_out = nullptr;
};

namespace {

thread_local char g_err[256] = "";

int bfail(int st, const char *msg, cudaError_t e = cudaSuccess) {
    if (e != cudaSuccess)
        snprintf(g_err, sizeof g_err, "%s: %s", msg, cudaGetErrorString(e));
    else
        snprintf(g_err, sizeof g_err, "%s", msg);
    return st;
}

// Non-negative segment counts whose running sum stays within INT64_MAX / 8,
// so that the tile ranges and the byte sizes of the overlap checks cannot
// overflow.
bool counts_fit(const int64_t *counts, int n_segments) {
    int64_t total = 0;
    for (int s = 0; s < n_segments; s++) {
        if (counts[s] > INT64_MAX / 8 - total)
            return false;
        total += counts[s];
    }
    return true;
}

size_t smem_bytes(const noa_dcs_batch_plan *p, int threads, int items) {
    const bool third = noa_dcs::batch_third_queue(p->process, p->precision);
    return threads == 128 ? noa_dcs::BatchSmem<128>::bytes(items, third)
                          : noa_dcs::BatchSmem<256>::bytes(items, third);
}

int occupancy(const noa_dcs_batch_plan *p, int threads, int items) {
    const size_t smem = smem_bytes(p, threads, items);
    return p->precision == NOA_DCS_FP64 ? noa_dcs_batched_occupancy64(p->process, threads, smem)
                                        : noa_dcs_batched_occupancy32(p->process, threads, smem);
}

// Fills the tile prefix sums for the current tile shape.
void set_tiles(noa_dcs_batch_plan *p) {
    const int64_t tile = (int64_t)p->items * p->threads;
    p->params.items = p->items;
    p->params.tile_begin[0] = 0;
    for (int s = 0; s < p->params.n_seg; s++) {
        const int64_t cnt = p->params.seg_begin[s + 1] - p->params.seg_begin[s];
        p->params.tile_begin[s + 1] = p->params.tile_begin[s] + (cnt + tile - 1) / tile;
    }
}

int launch(noa_dcs_batch_plan *p, double *out, const double *K, const double *q, cudaStream_t s) {
    p->params.K = K;
    p->params.q = q;
    p->params.out = out;
    cudaError_t e = cudaMemsetAsync(p->params.counter, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess)
        return bfail(NOA_DCS_ERROR_CUDA, "cudaMemsetAsync(counter)", e);
    const long long tiles = p->params.tile_begin[p->params.n_seg];
    long long grid = (long long)p->sms * p->ctas_per_sm;
    if (grid > tiles)
        grid = tiles > 0 ? tiles : 1;
    const size_t smem = smem_bytes(p, p->threads, p->items);
    e = p->precision == NOA_DCS_FP64
            ? noa_dcs_batched_launch64(p->process, p->threads, &p->params, (int)grid, smem, s)
            : noa_dcs_batched_launch32(p->process, p->threads, &p->params, (int)grid, smem, s);
    if (e != cudaSuccess)
        return bfail(NOA_DCS_ERROR_CUDA, "batched kernel launch", e);
    return NOA_DCS_SUCCESS;
}

void drop_graph(noa_dcs_batch_plan *p) {
    if (p->graph) {
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
    p->graph_K = p->graph_q = nullptr;
    p->graph_out = nullptr;
}

int check_buffers(const noa_dcs_batch_plan *p, const void *out, const void *K, const void *q) {
    const int64_t n = p->params.seg_begin[p->params.n_seg];
    if (n == 0)
        return NOA_DCS_SUCCESS;
    const void *bufs[3] = {out, K, q};
    for (const void *b : bufs) {
        if (!b)
            return bfail(NOA_DCS_ERROR_INVALID_VALUE, "NULL buffer");
        if ((uintptr_t)b % 8u)
            return bfail(NOA_DCS_ERROR_MISALIGNED, "buffer not 8-byte aligned");
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, b) != cudaSuccess) {
            cudaGetLastError();
            return bfail(NOA_DCS_ERROR_NOT_DEVICE_MEMORY, "buffer is not device memory");
        }
        if ((a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) ||
            (a.type == cudaMemoryTypeDevice && a.device != p->device))
            return bfail(NOA_DCS_ERROR_NOT_DEVICE_MEMORY, "buffer is not device memory of the plan's device");
    }
    const uintptr_t o0 = (uintptr_t)out, o1 = o0 + (uintptr_t)n * 8u;
    for (const void *b : {K, q}) {
        const uintptr_t b0 = (uintptr_t)b, b1 = b0 + (uintptr_t)n * 8u;
        if (b != out && o0 < b1 && b0 < o1)
            return bfail(NOA_DCS_ERROR_OVERLAP, "result partially overlaps an input");
    }
    return NOA_DCS_SUCCESS;
}

} // namespace

extern "C" {

int noa_dcs_batch_plan_create(noa_dcs_batch_plan **out_plan, int process, int precision, int n_segments,
                              const noa_dcs_element *elements, const int64_t *counts, double mass) {
    g_err[0] = '\0';
    if (!out_plan)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "plan pointer is NULL");
    *out_plan = nullptr;
    if (process < 0 || process > 3 || (precision != NOA_DCS_FP64 && precision != NOA_DCS_FP32C))
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "unknown process or precision");
    if (n_segments < 1 || n_segments > NOA_DCS_MAX_SEGMENTS || !elements || !counts)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "segments must number 1..16 with elements and counts");
    if (!std::isfinite(mass) || !(mass > 0.))
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "invalid particle mass");
    for (int s = 0; s < n_segments; s++) {
        const noa_dcs_element &el = elements[s];
        if (!std::isfinite(el.A) || !(el.A > 0.) || !std::isfinite(el.I) || !(el.I > 0.) || el.Z < 1)
            return bfail(NOA_DCS_ERROR_INVALID_ELEMENT, "invalid element");
        if (counts[s] < 0)
            return bfail(NOA_DCS_ERROR_INVALID_VALUE, "negative segment count");
    }
    if (!counts_fit(counts, n_segments))
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "segment counts add up past INT64_MAX / 8");
    noa_dcs_batch_plan *p = new (std::nothrow) noa_dcs_batch_plan();
    if (!p)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "out of host memory");
    std::memset(&p->params, 0, sizeof p->params);
    cudaError_t e = cudaGetDevice(&p->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device);
    if (e != cudaSuccess) {
        delete p;
        return bfail(NOA_DCS_ERROR_CUDA, "device query", e);
    }
    p->process = process;
    p->precision = precision;
    p->params.n_seg = n_segments;
    p->params.tol = NOA_DCS_FP32C_DEFAULT_TOL;
    p->params.seg_begin[0] = 0;
    for (int s = 0; s < n_segments; s++) {
        p->params.seg_begin[s + 1] = p->params.seg_begin[s] + counts[s];
        noa_dcs_fill_consts(&p->params.consts[s], elements[s].A, elements[s].I, elements[s].Z, mass);
    }
    set_tiles(p);
    e = cudaMalloc((void **)&p->params.counter, sizeof(unsigned long long));
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&p->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        if (p->params.counter)
            cudaFree(p->params.counter);
        delete p;
        return bfail(NOA_DCS_ERROR_CUDA, "plan allocation", e);
    }
    *out_plan = p;
    return NOA_DCS_SUCCESS;
}

int noa_dcs_batch_plan_set_tile(noa_dcs_batch_plan *p, int threads, int items, int ctas_per_sm) {
    if (!p || (threads != 128 && threads != 256) || items < 1 || items > 8 || ctas_per_sm < 1 || ctas_per_sm > 16)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "tile shape: threads 128|256, items 1..8, ctas_per_sm 1..16");
    const int occ = occupancy(p, threads, items);
    if (occ < 1)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "tile shape does not fit on an SM");
    p->threads = threads;
    p->items = items;
    p->ctas_per_sm = ctas_per_sm < occ ? ctas_per_sm : occ;
    set_tiles(p);
    drop_graph(p);
    return NOA_DCS_SUCCESS;
}

int noa_dcs_batch_plan_get_tile(const noa_dcs_batch_plan *p, int *threads, int *items, int *ctas_per_sm) {
    if (!p || !threads || !items || !ctas_per_sm)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "NULL argument");
    *threads = p->threads;
    *items = p->items;
    *ctas_per_sm = p->ctas_per_sm;
    return NOA_DCS_SUCCESS;
}

int noa_dcs_batch_plan_set_tolerance(noa_dcs_batch_plan *p, float tolerance) {
    if (!p || !(tolerance > 0.f) || !(tolerance < 1.f))
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "tolerance must lie in (0, 1)");
    p->params.tol = tolerance;
    drop_graph(p);
    return NOA_DCS_SUCCESS;
}

int noa_dcs_batch_plan_execute(noa_dcs_batch_plan *p, double *result, const double *K, const double *q,
                               void *stream) {
    g_err[0] = '\0';
    if (!p)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "plan is NULL");
    int st = check_buffers(p, result, K, q);
    if (st)
        return st;
    if (p->params.seg_begin[p->params.n_seg] == 0)
        return NOA_DCS_SUCCESS;
    return launch(p, result, K, q, (cudaStream_t)stream);
}

int noa_dcs_batch_plan_execute_graph(noa_dcs_batch_plan *p, double *result, const double *K, const double *q,
                                     void *stream) {
    g_err[0] = '\0';
    if (!p)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "plan is NULL");
    int st = check_buffers(p, result, K, q);
    if (st)
        return st;
    if (p->params.seg_begin[p->params.n_seg] == 0)
        return NOA_DCS_SUCCESS;
    if (!p->graph || p->graph_K != K || p->graph_q != q || p->graph_out != result) {
        drop_graph(p);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(p->capture_stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess)
            return bfail(NOA_DCS_ERROR_CUDA, "cudaStreamBeginCapture", e);
        st = launch(p, result, K, q, p->capture_stream);
        e = cudaStreamEndCapture(p->capture_stream, &g);
        if (st)
            return st;
        if (e != cudaSuccess)
            return bfail(NOA_DCS_ERROR_CUDA, "cudaStreamEndCapture", e);
        e = cudaGraphInstantiate(&p->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            p->graph = nullptr;
            return bfail(NOA_DCS_ERROR_CUDA, "cudaGraphInstantiate", e);
        }
        p->graph_K = K;
        p->graph_q = q;
        p->graph_out = result;
    }
    const cudaError_t e = cudaGraphLaunch(p->graph, (cudaStream_t)stream);
    if (e != cudaSuccess)
        return bfail(NOA_DCS_ERROR_CUDA, "cudaGraphLaunch", e);
    return NOA_DCS_SUCCESS;
}

int noa_dcs_batch_plan_autotune(noa_dcs_batch_plan *p, double *result, const double *K, const double *q,
                                void *stream, int64_t sample_per_segment) {
    g_err[0] = '\0';
    if (!p)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "plan is NULL");
    int st = check_buffers(p, result, K, q);
    if (st)
        return st;
    if (p->params.seg_begin[p->params.n_seg] == 0)
        return NOA_DCS_SUCCESS;
    // Tune on a prefix of every segment (the pairs are i.i.d. within a
    // segment): a plan copy whose tile list covers only the first
    // sample_per_segment pairs of each segment, in place in the full buffers.
    noa_dcs_batch_plan t = *p;
    t.graph = nullptr;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int bt = p->threads, bi = p->items, bc = p->ctas_per_sm;
    const int thread_opts[2] = {128, 256};
    const int item_opts[4] = {1, 2, 4, 8};
    for (int ti = 0; ti < 2; ti++) {
        for (int ii = 0; ii < 4; ii++) {
            const int occ = occupancy(p, thread_opts[ti], item_opts[ii]);
            if (occ < 1)
                continue;
            const int cta_opts[4] = {1, 2, 4, occ};
            for (int ci = 0; ci < 4; ci++) {
                if (cta_opts[ci] > occ || (ci == 3 && (occ == 1 || occ == 2 || occ == 4)))
                    continue;
                t.threads = thread_opts[ti];
                t.items = item_opts[ii];
                t.ctas_per_sm = cta_opts[ci];
                // tiles per segment of the sample, laid out on the full buffers
                const int64_t tile = (int64_t)t.items * t.threads;
                t.params.items = t.items;
                t.params.tile_begin[0] = 0;
                for (int s = 0; s < t.params.n_seg; s++) {
                    int64_t cnt = p->params.seg_begin[s + 1] - p->params.seg_begin[s];
                    if (sample_per_segment > 0 && cnt > sample_per_segment)
                        cnt = sample_per_segment;
                    t.params.tile_begin[s + 1] = t.params.tile_begin[s] + (cnt + tile - 1) / tile;
                }
                float ms_sum = 0.f;
                bool ok = true;
                for (int rep = 0; rep < 3 && ok; rep++) {
                    cudaEventRecord(e0, (cudaStream_t)stream);
                    ok = launch(&t, result, K, q, (cudaStream_t)stream) == NOA_DCS_SUCCESS;
                    cudaEventRecord(e1, (cudaStream_t)stream);
                    if (cudaEventSynchronize(e1) != cudaSuccess)
                        ok = false;
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (rep > 0)
                        ms_sum += ms;
                }
                if (ok && ms_sum < best) {
                    best = ms_sum;
                    bt = t.threads;
                    bi = t.items;
                    bc = t.ctas_per_sm;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best >= 1e30f)
        return bfail(NOA_DCS_ERROR_CUDA, "autotune: no candidate ran");
    return noa_dcs_batch_plan_set_tile(p, bt, bi, bc);
}

int noa_dcs_batch_plan_destroy(noa_dcs_batch_plan *p) {
    if (!p)
        return NOA_DCS_SUCCESS;
    drop_graph(p);
    if (p->capture_stream)
        cudaStreamDestroy(p->capture_stream);
    if (p->params.counter)
        cudaFree(p->params.counter);
    delete p;
    return NOA_DCS_SUCCESS;
}

const char *noa_dcs_batch_last_error(void) { return g_err; }

} // extern "C"

// ---------------------------------------------------------------- allocation-free batched entry point
//
// Some callers cannot let a library allocate device memory: a host
// application that gives all of the GPU's memory to its own arena at
// start-up and owns every allocation, or a transport loop that may not pay
// for an allocation's device synchronisation.  For them the batched engine also runs with its only
// scratch -- the 64-bit tile counter -- in the static device array below
// instead of in a plan.  Every device that loads this library holds these
// 256 bytes until the process exits.

#define NOA_DCS_NOALLOC_SCRATCH_WORDS 32 /* 256 bytes; the engine uses word 0 */

static __device__ __align__(256) unsigned long long noa_dcs_noalloc_scratch[NOA_DCS_NOALLOC_SCRATCH_WORDS];

namespace {

constexpr int kNoallocDevices = 64;
std::mutex g_noalloc_mu;
unsigned long long *g_noalloc_addr[kNoallocDevices] = {};

// Device address of the static scratch on the current device.  The symbol's
// host-side name is not a device address, so the address is looked up once
// per device, with that device current, and cached.
int noalloc_scratch(int device, unsigned long long **out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, noa_dcs_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return bfail(NOA_DCS_ERROR_CUDA, "cudaGetSymbolAddress(noa_dcs_noalloc_scratch)", e);
        g_noalloc_addr[device] = static_cast<unsigned long long *>(ptr);
    }
    *out = g_noalloc_addr[device];
    return NOA_DCS_SUCCESS;
}

} // namespace

extern "C" int noa_dcs_cuda_vmap_batched_noalloc(int process, int precision, int n_segments,
                                                 const noa_dcs_element *elements, const int64_t *counts,
                                                 double mass, double *result, const double *K, const double *q,
                                                 void *stream) {
    g_err[0] = '\0';
    if (process < 0 || process > 3 || (precision != NOA_DCS_FP64 && precision != NOA_DCS_FP32C))
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "unknown process or precision");
    if (n_segments < 1 || !elements || !counts)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "need at least one segment with its element and count");
    if (n_segments > NOA_DCS_MAX_SEGMENTS)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE,
                     "too many segments for the allocation-free entry point (maximum 16 per call)");
    if (!std::isfinite(mass) || !(mass > 0.))
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "invalid particle mass");
    // The plan object on the stack: no host or device allocation.
    noa_dcs_batch_plan p;
    std::memset(&p.params, 0, sizeof p.params);
    for (int s = 0; s < n_segments; s++) {
        const noa_dcs_element &el = elements[s];
        if (!std::isfinite(el.A) || !(el.A > 0.) || !std::isfinite(el.I) || !(el.I > 0.) || el.Z < 1)
            return bfail(NOA_DCS_ERROR_INVALID_ELEMENT, "invalid element");
        if (counts[s] < 0)
            return bfail(NOA_DCS_ERROR_INVALID_VALUE, "negative segment count");
    }
    if (!counts_fit(counts, n_segments))
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "segment counts add up past INT64_MAX / 8");
    cudaError_t e = cudaGetDevice(&p.device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&p.sms, cudaDevAttrMultiProcessorCount, p.device);
    if (e != cudaSuccess)
        return bfail(NOA_DCS_ERROR_CUDA, "device query", e);
    if (p.device < 0 || p.device >= kNoallocDevices)
        return bfail(NOA_DCS_ERROR_INVALID_VALUE, "device ordinal out of range");
    p.process = process;
    p.precision = precision;
    p.params.n_seg = n_segments;
    p.params.tol = NOA_DCS_FP32C_DEFAULT_TOL;
    for (int s = 0; s < n_segments; s++) {
        p.params.seg_begin[s + 1] = p.params.seg_begin[s] + counts[s];
        noa_dcs_fill_consts(&p.params.consts[s], elements[s].A, elements[s].I, elements[s].Z, mass);
    }
    // Fixed tile shape (the plan default): 256 threads x 4 pairs, 2 CTAs per
    // SM.  Its queues take 43 KB of shared memory, 54 KB for FP32C pair
    // production (a third queue); above 48 KB the launch raises the kernel's
    // limit once per device, on its first call there.
    p.threads = 256;
    p.items = 4;
    p.ctas_per_sm = 2;
    set_tiles(&p);
    int st = check_buffers(&p, result, K, q);
    if (st)
        return st;
    if (p.params.seg_begin[n_segments] == 0)
        return NOA_DCS_SUCCESS;
    if ((st = noalloc_scratch(p.device, &p.params.counter)))
        return st;
    // launch() zeroes the counter on the stream before the kernel.
    return launch(&p, result, K, q, (cudaStream_t)stream);
}
