/*
 * Instantiations of the batched engine (dcs_batched.cuh) for precision
 * NOA_DCS_FP64; the other precision lives in its own translation unit so the
 * two compile in parallel.
 */
#include "dcs_batched.cuh"

namespace noa_dcs {

// One opt-in flag table per kernel instantiation (see smem_optin_once).
template <int PROC, int THREADS>
static std::atomic<bool> g_optin[kSmemOptinDevices];

template <int PROC, int THREADS>
static cudaError_t launch_one(const void *params, int grid, size_t smem, cudaStream_t s) {
    auto k = dcs_batched_kernel<PROC, NOA_DCS_FP64, THREADS>;
    const cudaError_t e = smem_optin_once(k, smem, g_optin<PROC, THREADS>);
    if (e != cudaSuccess)
        return e;
    k<<<grid, THREADS, smem, s>>>(*static_cast<const BatchParams *>(params));
    return cudaGetLastError();
}

template <int PROC, int THREADS>
static int occupancy_one(size_t smem) {
    auto k = dcs_batched_kernel<PROC, NOA_DCS_FP64, THREADS>;
    if (smem_optin_once(k, smem, g_optin<PROC, THREADS>) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, THREADS, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

template <int THREADS>
static cudaError_t dispatch(int process, const void *params, int grid, size_t smem, cudaStream_t s) {
    switch (process) {
    case NOA_DCS_PROC_BREMS:
        return launch_one<NOA_DCS_PROC_BREMS, THREADS>(params, grid, smem, s);
    case NOA_DCS_PROC_PPROD:
        return launch_one<NOA_DCS_PROC_PPROD, THREADS>(params, grid, smem, s);
    case NOA_DCS_PROC_PHOTO:
        return launch_one<NOA_DCS_PROC_PHOTO, THREADS>(params, grid, smem, s);
    case NOA_DCS_PROC_ION:
        return launch_one<NOA_DCS_PROC_ION, THREADS>(params, grid, smem, s);
    default:
        return cudaErrorInvalidValue;
    }
}

template <int THREADS>
static int occ_dispatch(int process, size_t smem) {
    switch (process) {
    case NOA_DCS_PROC_BREMS:
        return occupancy_one<NOA_DCS_PROC_BREMS, THREADS>(smem);
    case NOA_DCS_PROC_PPROD:
        return occupancy_one<NOA_DCS_PROC_PPROD, THREADS>(smem);
    case NOA_DCS_PROC_PHOTO:
        return occupancy_one<NOA_DCS_PROC_PHOTO, THREADS>(smem);
    default:
        return occupancy_one<NOA_DCS_PROC_ION, THREADS>(smem);
    }
}

} // namespace noa_dcs

cudaError_t noa_dcs_batched_launch64(int process, int threads, const void *params, int grid, size_t smem,
                                     cudaStream_t stream) {
    if (threads == 128)
        return noa_dcs::dispatch<128>(process, params, grid, smem, stream);
    if (threads == 256)
        return noa_dcs::dispatch<256>(process, params, grid, smem, stream);
    return cudaErrorInvalidValue;
}

int noa_dcs_batched_occupancy64(int process, int threads, size_t smem) {
    return threads == 128 ? noa_dcs::occ_dispatch<128>(process, smem) : noa_dcs::occ_dispatch<256>(process, smem);
}
