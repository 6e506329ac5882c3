/*
 * cal_noalloc.cu -- active-cell compaction for callers that cannot allocate
 * device memory (calCompactActiveCellsNoAlloc2D, declared in cal2D.h).
 *
 * calUpdateActiveCells2D compacts the flags of a model into buffers the
 * model allocated with cudaMalloc, including a scratch array of per-block
 * counts.  Some callers cannot make that allocation: a host that has handed
 * all device memory to its own allocator at start-up, or a simulation loop
 * that must never call cudaMalloc/cudaFree because those calls can
 * synchronise the device.  This entry point runs the same two-pass
 * compaction on flags and output buffers that the caller owns, and keeps the
 * per-block counts in a fixed array in device memory that is part of the
 * library image instead of allocating it.
 *
 * Limits and sharing:
 *   - the scratch array holds a ticket word and CAL_NOALLOC_MAX_BLOCKS
 *     counts, so the grid may have at most CAL_NOALLOC_MAX_CELLS cells;
 *     larger grids are rejected with CAL_ERROR_LIMIT and nothing is
 *     launched;
 *   - every call on a device uses the same array: calls whose kernels
 *     overlap on the GPU (different streams, or different host threads
 *     without ordering) race on it.  Order them on one stream.
 *   - the array keeps the previous call's contents.  Only the ticket (which
 *     elects the block that scans the counts) must start at zero; each call
 *     clears it on its stream before its kernels run.  The per-block counts
 *     are written by the first pass before anything reads them;
 *   - the array lives on every GPU that loads the library until the process
 *     exits.
 * Alignment: `flags` may have any alignment (it is read a byte per lane);
 * `cells`, `linear` and `count` must be 4-byte aligned, else the call
 * returns CAL_ERROR_INVALID_ARGUMENT and launches nothing.
 * Set-up: the device address of the array is looked up once per device
 * (cudaGetSymbolAddress, with that device current) on the first call made
 * on it; that first call should therefore come before any stream capture.
 * The address is kept for the rest of the process, so a cudaDeviceReset
 * after the first call on a device is not supported.
 */
#define CAL_BUILDING_LIBRARY
#include <mutex>

#include "cal_core.cuh"
#include "opencal/cal2D.h"

#define CAL_NOALLOC_MAX_BLOCKS 65536
#define CAL_NOALLOC_HEAD_INTS 32 /* the ticket, on a 128-byte line of its own */
#define CAL_NOALLOC_MAX_DEVICES 64

/* the compaction's scratch: ticket line, then per-block counts (4096 flags
 * per block) */
static __device__ __align__(256) int cal_noalloc_block_counts[CAL_NOALLOC_HEAD_INTS + CAL_NOALLOC_MAX_BLOCKS];

static std::mutex g_setup_mutex;
static int* g_scratch[CAL_NOALLOC_MAX_DEVICES];

/* device address of the scratch array on the current device (set-up on the
 * first call per device) */
static int* scratch_for_current_device()
{
    int dev = 0;
    if (!cal::cuda_ok(cudaGetDevice(&dev), "cudaGetDevice"))
        return nullptr;
    if (dev < 0 || dev >= CAL_NOALLOC_MAX_DEVICES) {
        cal::set_error(CAL_ERROR_LIMIT, "calCompactActiveCellsNoAlloc2D: device index out of range");
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch[dev]) {
        void* ptr = nullptr;
        if (!cal::cuda_ok(cudaGetSymbolAddress(&ptr, cal_noalloc_block_counts),
                          "cudaGetSymbolAddress(no-alloc scratch)"))
            return nullptr;
        g_scratch[dev] = (int*)ptr;
    }
    return g_scratch[dev];
}

extern "C" int calCompactActiveCellsNoAlloc2D(const CALbyte* flags, int rows, int columns, struct CALCell2D* cells,
                                              int* linear, int* count, void* stream)
{
    if (!flags || !cells || !linear || !count || rows <= 0 || columns <= 0) {
        cal::set_error(CAL_ERROR_INVALID_ARGUMENT, "calCompactActiveCellsNoAlloc2D: null buffer or empty grid");
        return CAL_ERROR_INVALID_ARGUMENT;
    }
    if ((((uintptr_t)cells) | ((uintptr_t)linear) | ((uintptr_t)count)) & 3u) {
        cal::set_error(CAL_ERROR_INVALID_ARGUMENT,
                       "calCompactActiveCellsNoAlloc2D: cells, linear and count must be 4-byte aligned");
        return CAL_ERROR_INVALID_ARGUMENT;
    }
    const long long ncells = (long long)rows * columns;
    if (ncells > (long long)CAL_NOALLOC_MAX_CELLS ||
        cal::compact_scratch_ints(ncells) > CAL_NOALLOC_HEAD_INTS + CAL_NOALLOC_MAX_BLOCKS) {
        cal::set_error(CAL_ERROR_LIMIT, "calCompactActiveCellsNoAlloc2D: grid larger than CAL_NOALLOC_MAX_CELLS "
                                        "(268435456 cells)");
        return CAL_ERROR_LIMIT;
    }
    int* scratch = scratch_for_current_device();
    if (!scratch)
        return calGetLastError();
    /* the ticket starts at zero whatever an earlier call left */
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(int), (cudaStream_t)stream);
    if (e == cudaSuccess)
        e = cal::compact_flags((const unsigned char*)flags, 2, rows, columns, 1, (int*)cells, linear, count, scratch,
                               CAL_NOALLOC_HEAD_INTS + CAL_NOALLOC_MAX_BLOCKS, (cudaStream_t)stream);
    if (!cal::cuda_ok(e, "calCompactActiveCellsNoAlloc2D"))
        return CAL_ERROR_CUDA;
    return CAL_SUCCESS;
}
