/*
 * cal_tma.cuh -- tensor-memory-accelerator (TMA) staging of 2D tiles into
 * shared memory: an mbarrier with a transaction count, one
 * cp.async.bulk.tensor.2d load per tile, a bounded wait; and on the host the
 * tensor map, encoded through the runtime's driver entry point (no link to
 * libcuda).
 *
 * Rules the callers keep:
 *  - the innermost coordinate x times the element size is a multiple of 16
 *    bytes (x even for 8-byte elements); x and y may be negative or beyond
 *    the array for a load: those elements read as 0 (zero fill), which is
 *    exactly the flat boundary's "outside cells read 0";
 *  - the global base is 16-byte aligned and a row is a multiple of 16 bytes
 *    (encode_2d refuses otherwise and the caller keeps its plain loads);
 *  - the shared destination is 128-byte aligned.
 */
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace caltma {

static __device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

/* one arrival (the issuing thread) per phase; the TMA unit completes the
 * transaction bytes */
static __device__ __forceinline__ void bar_init(uint64_t* bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

static __device__ __forceinline__ void bar_expect(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

/* box at (x, y) of `map` into dst; completes `bar`'s transaction bytes */
static __device__ __forceinline__ void load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
                 "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
                 : "memory");
}

/* waits for phase `parity` of `bar` for at most `limit` polls (each poll may
 * suspend the thread for a while); true when the phase completed */
static __device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t k = 0; k < limit; k++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(smem_u32(bar)), "r"(parity)
                     : "memory");
        if (done)
            return true;
    }
    return false;
}

/* ---- host ---- */

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        else
            cudaGetLastError(); /* leave no sticky error behind */
    }
    return fn;
}

/* a 2D map over a row-major rows x cols array of esize-byte elements, box
 * bw x bh, zero fill outside the array; false when the layout does not
 * allow TMA or the driver refuses */
static inline bool encode_2d(CUtensorMap* map, const void* base, CUtensorMapDataType type, int esize, long long rows,
                             long long cols, int bw, int bh)
{
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn || ((uintptr_t)base & 15) || ((cols * esize) & 15) || bw < 1 || bw > 256 || bh < 1 || bh > 256 ||
        ((long long)bw * esize) % 16 != 0)
        return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(cols * esize)};
    cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh};
    cuuint32_t estr[2] = {1, 1};
    return fn(map, type, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

} // namespace caltma
