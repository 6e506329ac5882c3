/*
 * calReduction.cu -- global reductions of a substate (cal2DReduction.h,
 * cal3DReduction.h), restating OpenCAL-OMP/source/cal2DReduction.c:15-641:
 * fold every cell with max / min / sum / prod / logical and-or-xor /
 * binary and-or-xor; logical results are 0/1 and binary operations on reals
 * act on (CALint) casts.
 *
 * Two passes with a fixed grid: each block folds a grid-stride range in
 * order and reduces its threads with a fixed shuffle tree; one block then
 * folds the per-block partials in order.  The result does not depend on
 * scheduling; integer, byte, min/max, logical and binary results are exact.
 */
#define CAL_BUILDING_LIBRARY
#include <float.h>
#include <limits.h>

#include "cal_model_internal.cuh"
#include "opencal/cal2DReduction.h"
#include "opencal/cal3DReduction.h"

namespace {

constexpr int RT = 256;     /* threads per block */
constexpr int RBLOCKS = 512; /* partials */

/* accumulator: long long for byte/int (wraps like C arithmetic modulo the
 * result width), double for reals */
template <typename T>
struct Acc {
    typedef long long type;
};
template <>
struct Acc<double> {
    typedef double type;
};

template <typename A>
__device__ __forceinline__ A identity(int op)
{
    switch (op) {
    case REDUCTION_MAX: return sizeof(A) == 8 && (A)0.5 != 0 ? (A)-DBL_MAX * 2 : (A)LLONG_MIN;
    case REDUCTION_MIN: return sizeof(A) == 8 && (A)0.5 != 0 ? (A)DBL_MAX * 2 : (A)LLONG_MAX;
    case REDUCTION_PROD:
    case REDUCTION_LOGICAL_AND: return (A)1;
    case REDUCTION_BINARY_AND: return (A)-1;
    default: return (A)0;
    }
}

template <typename A>
__device__ __forceinline__ A combine(int op, A acc, A x)
{
    switch (op) {
    case REDUCTION_MAX: return acc < x ? x : acc;
    case REDUCTION_MIN: return acc > x ? x : acc;
    case REDUCTION_SUM: return acc + x;
    case REDUCTION_PROD: return acc * x;
    case REDUCTION_LOGICAL_AND: return (A)((acc != 0) && (x != 0));
    case REDUCTION_LOGICAL_OR: return (A)((acc != 0) || (x != 0));
    case REDUCTION_LOGICAL_XOR: return (A)((acc != 0) != (x != 0));
    case REDUCTION_BINARY_AND: return (A)((long long)(CALint)acc & (long long)(CALint)x);
    case REDUCTION_BINARY_OR: return (A)((long long)(CALint)acc | (long long)(CALint)x);
    case REDUCTION_BINARY_XOR: return (A)((long long)(CALint)acc ^ (long long)(CALint)x);
    default: return acc;
    }
}

/* sum and product of integers wrap: fold them in 64-bit unsigned arithmetic */
template <>
__device__ __forceinline__ long long combine<long long>(int op, long long acc, long long x)
{
    switch (op) {
    case REDUCTION_MAX: return acc < x ? x : acc;
    case REDUCTION_MIN: return acc > x ? x : acc;
    case REDUCTION_SUM: return (long long)((unsigned long long)acc + (unsigned long long)x);
    case REDUCTION_PROD: return (long long)((unsigned long long)acc * (unsigned long long)x);
    case REDUCTION_LOGICAL_AND: return (acc != 0) && (x != 0);
    case REDUCTION_LOGICAL_OR: return (acc != 0) || (x != 0);
    case REDUCTION_LOGICAL_XOR: return (acc != 0) != (x != 0);
    case REDUCTION_BINARY_AND: return (long long)((CALint)acc & (CALint)x);
    case REDUCTION_BINARY_OR: return (long long)((CALint)acc | (CALint)x);
    case REDUCTION_BINARY_XOR: return (long long)((CALint)acc ^ (CALint)x);
    default: return acc;
    }
}

template <typename A>
__device__ __forceinline__ A shfl_down(A v, int o)
{
    return __shfl_down_sync(0xffffffffu, v, o);
}

template <typename T>
__global__ void __launch_bounds__(RT) k_reduce_partial(const T* x, long long n, int op,
                                                       typename Acc<T>::type* partial)
{
    typedef typename Acc<T>::type A;
    __shared__ A warp_acc[RT / 32];
    A acc = identity<A>(op);
    for (long long c = (long long)blockIdx.x * RT + threadIdx.x; c < n; c += (long long)gridDim.x * RT)
        acc = combine<A>(op, acc, (A)x[c]);
    for (int o = 16; o > 0; o >>= 1)
        acc = combine<A>(op, acc, shfl_down<A>(acc, o));
    if ((threadIdx.x & 31) == 0)
        warp_acc[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        A b = warp_acc[0];
        for (int w = 1; w < RT / 32; w++)
            b = combine<A>(op, b, warp_acc[w]);
        partial[blockIdx.x] = b;
    }
}

template <typename T>
__global__ void k_reduce_final(const typename Acc<T>::type* partial, int nb, int op, T* out)
{
    typedef typename Acc<T>::type A;
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        A acc = partial[0];
        for (int b = 1; b < nb; b++)
            acc = combine<A>(op, acc, partial[b]);
        *out = (T)acc;
    }
}

template <typename T>
bool reduce_device(cal::CalGrid& g, int type, int slot, int op, T* out)
{
    if (op < REDUCTION_MAX || op > REDUCTION_BINARY_XOR) {
        cal::set_error(CAL_ERROR_INVALID_ARGUMENT, "reduction: unknown operation");
        return false;
    }
    if (!g.to_device_all())
        return false;
    static_assert(RBLOCKS <= 512, "the grid allocates 512 partials");
    if (!g.d_reduce_partial) {
        cal::set_error(CAL_ERROR_CUDA, "reduction: no scratch");
        return false;
    }
    typedef typename Acc<T>::type A;
    const T* x = (const T*)g.sub[type][slot].layer[0].dev;
    long long blocks = (g.ncells + RT - 1) / RT;
    if (blocks > RBLOCKS)
        blocks = RBLOCKS;
    A* partial = (A*)g.d_reduce_partial;
    k_reduce_partial<T><<<(int)blocks, RT, 0, g.stream>>>(x, g.ncells, op, partial);
    k_reduce_final<T><<<1, 32, 0, g.stream>>>(partial, (int)blocks, op, out);
    return cal::cuda_ok(cudaGetLastError(), "reduction kernels");
}

template <typename T>
T reduce_host(cal::CalGrid& g, int type, int slot, int op)
{
    if (!g.d_reduce_result) {
        cal::set_error(CAL_ERROR_CUDA, "reduction: no result word");
        return (T)0;
    }
    T v = (T)0;
    if (reduce_device<T>(g, type, slot, op, (T*)g.d_reduce_result) &&
        cal::cuda_ok(cudaMemcpyAsync(&v, g.d_reduce_result, sizeof(T), cudaMemcpyDeviceToHost, g.stream),
                     "read reduction") &&
        g.sync())
        return v;
    return (T)0;
}

inline int slot_of(cal::CalGrid& g, int type, const void* q)
{
    return (int)(((const char*)q - (const char*)g.pool[type]) / 32);
}

} // namespace

#define CAL_REDUCTION_OPS(D, S, T, TC)                                                                       \
    extern "C" T calReductionOperation##D##S(struct CALModel##D* m, struct CALSubstate##D##S* q,            \
                                             enum REDUCTION_OPERATION op)                                    \
    {                                                                                                        \
        cal::CalGrid& g = m->gpu->g;                                                                         \
        return reduce_host<T>(g, TC, slot_of(g, TC, q), (int)op);                                            \
    }                                                                                                        \
    extern "C" void calReductionOperationDevice##D##S(struct CALModel##D* m, struct CALSubstate##D##S* q,   \
                                                      enum REDUCTION_OPERATION op, T* result)                \
    {                                                                                                        \
        cal::CalGrid& g = m->gpu->g;                                                                         \
        reduce_device<T>(g, TC, slot_of(g, TC, q), (int)op, result);                                         \
    }                                                                                                        \
    extern "C" T getValue##D##S##AtIndex(struct CALSubstate##D##S* q, CALint index)                         \
    {                                                                                                        \
        cal::CalGrid* g = (cal::CalGrid*)q->cal_reserved_[0];                                                \
        if (g)                                                                                               \
            g->to_host(TC, (int)(intptr_t)q->cal_reserved_[1], 0);                                           \
        return q->current[index];                                                                            \
    }

#define CAL_REDUCTION_NAMED(D, S, T, OP, ENUM)                                                               \
    extern "C" T calReductionCompute##OP##D##S(struct CALModel##D* m, struct CALSubstate##D##S* q)          \
    {                                                                                                        \
        return calReductionOperation##D##S(m, q, ENUM);                                                      \
    }

#define CAL_REDUCTION_ALL(D, S, T, TC)                                     \
    CAL_REDUCTION_OPS(D, S, T, TC)                                         \
    CAL_REDUCTION_NAMED(D, S, T, Max, REDUCTION_MAX)                       \
    CAL_REDUCTION_NAMED(D, S, T, Min, REDUCTION_MIN)                       \
    CAL_REDUCTION_NAMED(D, S, T, Sum, REDUCTION_SUM)                       \
    CAL_REDUCTION_NAMED(D, S, T, Prod, REDUCTION_PROD)                     \
    CAL_REDUCTION_NAMED(D, S, T, LogicalAnd, REDUCTION_LOGICAL_AND)        \
    CAL_REDUCTION_NAMED(D, S, T, BinaryAnd, REDUCTION_BINARY_AND)          \
    CAL_REDUCTION_NAMED(D, S, T, LogicalOr, REDUCTION_LOGICAL_OR)          \
    CAL_REDUCTION_NAMED(D, S, T, BinaryOr, REDUCTION_BINARY_OR)            \
    CAL_REDUCTION_NAMED(D, S, T, LogicalXor, REDUCTION_LOGICAL_XOR)        \
    CAL_REDUCTION_NAMED(D, S, T, BinaryXor, REDUCTION_BINARY_XOR)

CAL_REDUCTION_ALL(2D, b, CALbyte, 0)
CAL_REDUCTION_ALL(2D, i, CALint, 1)
CAL_REDUCTION_ALL(2D, r, CALreal, 2)
CAL_REDUCTION_ALL(3D, b, CALbyte, 0)
CAL_REDUCTION_ALL(3D, i, CALint, 1)
CAL_REDUCTION_ALL(3D, r, CALreal, 2)
