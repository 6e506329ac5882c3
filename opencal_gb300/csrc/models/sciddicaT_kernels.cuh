/*
 * sciddicaT_kernels.cuh -- device code of the SCIDDICA-T step shared by the
 * forward paths (sciddicaT.cu) and the adjoint (sciddicaT_adjoint.cu): the
 * wet test, the outflow computation (the reference's minimisation of
 * differences, operation by operation) and the single fused step kernel.
 * Reference: OpenCAL-OMP/examples/calomp_sciddicaT/source/sciddicaT.c:36-100.
 */
#pragma once

#include <stdlib.h>
#include <string.h>

#include "cal_tma.cuh"
#include "exact_div.cuh"

namespace sdt {

/* The fused step.  A block owns a TW x TH tile.  EP 1 (outflows) runs on the
 * tile plus a ring of 1 cell -- EP 2 needs the outflows of every neighbour --
 * so z and h are staged on the tile plus a ring of 2.  Shared memory holds
 * z, h (load region) and the four outflows (outflow region). */
constexpr int THREADS = 256;

struct Params {
    const double* __restrict__ z;
    const double* __restrict__ h;
    double* __restrict__ h_next;
    int rows, cols;
    int toroidal;
    double eps, r;
    long long eps_bits;
    /* dense step only, optional: per tile (row-major over the launch grid)
     * bit 0 = a cell of the tile is wet before the step, bit 1 = after */
    unsigned char* tile_wet = nullptr;
};

/* h > eps as the reference evaluates `!(h <= eps)`, on the bit pattern:
 * for a non-negative double the IEEE encoding orders like the value; NaN
 * compares false with <= and therefore counts as wet */
static __device__ __forceinline__ bool is_wet(double h, long long eps_bits)
{
    const long long b = __double_as_longlong(h);
    if (b >= 0)
        return b > eps_bits;                                  /* +0 .. +inf, +NaN */
    return (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; /* -NaN; other negatives are dry */
}

/* The outflows of one wet cell, exactly as sciddicaT_flows_computation:
 * the same additions in the same order; the division by the number of
 * remaining cells and the comparisons are done on the integer pipe with
 * bit-identical results (exact_div.cuh). */
static __device__ __forceinline__ void outflows_u0(double hc, double u0, const double u1, const double u2,
                                                   const double u3, const double u4, double eps, double r,
                                                   double f[4], unsigned* elim_out = nullptr);

static __device__ __forceinline__ void outflows(double hc, double zc, const double u1, const double u2,
                                                const double u3, const double u4, double eps, double r, double f[4],
                                                unsigned* elim_out = nullptr)
{
    outflows_u0(hc, zc + eps, u1, u2, u3, u4, eps, r, f, elim_out);
}

/* the same with u[0] = z + eps of the cell given (a caller that keeps it
 * per cell saves the addition) */
static __device__ __forceinline__ void outflows_u0(double hc, double u0, const double u1, const double u2,
                                                   const double u3, const double u4, double eps, double r,
                                                   double f[4], unsigned* elim_out)
{
    double u[5];
    const double m = hc - eps;
    u[0] = u0;
    u[1] = u1;
    u[2] = u2;
    u[3] = u3;
    u[4] = u4;
    unsigned elim = 0;
    double average;
    bool again;
    do {
        again = false;
        average = m;
        int cells_count = 0;
#pragma unroll
        for (int n = 0; n < 5; n++)
            if (!(elim & (1u << n))) {
                average += u[n];
                cells_count++;
            }
        if (cells_count != 0)
            average = cal_div_small(average, cells_count);
#pragma unroll
        for (int n = 0; n < 5; n++)
            if (!(elim & (1u << n)) && cal_le(average, u[n])) {
                elim |= 1u << n;
                again = true;
            }
    } while (again);
#pragma unroll
    for (int n = 1; n < 5; n++)
        f[n - 1] = (elim & (1u << n)) ? 0.0 : (average - u[n]) * r;
    if (elim_out)
        *elim_out = elim; /* bit n: neighbour n (1..4) eliminated; bit 0: the cell itself */
}

static __device__ __forceinline__ int wrapi(int x, int n)
{
    return x < 0 ? x + n : (x >= n ? x - n : x);
}

static __device__ __forceinline__ double plus_zero(double x)
{
    /* x + 0.0 without the FP64 pipe: only -0.0 changes (to +0.0) */
    long long b = __double_as_longlong(x);
    return __longlong_as_double(b == (long long)0x8000000000000000ULL ? 0LL : b);
}

template <int TW, int TH>
struct Tile {
    static constexpr int R1W = TW + 2, R1H = TH + 2; /* outflow region */
    static constexpr int R2W = TW + 4, R2H = TH + 4; /* load region */
    /* z, h (load region), four outflows (outflow region), then the compacted
     * list of wet cells of the outflow region (16-bit indices) and its count */
    static constexpr size_t list_offset = sizeof(double) * (2 * R2W * R2H + 4 * R1W * R1H);
    static constexpr size_t smem_bytes =
        list_offset + ((sizeof(unsigned short) * ((R1W * R1H + 1) & ~1) + sizeof(int) + 15) / 16) * 16;
};

/* append the lanes whose predicate holds to a shared-memory list (one
 * shared atomic per warp) */
static __device__ __forceinline__ void warp_append_shared(bool pred, int value, unsigned short* list, int* count)
{
    const unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0)
        return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0)
        base = atomicAdd(count, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (pred)
        list[base + __popc(mask & ((1u << lane) - 1u))] = (unsigned short)value;
}

/* one TW x TH tile of one step; i0, j0 = tile origin; smem sized
 * Tile<TW, TH>::smem_bytes; every thread of the block calls it.  With TRACK
 * the block-uniform result has bit 0 set when a cell of the tile was wet
 * before the step and bit 1 when one is wet after it (0 without TRACK). */
template <int TW, int TH, bool TRACK = false>
__device__ __forceinline__ int fused_tile(const Params& p, int i0, int j0, double* smem, bool staged = false,
                                          unsigned char* elim_tile = nullptr)
{
    using T = Tile<TW, TH>;
    double* sz = smem;                      /* [R2H][R2W] */
    double* sh = sz + T::R2W * T::R2H;      /* [R2H][R2W] */
    double* sf = sh + T::R2W * T::R2H;      /* [4][R1H][R1W] */
    constexpr int F = T::R1W * T::R1H;

    /* 16-byte loads need an even row length and 16-byte aligned fields */
    const bool interior = i0 >= 2 && j0 >= 2 && i0 + TH + 2 <= p.rows && j0 + TW + 2 <= p.cols && (p.cols & 1) == 0 &&
                          ((reinterpret_cast<unsigned long long>(p.z) | reinterpret_cast<unsigned long long>(p.h)) &
                           15) == 0;

    /* 1. z and h on the tile + 2 ring.  Interior tiles: 16-byte loads (j0-2
     * is even, so every pair starts 16-byte aligned).  Edge tiles: flat ->
     * 0 outside, toroidal -> wrapped. */
    int wet_seen = 0, wet_in = 0, wet_out = 0;
    if (staged) {
        /* z and h are in shared memory already (TMA, zero outside a flat
         * grid): only the wet flags */
        for (int t = threadIdx.x; t < T::R2H * T::R2W; t += THREADS) {
            const int a = t / T::R2W, b = t - a * T::R2W;
            const int w = is_wet(sh[t], p.eps_bits);
            wet_seen |= w;
            if (TRACK && a >= 2 && a < TH + 2 && b >= 2 && b < TW + 2 && i0 - 2 + a < p.rows && j0 - 2 + b < p.cols)
                wet_in |= w;
        }
    } else if (interior) {
        constexpr int PW = T::R2W / 2;
        for (int t = threadIdx.x; t < PW * T::R2H; t += THREADS) {
            const int a = t / PW, b = 2 * (t - a * PW);
            const long long c = (long long)(i0 - 2 + a) * p.cols + (j0 - 2 + b);
            const double2 zv = __ldg(reinterpret_cast<const double2*>(p.z + c));
            const double2 hv = __ldg(reinterpret_cast<const double2*>(p.h + c));
            *reinterpret_cast<double2*>(sz + a * T::R2W + b) = zv;
            *reinterpret_cast<double2*>(sh + a * T::R2W + b) = hv;
            const int w = is_wet(hv.x, p.eps_bits) | is_wet(hv.y, p.eps_bits);
            wet_seen |= w;
            if (TRACK && a >= 2 && a < TH + 2 && b >= 2 && b < TW + 2)
                wet_in |= w;
        }
    } else {
        for (int t = threadIdx.x; t < T::R2H * T::R2W; t += THREADS) {
            const int a = t / T::R2W, b = t - a * T::R2W;
            int gi = i0 - 2 + a, gj = j0 - 2 + b;
            double zv = 0.0, hv = 0.0;
            bool inside = (unsigned)gi < (unsigned)p.rows && (unsigned)gj < (unsigned)p.cols;
            if (!inside && p.toroidal) {
                gi = wrapi(gi, p.rows);
                gj = wrapi(gj, p.cols);
                inside = true;
            }
            if (inside) {
                const long long c = (long long)gi * p.cols + gj;
                zv = __ldg(p.z + c);
                hv = __ldg(p.h + c);
            }
            sz[t] = zv;
            sh[t] = hv;
            const int w = is_wet(hv, p.eps_bits);
            wet_seen |= w;
            if (TRACK && a >= 2 && a < TH + 2 && b >= 2 && b < TW + 2 && i0 - 2 + a < p.rows && j0 - 2 + b < p.cols)
                wet_in |= w;
        }
    }
    if (threadIdx.x == 0)
        *reinterpret_cast<int*>(reinterpret_cast<unsigned short*>(reinterpret_cast<char*>(smem) + T::list_offset) +
                                ((T::R1W * T::R1H + 1) & ~1)) = 0;
    if (__syncthreads_or(wet_seen) == 0) {
        /* no wet cell within two cells: h is unchanged (-0 becomes +0) */
        for (int t = threadIdx.x; t < TH * TW; t += THREADS) {
            const int a = t / TW, b = t - a * TW;
            const int gi = i0 + a, gj = j0 + b;
            if (gi < p.rows && gj < p.cols)
                p.h_next[(long long)gi * p.cols + gj] = plus_zero(sh[(a + 2) * T::R2W + b + 2]);
        }
        return 0;
    }

    /* 2. EP 1 on the tile + 1 ring; cells outside a flat grid have none.
     * 2a: outflows start at +0 and the wet cells are compacted into a list,
     * 2b: one thread per listed cell, so that the FP64 work of a warp is not
     * spread over the dry lanes of a partly wet tile. */
    unsigned short* s_list = reinterpret_cast<unsigned short*>(reinterpret_cast<char*>(smem) + T::list_offset);
    int* s_count = reinterpret_cast<int*>(s_list + ((F + 1) & ~1));
    for (int t0 = 0; t0 < F; t0 += THREADS) {
        const int t = t0 + threadIdx.x;
        bool wet = false;
        if (t < F) {
            const int a = t / T::R1W, b = t - a * T::R1W;
            const int gi = i0 - 1 + a, gj = j0 - 1 + b;
            const bool inside = p.toroidal || ((unsigned)gi < (unsigned)p.rows && (unsigned)gj < (unsigned)p.cols);
            wet = inside && is_wet(sh[(a + 1) * T::R2W + (b + 1)], p.eps_bits);
#pragma unroll
            for (int q = 0; q < 4; q++)
                sf[q * F + t] = 0.0;
        }
        warp_append_shared(wet, t, s_list, s_count);
    }
    __syncthreads();
    const int nwet = *s_count;
    for (int k = threadIdx.x; k < nwet; k += THREADS) {
        const int t = s_list[k];
        const int a = t / T::R1W, b = t - a * T::R1W;
        const int c = (a + 1) * T::R2W + (b + 1); /* this cell in the load region */
        /* von Neumann order n = 1..4: north, west, east, south; u = z + h */
        const double u1 = sz[c - T::R2W] + sh[c - T::R2W];
        const double u2 = sz[c - 1] + sh[c - 1];
        const double u3 = sz[c + 1] + sh[c + 1];
        const double u4 = sz[c + T::R2W] + sh[c + T::R2W];
        double f[4];
        unsigned elim;
        outflows(sh[c], sz[c], u1, u2, u3, u4, p.eps, p.r, f, &elim);
#pragma unroll
        for (int q = 0; q < 4; q++)
            sf[q * F + t] = f[q];
        /* the tile's own cells' elimination sets, for an adjoint that
         * reuses them (elim_tile: TW x TH bytes, row-major) */
        if (elim_tile && a >= 1 && a <= TH && b >= 1 && b <= TW)
            elim_tile[(a - 1) * TW + (b - 1)] = (unsigned char)elim;
    }
    __syncthreads();

    /* 3. EP 2 on the tile: h' = h + sum_n (f_in(n) - f_out(n-1)), n = 1..4 */
    for (int t = threadIdx.x; t < TH * TW; t += THREADS) {
        const int a = t / TW, b = t - a * TW;
        const int gi = i0 + a, gj = j0 + b;
        if (gi >= p.rows || gj >= p.cols)
            continue;
        const int c = (a + 1) * T::R1W + (b + 1); /* this cell in the outflow region */
        /* inflow from neighbour n is its outflow f[4-n] */
        const double in1 = sf[3 * F + c - T::R1W], in2 = sf[2 * F + c - 1];
        const double in3 = sf[1 * F + c + 1], in4 = sf[0 * F + c + T::R1W];
        const double o0 = sf[0 * F + c], o1 = sf[1 * F + c], o2 = sf[2 * F + c], o3 = sf[3 * F + c];
        const double hc = sh[(a + 2) * T::R2W + b + 2];
        double hn;
        const long long any = __double_as_longlong(in1) | __double_as_longlong(in2) | __double_as_longlong(in3) |
                              __double_as_longlong(in4) | __double_as_longlong(o0) | __double_as_longlong(o1) |
                              __double_as_longlong(o2) | __double_as_longlong(o3);
        if (any == 0) {
            hn = plus_zero(hc);
        } else {
            hn = hc;
            hn += in1 - o0;
            hn += in2 - o1;
            hn += in3 - o2;
            hn += in4 - o3;
        }
        p.h_next[(long long)gi * p.cols + gj] = hn;
        if (TRACK)
            wet_out |= is_wet(hn, p.eps_bits);
    }
    if (TRACK) {
        /* __syncthreads_or returns non-zero, not the OR of the values: one
         * barrier per bit */
        const int before = __syncthreads_or(wet_in) ? 1 : 0;
        const int after = __syncthreads_or(wet_out) ? 2 : 0;
        return before | after;
    }
    return 0;
}

template <int TW, int TH>
__global__ void __launch_bounds__(THREADS) fused_step(const __grid_constant__ Params p)
{
    extern __shared__ __align__(16) double smem[];
    if (p.tile_wet) {
        const int wet = fused_tile<TW, TH, true>(p, blockIdx.y * TH, blockIdx.x * TW, smem);
        if (threadIdx.x == 0)
            p.tile_wet[blockIdx.y * gridDim.x + blockIdx.x] = (unsigned char)wet;
    } else {
        fused_tile<TW, TH>(p, blockIdx.y * TH, blockIdx.x * TW, smem);
    }
}

/* The dense step with z and h staged by TMA: thread 0 arms an mbarrier with
 * the two boxes' bytes and issues one cp.async.bulk.tensor.2d load per
 * field (box R2W x R2H at (j0 - 2, i0 - 2); j0 - 2 is even, so x * 8 bytes
 * is a multiple of 16); cells outside the array arrive as +0, which is the
 * flat boundary's rule, so every tile of a flat grid takes this path.  The
 * wait is bounded: a block whose copies do not complete counts itself in
 * *timeouts, waits once more (bounded) for the copies in flight and leaves
 * its tile unwritten. */
constexpr uint32_t TMA_WAIT_LIMIT = 1u << 22;

template <int TW, int TH>
__global__ void __launch_bounds__(THREADS) fused_step_tma(const __grid_constant__ Params p,
                                                          const __grid_constant__ CUtensorMap tz,
                                                          const __grid_constant__ CUtensorMap th, int* timeouts)
{
    using T = Tile<TW, TH>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    double* smem = reinterpret_cast<double*>(smem_raw + ((128u - (caltma::smem_u32(smem_raw) & 127u)) & 127u));
    const int i0 = blockIdx.y * TH, j0 = blockIdx.x * TW;
    if (threadIdx.x == 0) {
        caltma::bar_init(&bar);
        caltma::bar_expect(&bar, 2u * T::R2W * T::R2H * (uint32_t)sizeof(double));
        caltma::load_2d(smem, &tz, j0 - 2, i0 - 2, &bar);
        caltma::load_2d(smem + T::R2W * T::R2H, &th, j0 - 2, i0 - 2, &bar);
    }
    __syncthreads(); /* the barrier is initialised before anyone waits on it */
    const bool done = caltma::bar_wait(&bar, 0, TMA_WAIT_LIMIT);
    if (!__syncthreads_and(done)) {
        if (threadIdx.x == 0) {
            atomicAdd(timeouts, 1);
            caltma::bar_wait(&bar, 0, TMA_WAIT_LIMIT);
        }
        __syncthreads();
        return;
    }
    if (p.tile_wet) {
        const int wet = fused_tile<TW, TH, true>(p, i0, j0, smem, true);
        if (threadIdx.x == 0)
            p.tile_wet[blockIdx.y * gridDim.x + blockIdx.x] = (unsigned char)wet;
    } else {
        fused_tile<TW, TH>(p, i0, j0, smem, true);
    }
}

/* TMA launches queued and blocks whose copies timed out, per translation
 * unit that launches the dense step */
static long long g_tma_launches = 0;
static __device__ int g_tma_timeouts;

static int* tma_timeouts_ptr()
{
    static int* ptr = nullptr;
    if (!ptr && cudaGetSymbolAddress((void**)&ptr, g_tma_timeouts) != cudaSuccess)
        ptr = nullptr;
    return ptr;
}

/* OPENCAL_SDT_TMA=0 keeps the plain loads (for comparison) */
static bool tma_enabled()
{
    const char* e = getenv("OPENCAL_SDT_TMA");
    return !(e && !strcmp(e, "0"));
}

/* queues the TMA form of the dense step; false (nothing queued) for a
 * toroidal grid or a layout TMA cannot address */
template <int TW, int TH>
static bool launch_tma(const Params& p, cudaStream_t s)
{
    using T = Tile<TW, TH>;
    if (p.toroidal || !tma_enabled())
        return false;
    int* timeouts = tma_timeouts_ptr();
    CUtensorMap tz, th;
    if (!timeouts ||
        !caltma::encode_2d(&tz, p.z, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, p.rows, p.cols, T::R2W, T::R2H) ||
        !caltma::encode_2d(&th, p.h, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, p.rows, p.cols, T::R2W, T::R2H))
        return false;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(fused_step_tma<TW, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)T::smem_bytes + 128);
        attr_set = true;
    }
    dim3 grid((p.cols + TW - 1) / TW, (p.rows + TH - 1) / TH);
    fused_step_tma<TW, TH><<<grid, THREADS, T::smem_bytes + 128, s>>>(p, tz, th, timeouts);
    g_tma_launches++;
    return true;
}

template <int TW, int TH>
static void launch(const Params& p, cudaStream_t s)
{
    if (launch_tma<TW, TH>(p, s))
        return;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(fused_step<TW, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)Tile<TW, TH>::smem_bytes);
        attr_set = true;
    }
    dim3 grid((p.cols + TW - 1) / TW, (p.rows + TH - 1) / TH);
    fused_step<TW, TH><<<grid, THREADS, Tile<TW, TH>::smem_bytes, s>>>(p);
}

/* tile shape: 32 x 16 by default (at 2048 x 2048, 1000 steps from the
 * bench's initial state: 35.0 us per step against 55.3 for 64 x 32, 39.4
 * for 32 x 8, 62.6 for 16 x 8); OPENCAL_SDT_TILE=16x8|32x8|32x16|64x16|64x32
 * overrides */
static int tile_choice()
{
    static int choice = -1;
    if (choice < 0) {
        const char* e = getenv("OPENCAL_SDT_TILE");
        choice = 0;
        if (e && !strcmp(e, "64x32"))
            choice = 2;
        else if (e && !strcmp(e, "32x16"))
            choice = 0;
        else if (e && !strcmp(e, "64x16"))
            choice = 1;
        else if (e && !strcmp(e, "16x8"))
            choice = 3;
        else if (e && !strcmp(e, "32x8"))
            choice = 4;
    }
    return choice;
}

static void launch_step(const Params& p, cudaStream_t s)
{
    switch (tile_choice()) {
    case 0: launch<32, 16>(p, s); break;
    case 1: launch<64, 16>(p, s); break;
    case 3: launch<16, 8>(p, s); break;
    case 4: launch<32, 8>(p, s); break;
    default: launch<64, 32>(p, s); break;
    }
}

} // namespace sdt
