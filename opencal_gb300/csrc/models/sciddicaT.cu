/*
 * sciddicaT.cu -- the SCIDDICA-T debris-flow model on opencal-gb300.
 *
 * Two ways to run the same model, both through the C API:
 *
 * 1. The reference program as written (OpenCAL-OMP/examples/calomp_sciddicaT/
 *    source/sciddicaT.c:36-136 plain; OpenCAL/examples/
 *    cal_sciddicaT-activecells-glut/source/sciddicaT.c:20-146 active cells):
 *    elementary processes are device functions registered with
 *    calAddElementaryProcess2D; init and steering are host callbacks.  Exact
 *    reference semantics, including the active-cell list and the update after
 *    every process.
 *
 * 2. The fused step (plain mode): one kernel per step computes the outflows
 *    (EP 1) on the tile plus a one-cell ring in shared memory and the
 *    thickness update (EP 2) on the tile, then the h layers are swapped.  The
 *    outflows never reach memory: after a plain-mode step the steering
 *    resets them to 0 everywhere, so they are 0 at every step boundary and a
 *    step is fully determined by z and h.  HBM traffic per cell-update:
 *    z read 8 B + h read 8 B + h write 8 B = 24 B.
 *    Arithmetic is the reference's, operation by operation (same evaluation
 *    order, IEEE division, no FMA contraction: the file is built with
 *    --fmad=false), so results are bit-identical to serial OpenCAL.
 *    Dry cells (h <= epsilon, tested on the bit pattern) and cells whose
 *    whole neighbourhood is dry take no FP64 instruction at all: on GB300 the
 *    FP64 pipe is narrow, and x + 0.0 - 0.0 leaves x unchanged except for
 *    turning -0.0 into +0.0, which is reproduced with an integer select.
 *    For the same reason the division by the number of remaining cells and
 *    the comparisons of the minimisation run on the integer pipe, with
 *    bit-identical results (exact_div.cuh).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "exact_div.cuh"
#include "opencal/cal2D.h"
#include "opencal/cal2DRun.h"

#define NUMBER_OF_OUTFLOWS 4

/* ======================= 1. the reference program ======================= */

struct sciddicaTSubstates {
    struct CALSubstate2Dr* z;
    struct CALSubstate2Dr* h;
    struct CALSubstate2Dr* f[NUMBER_OF_OUTFLOWS];
};
struct sciddicaTParameters {
    CALParameterr epsilon;
    CALParameterr r;
    int active;
    int steps; /* run length used by the device stop condition */
};

__managed__ struct sciddicaTSubstates Q;
__managed__ struct sciddicaTParameters P;

CAL_ELEMENTARY_PROCESS_2D(sciddicaT_flows_computation)(struct CALModel2D* sciddicaT, int i, int j)
{
    CALbyte eliminated_cells[5] = {CAL_FALSE, CAL_FALSE, CAL_FALSE, CAL_FALSE, CAL_FALSE};
    CALbyte again;
    CALint cells_count;
    CALreal average;
    CALreal m;
    CALreal u[5];
    CALint n;
    CALreal z, h;

    if (calGet2Dr(sciddicaT, Q.h, i, j) <= P.epsilon)
        return;

    m = calGet2Dr(sciddicaT, Q.h, i, j) - P.epsilon;
    u[0] = calGet2Dr(sciddicaT, Q.z, i, j) + P.epsilon;
    for (n = 1; n < sciddicaT->sizeof_X; n++) {
        z = calGetX2Dr(sciddicaT, Q.z, i, j, n);
        h = calGetX2Dr(sciddicaT, Q.h, i, j, n);
        u[n] = z + h;
    }
    do {
        again = CAL_FALSE;
        average = m;
        cells_count = 0;
        for (n = 0; n < sciddicaT->sizeof_X; n++)
            if (!eliminated_cells[n]) {
                average += u[n];
                cells_count++;
            }
        if (cells_count != 0)
            average /= cells_count;
        for (n = 0; n < sciddicaT->sizeof_X; n++)
            if ((average <= u[n]) && (!eliminated_cells[n])) {
                eliminated_cells[n] = CAL_TRUE;
                again = CAL_TRUE;
            }
    } while (again);

    for (n = 1; n < sciddicaT->sizeof_X; n++)
        if (eliminated_cells[n]) {
            calSet2Dr(sciddicaT, Q.f[n - 1], i, j, 0.0);
        } else {
            calSet2Dr(sciddicaT, Q.f[n - 1], i, j, (average - u[n]) * P.r);
            if (P.active)
                calAddActiveCellX2D(sciddicaT, i, j, n);
        }
}

CAL_ELEMENTARY_PROCESS_2D(sciddicaT_width_update)(struct CALModel2D* sciddicaT, int i, int j)
{
    CALreal h_next;
    CALint n;
    h_next = calGet2Dr(sciddicaT, Q.h, i, j);
    for (n = 1; n < sciddicaT->sizeof_X; n++)
        h_next += calGetX2Dr(sciddicaT, Q.f[NUMBER_OF_OUTFLOWS - n], i, j, n) - calGet2Dr(sciddicaT, Q.f[n - 1], i, j);
    calSet2Dr(sciddicaT, Q.h, i, j, h_next);
}

CAL_ELEMENTARY_PROCESS_2D(sciddicaT_remove_inactive_cells)(struct CALModel2D* sciddicaT, int i, int j)
{
    if (calGet2Dr(sciddicaT, Q.h, i, j) <= P.epsilon)
        calRemoveActiveCell2D(sciddicaT, i, j);
}

/* the active-cells example's stop condition (cal_sciddicaT-activecells-glut/
 * source/sciddicaT.c:149-154: step >= STEPS), evaluated on the GPU */
CAL_DEVICE_STOP_CONDITION_2D(sciddicaT_device_stop)(struct CALModel2D* sciddicaT)
{
    return calRunGetStep2D(sciddicaT) >= P.steps ? CAL_TRUE : CAL_FALSE;
}

/* host callbacks (sciddicaT.c:104-140) */
static void sciddicaT_simulation_init(struct CALModel2D* sciddicaT)
{
    CALreal z, h;
    CALint i, j;
    calInitSubstate2Dr(sciddicaT, Q.f[0], 0);
    calInitSubstate2Dr(sciddicaT, Q.f[1], 0);
    calInitSubstate2Dr(sciddicaT, Q.f[2], 0);
    calInitSubstate2Dr(sciddicaT, Q.f[3], 0);
    for (i = 0; i < sciddicaT->rows; i++)
        for (j = 0; j < sciddicaT->columns; j++) {
            h = calGet2Dr(sciddicaT, Q.h, i, j);
            if (h > 0.0) {
                z = calGet2Dr(sciddicaT, Q.z, i, j);
                calSet2Dr(sciddicaT, Q.z, i, j, z - h);
                if (P.active)
                    calAddActiveCell2D(sciddicaT, i, j);
            }
        }
}

static void sciddicaT_steering_plain(struct CALModel2D* sciddicaT)
{
    for (int q = 0; q < NUMBER_OF_OUTFLOWS; q++)
        calInitSubstate2Dr(sciddicaT, Q.f[q], 0);
}

static void sciddicaT_steering_ac(struct CALModel2D* sciddicaT)
{
    for (int q = 0; q < NUMBER_OF_OUTFLOWS; q++)
        calInitSubstateNext2Dr(sciddicaT, Q.f[q], 0);
}

/* ======================= 2. the fused step ============================== */

#include "sciddicaT_kernels.cuh"

/* ======================= 2b. the split step ============================= */
/* The same step as two kernels, so that the FP64 work of the outflows is
 * spread over the whole GPU instead of the few tiles the wet region covers:
 *
 *   K1 (outflows): one thread per WET cell, from a compact list built by the
 *      previous K2; writes the four outflows of the cell into private
 *      outflow arrays (never the model's f substates, which keep the 0 the
 *      steering gives them) and flags the K2 tiles that will read them.  It
 *      also clears the outflows of cells that dried up in the previous step
 *      (a second list, disjoint from the first).
 *   K2 (thickness update): only the tiles K1 flagged.  K1 appends every
 *      tile it flags to a tile work-list once per step (the flag is an epoch
 *      stamp, so it never needs clearing); K2 is a fixed grid of blocks that
 *      take work items from that list and update their tile's h in place
 *      (each cell reads and writes only its own h; the outflows it reads were
 *      completed by K1), then apply EP 1's wet test to the new h and append
 *      wet cells (and cells that just dried) to the next step's lists.  In
 *      every other tile all outflows in and out are +0, so h is unchanged
 *      bit for bit: K2's remaining work items carry the wet cells of the
 *      current list that lie in unflagged tiles over to the next list.
 *
 * The result is the reference's: EP 1's body runs exactly on the cells
 * where the reference runs it (h > epsilon), and a cell EP 2 does not visit
 * here is one where the reference's EP 2 adds eight zero terms.  The lists'
 * order does not matter: each cell's result depends only on its
 * neighbourhood.  A priming kernel canonicalises -0 to +0 in h (the first
 * reference step adds 0.0 to every cell) and builds the first wet list. */
namespace sdt2 {

constexpr int THREADS = 256;
constexpr int TW = 64, TH = 16; /* K2 tile: 16 rows x 64 columns, 4 cells per thread */

struct State {
    struct CALModel2D* ca = nullptr;
    double* f = nullptr;         /* 4 * n outflows, SoA */
    int* list[2] = {nullptr, nullptr};
    int* zlist[2] = {nullptr, nullptr};
    int* counts = nullptr;       /* [0..1] wet list lengths, [2..3] dried list lengths,
                                    [4] list parity, [5] K2 block ticket, [6] step epoch,
                                    [7] flagged tiles */
    int* tflag = nullptr;        /* per K2 tile: epoch of the step that flagged it */
    int* tlist = nullptr;        /* flagged tiles of the current step */
    long long n = 0;
    int tiles_x = 0, tiles_y = 0;
    bool primed = false;
};

/* The lists alternate between two buffers; which one a step reads is the
 * parity word counts[4], flipped by the last K2 block of the step, which
 * also advances the epoch counts[6] and empties the tile list counts[7].
 * Keeping them in device memory makes every step's launches identical, so a
 * step can be recorded once as a CUDA graph and replayed. */
struct K1Params {
    const double* __restrict__ z;
    const double* __restrict__ h;
    double* __restrict__ f;
    int* list0;
    int* list1;
    int* zlist0;
    int* zlist1;
    int* counts;
    int* tflag;
    int* tlist;
    int rows, cols, toroidal, tiles_x;
    long long n;
    double eps, r;
};

struct K2Params {
    double* __restrict__ h;
    const double* __restrict__ f;
    int* list0;
    int* list1;
    int* zlist0;
    int* zlist1;
    int* counts;
    const int* tflag;
    const int* tlist;
    int rows, cols, toroidal, tiles_x;
    long long n;
    long long eps_bits;
};

static __device__ __forceinline__ int tile_of(int i, int j, int tiles_x)
{
    return (i / TH) * tiles_x + (j / TW);
}

constexpr int K1_THREADS = 64; /* small blocks: the wet list spreads over every SM */
constexpr int K2_BLOCKS = 152 * 4;

/* flag tile t for this step's K2 and append it to the work-list once */
static __device__ __forceinline__ void flag_tile(int* tflag, int* tlist, int* tcount, int t, int epoch)
{
    if (tflag[t] != epoch && atomicExch(tflag + t, epoch) != epoch)
        tlist[atomicAdd(tcount, 1)] = t;
}

__global__ void __launch_bounds__(K1_THREADS) k1_outflows(const __grid_constant__ K1Params p)
{
    const int par = p.counts[4];
    const int epoch = p.counts[6];
    const int* list = par ? p.list1 : p.list0;
    const int* zlist = par ? p.zlist1 : p.zlist0;
    if (blockIdx.x == 0 && threadIdx.x < 2)
        p.counts[(1 - par) + 2 * threadIdx.x] = 0; /* the lists K2 will append to */
    const int stride = gridDim.x * blockDim.x;
    const int nw = p.counts[par];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nw; k += stride) {
        const int c = list[k];
        const int i = c / p.cols, j = c - i * p.cols;
        /* neighbours in von Neumann order n = 1..4: north, west, east, south */
        int ni[4] = {i - 1, i, i, i + 1}, nj[4] = {j, j - 1, j + 1, j};
        double u[4];
        bool in[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int a = ni[q], b = nj[q];
            in[q] = true;
            if (p.toroidal) {
                a = a < 0 ? a + p.rows : (a >= p.rows ? a - p.rows : a);
                b = b < 0 ? b + p.cols : (b >= p.cols ? b - p.cols : b);
            } else if ((unsigned)a >= (unsigned)p.rows || (unsigned)b >= (unsigned)p.cols) {
                in[q] = false;
            }
            ni[q] = a;
            nj[q] = b;
            if (in[q]) {
                const long long cn = (long long)a * p.cols + b;
                u[q] = __ldg(p.z + cn) + __ldg(p.h + cn);
            } else {
                u[q] = 0.0 + 0.0; /* an absent neighbour reads z = 0, h = 0 */
            }
        }
        double f[4];
        sdt::outflows(__ldg(p.h + c), __ldg(p.z + c), u[0], u[1], u[2], u[3], p.eps, p.r, f);
        bool any = false;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            p.f[q * p.n + c] = f[q];
            if (__double_as_longlong(f[q]) != 0) {
                any = true;
                if (in[q]) /* the receiver reads it */
                    flag_tile(p.tflag, p.tlist, p.counts + 7, tile_of(ni[q], nj[q], p.tiles_x), epoch);
            }
        }
        if (any)
            flag_tile(p.tflag, p.tlist, p.counts + 7, tile_of(i, j, p.tiles_x), epoch);
    }
    const int nz = p.counts[2 + par];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nz; k += stride) {
        const int c = zlist[k];
#pragma unroll
        for (int q = 0; q < 4; q++)
            p.f[q * p.n + c] = 0.0;
    }
}

/* append the lanes whose predicate holds to list/count (warp-aggregated) */
static __device__ __forceinline__ void warp_append(bool pred, int value, int* list, int* count)
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
        list[base + __popc(mask & ((1u << lane) - 1u))] = value;
}

/* Block-wide append of up to 4 items per thread to two lists, one atomicAdd
 * per list per block.  want[q] / dried[q]: item q goes to list / zlist. */
static __device__ __forceinline__ void block_append4(const bool want[4], const bool dried[4], const int value[4],
                                                     int* list, int* count, int* zlist, int* zcount)
{
    __shared__ int s_warp[2][THREADS / 32];
    __shared__ int s_base[2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    unsigned mw[4], md[4];
    int nw = 0, nd = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        mw[q] = __ballot_sync(0xffffffffu, want[q]);
        md[q] = __ballot_sync(0xffffffffu, dried[q]);
        nw += __popc(mw[q]);
        nd += __popc(md[q]);
    }
    if (lane == 0) {
        s_warp[0][warp] = nw;
        s_warp[1][warp] = nd;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        int tot = 0;
        for (int w = 0; w < THREADS / 32; w++)
            tot += s_warp[threadIdx.x][w];
        s_base[threadIdx.x] = tot ? atomicAdd(threadIdx.x == 0 ? count : zcount, tot) : 0;
    }
    __syncthreads();
    int bw = s_base[0], bd = s_base[1];
    for (int w = 0; w < warp; w++) {
        bw += s_warp[0][w];
        bd += s_warp[1][w];
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (want[q])
            list[bw + __popc(mw[q] & below)] = value[q];
        if (dried[q])
            zlist[bd + __popc(md[q] & below)] = value[q];
        bw += __popc(mw[q]);
        bd += __popc(md[q]);
    }
}

/* one flagged tile: h += inflows - outflows in place, then the wet test */
static __device__ __forceinline__ void k2_tile(const K2Params& p, int tile, int* list, int* count, int* zlist,
                                               int* zcount)
{
    const int ty = tile / p.tiles_x, tx = tile - ty * p.tiles_x;
    const int r = threadIdx.x / (TW / 4);       /* 0..15 */
    const int j4 = (threadIdx.x % (TW / 4)) * 4; /* 0, 4, ..., 60 */
    const int i = ty * TH + r;
    const int jb = tx * TW + j4;
    const long long c0 = (long long)i * p.cols + jb;
    double hv[4] = {0.0, 0.0, 0.0, 0.0};
    bool cell[4];
    const bool full = i < p.rows && jb + 3 < p.cols && (p.cols & 1) == 0;
    if (full) {
        /* c0 is a multiple of 2 (jb and cols even): two 16-byte loads */
        const double2 a = *reinterpret_cast<const double2*>(p.h + c0);
        const double2 b = *reinterpret_cast<const double2*>(p.h + c0 + 2);
        hv[0] = a.x;
        hv[1] = a.y;
        hv[2] = b.x;
        hv[3] = b.y;
#pragma unroll
        for (int q = 0; q < 4; q++)
            cell[q] = true;
    } else {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            cell[q] = i < p.rows && jb + q < p.cols;
            if (cell[q])
                hv[q] = p.h[c0 + q];
        }
    }
    bool want[4], dried[4];
    int value[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int j = jb + q;
        const long long c = c0 + q;
        double hn = hv[q];
        if (cell[q]) {
            const double o0 = p.f[c], o1 = p.f[p.n + c], o2 = p.f[2 * p.n + c], o3 = p.f[3 * p.n + c];
            /* inflow from neighbour n is its outflow f[4-n]; absent neighbours give 0 */
            double in1 = 0.0, in2 = 0.0, in3 = 0.0, in4 = 0.0;
            int a = i - 1, b = j - 1, d = j + 1, e = i + 1;
            if (p.toroidal) {
                a = a < 0 ? a + p.rows : a;
                e = e >= p.rows ? e - p.rows : e;
                b = b < 0 ? b + p.cols : b;
                d = d >= p.cols ? d - p.cols : d;
            }
            if ((unsigned)a < (unsigned)p.rows)
                in1 = p.f[3 * p.n + (long long)a * p.cols + j];
            if ((unsigned)b < (unsigned)p.cols)
                in2 = p.f[2 * p.n + (long long)i * p.cols + b];
            if ((unsigned)d < (unsigned)p.cols)
                in3 = p.f[1 * p.n + (long long)i * p.cols + d];
            if ((unsigned)e < (unsigned)p.rows)
                in4 = p.f[(long long)e * p.cols + j];
            const long long any = __double_as_longlong(in1) | __double_as_longlong(in2) |
                                  __double_as_longlong(in3) | __double_as_longlong(in4) |
                                  __double_as_longlong(o0) | __double_as_longlong(o1) |
                                  __double_as_longlong(o2) | __double_as_longlong(o3);
            if (any != 0) {
                double x = hv[q];
                x += in1 - o0;
                x += in2 - o1;
                x += in3 - o2;
                x += in4 - o3;
                hn = x;
                p.h[c] = x;
            }
        }
        const bool wb = cell[q] && sdt::is_wet(hv[q], p.eps_bits);
        want[q] = cell[q] && sdt::is_wet(hn, p.eps_bits);
        dried[q] = wb && !want[q];
        value[q] = (int)c;
    }
    block_append4(want, dried, value, list, count, zlist, zcount);
}

/* K2: a fixed grid working through the flagged tiles, then through the
 * current wet list in chunks of THREADS entries (carrying over the wet
 * cells of unflagged tiles, whose h did not change) */
__global__ void __launch_bounds__(THREADS) k2_update(const __grid_constant__ K2Params p)
{
    const int par = p.counts[4];
    const int epoch = p.counts[6];
    const int ntiles = p.counts[7];
    const int nwet = p.counts[par];
    const int* cur = par ? p.list1 : p.list0;
    int* list = par ? p.list0 : p.list1; /* next step's lists */
    int* zlist = par ? p.zlist0 : p.zlist1;
    int* count = p.counts + (1 - par);
    int* zcount = p.counts + 2 + (1 - par);
    const int items = ntiles + (nwet + THREADS - 1) / THREADS;
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        if (item < ntiles) {
            k2_tile(p, p.tlist[item], list, count, zlist, zcount);
            __syncthreads(); /* block_append4's shared words are reused */
        } else {
            const int k = (item - ntiles) * THREADS + threadIdx.x;
            bool carry = false;
            int c = 0;
            if (k < nwet) {
                c = cur[k];
                const int i = c / p.cols, j = c - i * p.cols;
                carry = p.tflag[tile_of(i, j, p.tiles_x)] != epoch;
            }
            warp_append(carry, c, list, count);
        }
    }
    if (threadIdx.x == 0) {
        /* every block read parity, epoch and counts at its start; the last
         * one to finish advances them for the next step (no block waits for
         * another) */
        __threadfence();
        if (atomicAdd(reinterpret_cast<unsigned*>(p.counts + 5), 1u) == gridDim.x - 1) {
            p.counts[4] = 1 - par;
            p.counts[5] = 0;
            p.counts[6] = epoch + 1;
            p.counts[7] = 0;
        }
    }
}

/* -0 -> +0 in h and the first wet list (counts[parity] must be 0) */
__global__ void __launch_bounds__(THREADS) k_prime(double* h, long long n, long long eps_bits, int* list, int* count)
{
    if (blockIdx.x == 0 && threadIdx.x == 0)
        count[6] = 1; /* first epoch (tile stamps start at 0) */
    for (long long c0 = (long long)blockIdx.x * blockDim.x; c0 < n; c0 += (long long)gridDim.x * blockDim.x) {
        const long long c = c0 + threadIdx.x;
        bool wet = false;
        if (c < n) {
            const double hv = h[c];
            if (__double_as_longlong(hv) == (long long)0x8000000000000000ULL)
                h[c] = 0.0;
            wet = sdt::is_wet(hv, eps_bits);
        }
        warp_append(wet, (int)c, list, count);
    }
}

static State g_state;

static void release()
{
    State& s = g_state;
    cudaFree(s.f);
    for (int k = 0; k < 2; k++) {
        cudaFree(s.list[k]);
        cudaFree(s.zlist[k]);
    }
    cudaFree(s.counts);
    cudaFree(s.tflag);
    cudaFree(s.tlist);
    s = State();
}

/* (re)allocate for `ca` and prime from the current h */
static bool prime(struct CALModel2D* ca, double* h, long long eps_bits, cudaStream_t st)
{
    State& s = g_state;
    const long long n = (long long)ca->rows * ca->columns;
    if (s.ca != ca || s.n != n) {
        release();
        s.ca = ca;
        s.n = n;
        s.tiles_x = (ca->columns + TW - 1) / TW;
        s.tiles_y = (ca->rows + TH - 1) / TH;
        bool ok = cudaMalloc(&s.f, 4 * n * sizeof(double)) == cudaSuccess &&
                  cudaMalloc(&s.counts, 8 * sizeof(int)) == cudaSuccess &&
                  cudaMalloc(&s.tflag, sizeof(int) * s.tiles_x * s.tiles_y) == cudaSuccess &&
                  cudaMalloc(&s.tlist, sizeof(int) * s.tiles_x * s.tiles_y) == cudaSuccess;
        for (int k = 0; k < 2 && ok; k++)
            ok = cudaMalloc(&s.list[k], n * sizeof(int)) == cudaSuccess &&
                 cudaMalloc(&s.zlist[k], n * sizeof(int)) == cudaSuccess;
        if (!ok) {
            release();
            return false;
        }
    }
    cudaMemsetAsync(s.f, 0, 4 * n * sizeof(double), st);
    cudaMemsetAsync(s.counts, 0, 8 * sizeof(int), st); /* parity 0, ticket 0, no flagged tile */
    cudaMemsetAsync(s.tflag, 0, sizeof(int) * s.tiles_x * s.tiles_y, st);
    int blocks = (int)((n + THREADS - 1) / THREADS);
    if (blocks > 152 * 16)
        blocks = 152 * 16;
    k_prime<<<blocks, THREADS, 0, st>>>(h, n, eps_bits, s.list[0], s.counts + 0);
    s.primed = true;
    return cudaGetLastError() == cudaSuccess;
}

/* one step: K1 then K2 on the model's stream; false on a CUDA error */
static bool step(struct CALModel2D* ca, const double* z, double* h, double eps, double r, long long eps_bits,
                 cudaStream_t st, cudaEvent_t* ev /* optional: 3 events around K1 and K2 */)
{
    State& s = g_state;
    K1Params a;
    a.z = z;
    a.h = h;
    a.f = s.f;
    a.list0 = s.list[0];
    a.list1 = s.list[1];
    a.zlist0 = s.zlist[0];
    a.zlist1 = s.zlist[1];
    a.counts = s.counts;
    a.tflag = s.tflag;
    a.tlist = s.tlist;
    a.rows = ca->rows;
    a.cols = ca->columns;
    a.toroidal = ca->T == CAL_SPACE_TOROIDAL;
    a.tiles_x = s.tiles_x;
    a.n = s.n;
    a.eps = eps;
    a.r = r;
    K2Params b;
    b.h = h;
    b.f = s.f;
    b.list0 = s.list[0];
    b.list1 = s.list[1];
    b.zlist0 = s.zlist[0];
    b.zlist1 = s.zlist[1];
    b.counts = s.counts;
    b.tflag = s.tflag;
    b.tlist = s.tlist;
    b.rows = ca->rows;
    b.cols = ca->columns;
    b.toroidal = a.toroidal;
    b.tiles_x = s.tiles_x;
    b.n = s.n;
    b.eps_bits = eps_bits;
    if (ev)
        cudaEventRecord(ev[0], st);
    k1_outflows<<<152 * 32, K1_THREADS, 0, st>>>(a);
    if (ev)
        cudaEventRecord(ev[1], st);
    k2_update<<<K2_BLOCKS, THREADS, 0, st>>>(b);
    if (ev)
        cudaEventRecord(ev[2], st);
    return cudaGetLastError() == cudaSuccess;
}

} // namespace sdt2

static bool sdt_use_split()
{
    const char* e = getenv("OPENCAL_SDT_KERNEL");
    return !(e && !strcmp(e, "single"));
}

/* the split step as a global transition (h updated in place) */
static void sciddicaT_split_transition_timed(struct CALModel2D* ca, cudaEvent_t* ev)
{
    const double* z = (const double*)calGetDeviceBuffer2Dr(ca, Q.z, 0);
    double* h = (double*)calGetDeviceBuffer2Dr(ca, Q.h, 0);
    cudaStream_t st = (cudaStream_t)calGetStream2D(ca);
    long long eps_bits;
    memcpy(&eps_bits, &P.epsilon, sizeof(double));
    if (sdt2::g_state.ca != ca || !sdt2::g_state.primed)
        sdt2::prime(ca, h, eps_bits, st);
    sdt2::step(ca, z, h, P.epsilon, P.r, eps_bits, st, ev);
    calMarkCurrentWritten2Dr(ca, Q.h);
}

static void sciddicaT_split_invalidate() { sdt2::g_state.primed = false; }

/* prime now (eagerly) if the next split step would: keeps the priming out of
 * a step that is being recorded as a graph */
static void sciddicaT_split_prepare(struct CALModel2D* ca)
{
    if (!sdt_use_split() || (sdt2::g_state.ca == ca && sdt2::g_state.primed))
        return;
    long long eps_bits;
    memcpy(&eps_bits, &P.epsilon, sizeof(double));
    sdt2::prime(ca, (double*)calGetDeviceBuffer2Dr(ca, Q.h, 0), eps_bits, (cudaStream_t)calGetStream2D(ca));
}

/* host side of the fused step: queue the kernel, then exchange the h layers */
static void sciddicaT_fused_transition(struct CALModel2D* ca)
{
    if (sdt_use_split()) {
        sciddicaT_split_transition_timed(ca, nullptr);
        return;
    }
    sdt::Params p;
    p.z = (const double*)calGetDeviceBuffer2Dr(ca, Q.z, 0);
    p.h = (const double*)calGetDeviceBuffer2Dr(ca, Q.h, 0);
    p.h_next = (double*)calGetDeviceBuffer2Dr(ca, Q.h, 2);
    p.rows = ca->rows;
    p.cols = ca->columns;
    p.toroidal = ca->T == CAL_SPACE_TOROIDAL;
    p.eps = P.epsilon;
    p.r = P.r;
    memcpy(&p.eps_bits, &P.epsilon, sizeof(double));
    sdt::launch_step(p, (cudaStream_t)calGetStream2D(ca));
    calSwapSubstate2Dr(ca, Q.h);
}

/* init of the fused/split program: the reference init, then the split
 * step's priming, so that no recorded step ever contains the priming */
static void sciddicaT_simulation_init_fused(struct CALModel2D* sciddicaT)
{
    sciddicaT_simulation_init(sciddicaT);
    sciddicaT_split_invalidate();
    sciddicaT_split_prepare(sciddicaT);
}

/* ======================= driver entry points ============================ */

enum { SDT_MODE_PROCESSES = 0, SDT_MODE_FUSED = 1 };

/* how many device-loop runs had to fall back to a launch sequence per step */
static int g_fallbacks = 0;
static void cal_note_fallback() { g_fallbacks++; }
extern "C" int cal_sciddicaT_device_loop_fallbacks(void) { return g_fallbacks; }

/* Runs SCIDDICA-T for `steps` steps on (z0, h0) and returns the final z, h
 * and active list -- the same contract as the oracle's orc_sciddicaT.
 * mode 0 runs the reference program (device processes); mode 1 the fused
 * step (plain mode only).  graph != 0 replays the step as a CUDA graph.
 * *ms receives the device time of the step loop (CUDA events).  Returns 0
 * on success, else the CALError code. */
extern "C" int cal_sciddicaT_run(int rows, int cols, int toroidal, int ac, int steps, double p_r, double p_eps,
                                 const double* z0, const double* h0, double* z_out, double* h_out, long* n_active,
                                 int* cells_out, int mode, int graph, double* ms)
{
    calClearError();
    if (mode == SDT_MODE_FUSED && ac)
        return CAL_ERROR_INVALID_ARGUMENT;
    sciddicaT_split_invalidate();
    struct CALModel2D* ca = calCADef2D(rows, cols, CAL_VON_NEUMANN_NEIGHBORHOOD_2D,
                                       toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT,
                                       ac ? CAL_OPT_ACTIVE_CELLS : CAL_NO_OPT);
    if (!ca)
        return calGetLastError();
    struct CALRun2D* run = calRunDef2D(ca, 1, steps, CAL_UPDATE_IMPLICIT);
    P.epsilon = p_eps;
    P.r = p_r;
    P.active = ac;
    if (mode == SDT_MODE_PROCESSES) {
        calAddElementaryProcess2D(ca, sciddicaT_flows_computation);
        calAddElementaryProcess2D(ca, sciddicaT_width_update);
        if (ac)
            calAddElementaryProcess2D(ca, sciddicaT_remove_inactive_cells);
    }
    Q.z = calAddSubstate2Dr(ca);
    Q.h = calAddSubstate2Dr(ca);
    for (int q = 0; q < NUMBER_OF_OUTFLOWS; q++)
        Q.f[q] = calAddSubstate2Dr(ca);
    if (calGetLastError() != CAL_SUCCESS) {
        int e = calGetLastError();
        calRunFinalize2D(run);
        calFinalize2D(ca);
        return e;
    }
    const size_t bytes = sizeof(double) * (size_t)rows * cols;
    memcpy(Q.z->current, z0, bytes);
    memcpy(Q.z->next, z0, bytes);
    memcpy(Q.h->current, h0, bytes);
    memcpy(Q.h->next, h0, bytes);
    calMarkHostDirty2D(ca);

    calRunAddInitFunc2D(run, mode == SDT_MODE_FUSED ? sciddicaT_simulation_init_fused : sciddicaT_simulation_init);
    if (mode == SDT_MODE_FUSED)
        calRunAddGlobalTransitionFunc2D(run, sciddicaT_fused_transition);
    else
        calRunAddSteeringFunc2D(run, ac ? sciddicaT_steering_ac : sciddicaT_steering_plain);
    calRunSetGraph2D(run, graph ? CAL_TRUE : CAL_FALSE);

    /* calRun2D, with the step loop timed on the model's stream */
    cudaStream_t s = (cudaStream_t)calGetStream2D(ca);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    calRunInitSimulation2D(run);
    cudaEventRecord(e0, s);
    if (graph == 2) {
        /* the whole step loop as one device-driven graph launch, bounded by
         * the final step */
        calRunDeviceSteps2D(run, run->initial_step, run->final_step);
    } else if (graph == 3) {
        /* the same, as an open loop ended by the device stop condition */
        P.steps = steps;
        calRunAddDeviceStopConditionFunc2D(run, sciddicaT_device_stop);
        calRunDeviceSteps2D(run, run->initial_step, CAL_RUN_LOOP);
    } else {
        for (run->step = run->initial_step; run->step <= run->final_step; run->step++)
            if (!calRunCAStep2D(run))
                break;
    }
    cudaEventRecord(e1, s);
    calRunFinalizeSimulation2D(run);
    calSync2D(ca);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    if (ms)
        *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (graph >= 2 && !calRunDeviceLoopUsed2D(run) && calGetLastError() == CAL_SUCCESS)
        cal_note_fallback();

    if (z_out)
        memcpy(z_out, Q.z->current, bytes);
    if (h_out)
        memcpy(h_out, Q.h->current, bytes);
    if (n_active)
        *n_active = ac ? ca->A.size_current : 0;
    if (cells_out && ac)
        memcpy(cells_out, ca->A.cells, sizeof(int) * 2 * (size_t)ca->A.size_current);
    int err = calGetLastError();
    sdt2::release();
    calRunFinalize2D(run);
    calFinalize2D(ca);
    return err;
}

/* ======================= benchmark session ============================== */
/* A model created once and rerun many times from its initial state: the
 * benchmark times the step loop with the inputs already resident in HBM
 * (value) and, separately, host->device->host runs through the same API
 * (e2e). */

struct SdtSession {
    struct CALModel2D* ca;
    struct CALRun2D* run;
    int mode, ac;
    size_t bytes;
    double* snap[6][2]; /* device copies of z, h, f0..f3 (both layers) after init */
    CALbyte* snap_flags;
};

static struct CALSubstate2Dr* sdt_sub(int k) { return k == 0 ? Q.z : (k == 1 ? Q.h : Q.f[k - 2]); }

extern "C" void* cal_sciddicaT_open(int rows, int cols, int toroidal, int ac, double p_r, double p_eps,
                                    const double* z0, const double* h0, int mode)
{
    calClearError();
    if (mode == SDT_MODE_FUSED && ac)
        return nullptr;
    sciddicaT_split_invalidate();
    SdtSession* s = (SdtSession*)calloc(1, sizeof(SdtSession));
    s->mode = mode;
    s->ac = ac;
    s->bytes = sizeof(double) * (size_t)rows * cols;
    s->ca = calCADef2D(rows, cols, CAL_VON_NEUMANN_NEIGHBORHOOD_2D, toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT,
                       ac ? CAL_OPT_ACTIVE_CELLS : CAL_NO_OPT);
    if (!s->ca) {
        free(s);
        return nullptr;
    }
    s->run = calRunDef2D(s->ca, 1, CAL_RUN_LOOP, CAL_UPDATE_IMPLICIT);
    P.epsilon = p_eps;
    P.r = p_r;
    P.active = ac;
    if (mode == SDT_MODE_PROCESSES) {
        calAddElementaryProcess2D(s->ca, sciddicaT_flows_computation);
        calAddElementaryProcess2D(s->ca, sciddicaT_width_update);
        if (ac)
            calAddElementaryProcess2D(s->ca, sciddicaT_remove_inactive_cells);
        calRunAddSteeringFunc2D(s->run, ac ? sciddicaT_steering_ac : sciddicaT_steering_plain);
    } else {
        calRunAddGlobalTransitionFunc2D(s->run, sciddicaT_fused_transition);
    }
    Q.z = calAddSubstate2Dr(s->ca);
    Q.h = calAddSubstate2Dr(s->ca);
    for (int q = 0; q < NUMBER_OF_OUTFLOWS; q++)
        Q.f[q] = calAddSubstate2Dr(s->ca);
    memcpy(Q.z->current, z0, s->bytes);
    memcpy(Q.z->next, z0, s->bytes);
    memcpy(Q.h->current, h0, s->bytes);
    memcpy(Q.h->next, h0, s->bytes);
    calMarkHostDirty2D(s->ca);
    calRunAddInitFunc2D(s->run, mode == SDT_MODE_FUSED ? sciddicaT_simulation_init_fused : sciddicaT_simulation_init);
    calRunInitSimulation2D(s->run);
    cudaStream_t st = (cudaStream_t)calGetStream2D(s->ca);
    for (int k = 0; k < 6; k++)
        for (int l = 0; l < 2; l++) {
            cudaMalloc(&s->snap[k][l], s->bytes);
            cudaMemcpyAsync(s->snap[k][l], calGetDeviceBuffer2Dr(s->ca, sdt_sub(k), l), s->bytes,
                            cudaMemcpyDeviceToDevice, st);
        }
    if (ac) {
        CALbyte* flags;
        calGetDeviceActiveCells2D(s->ca, &flags, nullptr, nullptr);
        cudaMalloc(&s->snap_flags, (size_t)rows * cols);
        cudaMemcpyAsync(s->snap_flags, flags, (size_t)rows * cols, cudaMemcpyDeviceToDevice, st);
    }
    calFinish2D(s->ca);
    if (calGetLastError() != CAL_SUCCESS)
        return nullptr;
    return s;
}

/* back to the state right after init (device to device; queued) */
extern "C" int cal_sciddicaT_reset(void* handle)
{
    SdtSession* s = (SdtSession*)handle;
    sciddicaT_split_invalidate();
    cudaStream_t st = (cudaStream_t)calGetStream2D(s->ca);
    for (int k = 0; k < 6; k++)
        for (int l = 0; l < 2; l++)
            cudaMemcpyAsync(calGetDeviceBuffer2Dr(s->ca, sdt_sub(k), l == 0 ? 0 : 2), s->snap[k][l], s->bytes,
                            cudaMemcpyDeviceToDevice, st);
    if (s->ac) {
        CALbyte* flags;
        calGetDeviceActiveCells2D(s->ca, &flags, nullptr, nullptr);
        cudaMemcpyAsync(flags, s->snap_flags, (size_t)s->ca->rows * s->ca->columns, cudaMemcpyDeviceToDevice, st);
        calUpdateActiveCells2D(s->ca);
    }
    calMarkDeviceWritten2D(s->ca);
    return calGetLastError();
}

/* queue `steps` steps; graph != 0 replays a recorded step */
extern "C" int cal_sciddicaT_steps(void* handle, int steps, int graph)
{
    SdtSession* s = (SdtSession*)handle;
    if (s->mode == SDT_MODE_FUSED)
        sciddicaT_split_prepare(s->ca);
    if (graph == 2) {
        /* one device-driven graph launch for all the steps */
        calRunDeviceSteps2D(s->run, 1, steps);
        return calGetLastError();
    }
    calRunSetGraph2D(s->run, graph ? CAL_TRUE : CAL_FALSE);
    for (int k = 0; k < steps; k++)
        calRunCAStep2D(s->run);
    return calGetLastError();
}

/* new p_r, p_epsilon for the following runs of the session (a recorded
 * step, which bakes them into its launches, is dropped) */
extern "C" int cal_sciddicaT_set_params(void* handle, double p_r, double p_eps)
{
    SdtSession* s = (SdtSession*)handle;
    P.r = p_r;
    P.epsilon = p_eps;
    calRunSetGraph2D(s->run, CAL_FALSE);
    return calGetLastError();
}

extern "C" void* cal_sciddicaT_stream(void* handle) { return calGetStream2D(((SdtSession*)handle)->ca); }

/* host-buffer round trip through the API: load z and h into the host
 * mirrors (uploaded by the next device operation), run, read h back */
extern "C" int cal_sciddicaT_host_run(void* handle, const double* z_host, const double* h_host, int steps,
                                      double* h_out)
{
    SdtSession* s = (SdtSession*)handle;
    memcpy(Q.z->current, z_host, s->bytes);
    memcpy(Q.z->next, z_host, s->bytes);
    memcpy(Q.h->current, h_host, s->bytes);
    memcpy(Q.h->next, h_host, s->bytes);
    calMarkHostDirty2D(s->ca);
    sciddicaT_split_invalidate();
    cal_sciddicaT_steps(handle, steps, 0);
    calSyncSubstate2Dr(s->ca, Q.h);
    memcpy(h_out, Q.h->current, s->bytes);
    return calGetLastError();
}

/* device time of each of n steps' kernels, events around every launch:
 * split step -> ms_a[k] = K1 (outflows), ms_b[k] = K2 (update);
 * single fused kernel -> ms_a[k] = the kernel, ms_b[k] = 0 */
extern "C" int cal_sciddicaT_kernel_times(void* handle, int n, float* ms_a, float* ms_b)
{
    SdtSession* s = (SdtSession*)handle;
    cudaStream_t st = (cudaStream_t)calGetStream2D(s->ca);
    cudaEvent_t* ev = (cudaEvent_t*)malloc(sizeof(cudaEvent_t) * 3 * n);
    for (int k = 0; k < 3 * n; k++)
        cudaEventCreate(&ev[k]);
    const bool split = sdt_use_split();
    for (int k = 0; k < n; k++) {
        if (split) {
            sciddicaT_split_transition_timed(s->ca, ev + 3 * k);
        } else {
            cudaEventRecord(ev[3 * k], st);
            sciddicaT_fused_transition(s->ca);
            cudaEventRecord(ev[3 * k + 1], st);
            cudaEventRecord(ev[3 * k + 2], st);
        }
    }
    cudaStreamSynchronize(st);
    for (int k = 0; k < n; k++) {
        cudaEventElapsedTime(&ms_a[k], ev[3 * k], ev[3 * k + 1]);
        cudaEventElapsedTime(&ms_b[k], ev[3 * k + 1], ev[3 * k + 2]);
    }
    for (int k = 0; k < 3 * n; k++)
        cudaEventDestroy(ev[k]);
    free(ev);
    return calGetLastError();
}

/* number of wet cells the split step will process next (synchronises) */
extern "C" int cal_sciddicaT_wet_count(void* handle)
{
    SdtSession* s = (SdtSession*)handle;
    int c[6] = {-1, -1, -1, -1, 0, 0};
    if (sdt2::g_state.counts) {
        /* the model's stream does not synchronise with the legacy stream */
        cudaStreamSynchronize((cudaStream_t)calGetStream2D(s->ca));
        cudaMemcpy(c, sdt2::g_state.counts, sizeof(c), cudaMemcpyDeviceToHost);
    }
    return c[c[4] & 1];
}

extern "C" int cal_sciddicaT_read(void* handle, double* h_out)
{
    SdtSession* s = (SdtSession*)handle;
    calSyncSubstate2Dr(s->ca, Q.h);
    memcpy(h_out, Q.h->current, s->bytes);
    return calGetLastError();
}

extern "C" void cal_sciddicaT_close(void* handle)
{
    SdtSession* s = (SdtSession*)handle;
    if (!s)
        return;
    calFinish2D(s->ca);
    for (int k = 0; k < 6; k++)
        for (int l = 0; l < 2; l++)
            cudaFree(s->snap[k][l]);
    cudaFree(s->snap_flags);
    sdt2::release();
    calRunFinalize2D(s->run);
    calFinalize2D(s->ca);
    free(s);
}
