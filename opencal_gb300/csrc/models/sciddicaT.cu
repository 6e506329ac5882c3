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
#include "opencal/cal2DIO.h"
#include "opencal/cal2DRun.h"

#include <string>
#include <vector>

namespace cal {
void set_error(CALError code, const std::string& msg); /* the library's error state (calGetLastError) */
}

/* false (and the library's error state set) when a CUDA call failed */
static bool cal_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess)
        return true;
    cal::set_error(CAL_ERROR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

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
/* the body of the program's initialisation loop (sciddicaT_simulation_init,
 * sciddicaT.c:104-131) at one cell: the source's depth is removed from the
 * altitude, and with active cells on the source cells become active.  The
 * reference runs it as a host loop over calGet2Dr / calSet2Dr; here it is
 * a device process applied once, so the run needs no host pass over the
 * grid (same arithmetic, same active list after the update). */
CAL_ELEMENTARY_PROCESS_2D(sciddicaT_init_cell)(struct CALModel2D* sciddicaT, int i, int j)
{
    const CALreal h = calGet2Dr(sciddicaT, Q.h, i, j);
    if (h > 0.0) {
        const CALreal z = calGet2Dr(sciddicaT, Q.z, i, j);
        calSet2Dr(sciddicaT, Q.z, i, j, z - h);
        if (P.active)
            calAddActiveCell2D(sciddicaT, i, j);
    }
}

static void sciddicaT_simulation_init(struct CALModel2D* sciddicaT)
{
    calInitSubstate2Dr(sciddicaT, Q.f[0], 0);
    calInitSubstate2Dr(sciddicaT, Q.f[1], 0);
    calInitSubstate2Dr(sciddicaT, Q.f[2], 0);
    calInitSubstate2Dr(sciddicaT, Q.f[3], 0);
    calApplyElementaryProcess2D(sciddicaT, sciddicaT_init_cell);
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
/* the split step's update tile (compile-time; measured on the 2048 x 2048
 * bench run, ms per 4000 steps, persistent / eager loop, identical bits):
 * 16 x 16 (one cell per thread) 66.7 / 76.7, 16 x 32 66.6 / 80.2, 32 x 16
 * (two per thread) 69.5 / 81.6, 8 x 16 69.9 / 80.6, 32 x 8 70.0 / 100.3,
 * 64 x 8 70.8 / 81.4, 16 x 8 71.4 / 81.0; with four cells per thread,
 * 32 x 16 73.0, 64 x 16 76.5 */
#ifndef SDT2_TW
#define SDT2_TW 16
#endif
#ifndef SDT2_TH
#define SDT2_TH 16
#endif
namespace sdt2 {

constexpr int THREADS = 256;
constexpr int TW = SDT2_TW, TH = SDT2_TH; /* K2 tile: TH rows x TW columns, 4 cells per thread */

struct State {
    struct CALModel2D* ca = nullptr;
    double* f = nullptr;         /* 4 * n outflows, SoA */
    double* zh = nullptr;        /* z + h per cell (u of a neighbour), kept where K2 writes h */
    double* zeps = nullptr;      /* z + epsilon per cell (u[0] of the cell), from the priming */
    int* list[2] = {nullptr, nullptr}; /* a step's cells: c for a wet cell, ~c for one that dried */
    int* counts = nullptr;       /* [4] list parity, [6] step epoch; [C_TICKET] K2 block
                                    ticket; [C_ARRIVED], [C_ERROR] the persistent kernel's
                                    placement barrier counter and error flag */
    unsigned long long* ctl = nullptr; /* 64-bit counters, one per 128-byte line (W_*) */
    int* tflag = nullptr;        /* per K2 tile: epoch of the step that flagged it */
    int* tlist = nullptr;        /* flagged tiles of the current step */
    long long n = 0;
    int tiles_x = 0, tiles_y = 0;
    bool primed = false;
    /* the device's list parity and epoch as of the next eager step, when
     * hknown: kept by step() and dropped whenever launches the host does not
     * see may have run (a recorded step replayed, the persistent kernel, any
     * entry point's start) */
    int hpar = 0, hepoch = 1;
    bool hknown = false;
};

/* The lists alternate between two buffers; which one a step reads is the
 * list parity, and tiles are flagged with the step's epoch; the step's
 * flagged tiles are counted in ctl[W_TILES + 16 * parity] (K1 empties the
 * other one for the next step).  Two ways to know parity and epoch:
 *  - device words counts[4] and counts[6], flipped and advanced by the last
 *    K2 block of the step (a ticket): every step's launches are identical,
 *    so a step can be recorded once as a CUDA graph and replayed;
 *  - hpar >= 0: the host passes them (eager launches; the host tracks them
 *    from the device words it read once), so that no block reads them
 *    first and K2 ends without the fence and ticket atomic; block 0 of K2
 *    still writes the device words for a later recorded step. */
struct K1Params {
    const double* __restrict__ z;
    const double* __restrict__ h;
    const double* __restrict__ zh;   /* z + h (written by K2) */
    const double* __restrict__ zeps; /* z + eps */
    double* __restrict__ f;
    int* list0;
    int* list1;
    int* counts;
    unsigned long long* ctl;
    int* tflag;
    int* tlist;
    int rows, cols, toroidal, tiles_x;
    long long n;
    double eps, r;
    int hpar, hepoch; /* host-known parity and epoch; hpar < 0: read the device words */
};

struct K2Params {
    double* __restrict__ h;
    double* __restrict__ zh;
    const double* __restrict__ z;
    const double* __restrict__ f;
    int* list0;
    int* list1;
    int* counts;
    unsigned long long* ctl;
    const int* tflag;
    const int* tlist;
    int rows, cols, toroidal, tiles_x;
    long long n;
    long long eps_bits;
    int hpar, hepoch;
};

static __device__ __forceinline__ int tile_of(int i, int j, int tiles_x)
{
    return (i / TH) * tiles_x + (j / TW);
}

/* K1: 608 blocks of 256 threads.  Launch cost grows with the number of
 * blocks (measured on GB300: 4864 blocks of 64 threads cost ~2 us per
 * launch more than 608 blocks), so the wet cells' spread over every SM comes
 * from the mapping instead: chunks of 32 list entries go to consecutive
 * blocks (k1_outflows) */
constexpr int K1_THREADS = 256;
/* control words, each group on its own 128-byte line: the K2 ticket and the
 * persistent kernel's barrier counter are hit by every block and polled,
 * and must not share a line with the list and tile counters */
constexpr int NCOUNTS = 512;
constexpr int C_TICKET = 32, C_ARRIVED = 64, C_ERROR = 96;
/* the persistent kernel's placement census: a flag (own line) and blocks
 * per SM, for SM ids below MAX_SM */
constexpr int C_PLACE_BAD = 128, C_SMRANK = 256, MAX_SM = 256;
/* 64-bit counters (State::ctl), each on a 128-byte line of its own; the low
 * 32 bits count appended items, the high 32 bits a barrier's arrivals:
 *   W_TILES + 16 * parity   tiles flagged in a step (per-step launches)
 *   W_LIST + 16 * parity    entries of a step's list (per-step launches)
 *   W_PT + 16 * (s % 3)     step s of a persistent run: flagged tiles, then
 *                           the arrivals at the barrier that ends its K1 phase
 *   W_PL + 16 * (s % 3)     step s of a persistent run: entries of the next
 *                           list, then the arrivals at the barrier that ends
 *                           its K2 phase
 * so that the poll that releases a barrier returns the count the next phase
 * needs.  A persistent word is reused three steps later; block 0 clears it
 * one step before its use, when every block has finished polling it. */
constexpr int W_TILES = 0, W_LIST = 32, W_PT = 64, W_PL = 112, NCTL = 160;
static __host__ __device__ __forceinline__ int low32(unsigned long long v) { return (int)(unsigned)(v & 0xffffffffull); }
constexpr int K2_BLOCKS = 152 * 4;
static int g_k1_blocks = 152 * 4, g_k2_blocks = K2_BLOCKS; /* launch grids of K1 and K2 (tunable) */

/* Loads of data that other blocks write while the kernel runs.  In the
 * persistent kernel (CO = true) they are plain coherent loads through a
 * pointer passed through a register move, so that the compiler can neither
 * turn them into non-coherent loads (the parameters are const __restrict__)
 * nor is kept from batching them (inline-asm loads with a memory clobber,
 * __ldcg included, are issued one after another); the grid barrier between
 * the phases (a gpu-scope fence and acquire by one thread, then bar.sync)
 * orders them after every write of the previous phase.  The per-step
 * kernels use the ordinary paths (a kernel boundary orders them). */
template <typename T>
static __device__ __forceinline__ const T* launder(const T* p)
{
    const T* q;
    asm("mov.b64 %0, %1;" : "=l"(q) : "l"(p));
    return q;
}
template <bool CO, typename T>
static __device__ __forceinline__ T ldm(const T* p)
{
    return CO ? *launder(p) : *p;
}
template <bool CO>
static __device__ __forceinline__ double ldh(const double* p)
{
    return CO ? *launder(p) : __ldg(p);
}

/* flag tile t for this step's K2 and append it to the work-list once */
template <bool CO>
static __device__ __forceinline__ void flag_tile(int* tflag, int* tlist, unsigned long long* tcount, int t, int epoch)
{
    if (ldm<CO>(tflag + t) != epoch && atomicExch(tflag + t, epoch) != epoch)
        tlist[low32(atomicAdd(tcount, 1ull))] = t;
}

/* flag tile t for the lanes where `want` holds, once per distinct tile among
 * the lanes converged here: consecutive wet cells of the list mostly share
 * a tile, so the warp's leader for each tile does the (idempotent) flag
 * and the others skip its load and atomic */
template <bool CO>
static __device__ __forceinline__ void flag_tile_warp(bool want, int t, int* tflag, int* tlist,
                                                      unsigned long long* tcount, int epoch)
{
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, want ? t : -1);
    if (want && (threadIdx.x & 31) == __ffs(peers) - 1)
        flag_tile<CO>(tflag, tlist, tcount, t, epoch);
}

/* K1's work on the step's list (threads tid, tid + nthreads, ...): the
 * outflows of every wet cell (entry c >= 0) and the clearing of the outflows
 * of every cell that dried in the previous step (entry ~c) */
template <bool CO>
static __device__ __forceinline__ void k1_work(const K1Params& p, int par, int epoch, int nlist,
                                               unsigned long long* tcount, int tid, int nthreads)
{
    const int* list = par ? p.list1 : p.list0;
    for (int k = tid; k < nlist; k += nthreads) {
        const int e = ldm<CO>(list + k);
        if (e < 0) {
            const long long c = ~e;
#pragma unroll
            for (int q = 0; q < 4; q++)
                p.f[q * p.n + c] = 0.0;
            continue;
        }
        const int c = e;
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
                /* z + h of the neighbour, as K2 (or the priming) computed it
                 * from the same operands */
                u[q] = ldh<CO>(p.zh + (long long)a * p.cols + b);
            } else {
                u[q] = 0.0 + 0.0; /* an absent neighbour reads z = 0, h = 0 */
            }
        }
        double f[4];
        sdt::outflows_u0(ldh<CO>(p.h + c), __ldg(p.zeps + c), u[0], u[1], u[2], u[3], p.eps, p.r, f);
        bool any = false;
        const int own = tile_of(i, j, p.tiles_x);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            p.f[q * p.n + c] = f[q];
            if (__double_as_longlong(f[q]) != 0) {
                any = true;
                /* the receiver reads it; a receiver in this cell's own tile
                 * is covered by the flag of the own tile below */
                if (in[q]) {
                    const int t = tile_of(ni[q], nj[q], p.tiles_x);
                    if (t != own)
                        flag_tile<CO>(p.tflag, p.tlist, tcount, t, epoch);
                }
            }
        }
        flag_tile_warp<CO>(any, own, p.tflag, p.tlist, tcount, epoch);
    }
}

__global__ void __launch_bounds__(K1_THREADS) k1_outflows(const __grid_constant__ K1Params p)
{
    const bool host = p.hpar >= 0;
    const int par = host ? p.hpar : p.counts[4];
    const int epoch = host ? p.hepoch : p.counts[6];
    if (blockIdx.x == 0 && threadIdx.x < 2) {
        if (threadIdx.x == 0)
            p.ctl[W_LIST + 16 * (1 - par)] = 0; /* the list K2 will append to */
        else
            p.ctl[W_TILES + 16 * (1 - par)] = 0; /* next step's tile count (read last by the previous K2) */
    }
    /* list entries in chunks of 32 (one per warp); consecutive chunks on
     * consecutive blocks, which the hardware places on different SMs */
    const int tid = ((threadIdx.x >> 5) * (int)gridDim.x + blockIdx.x) * 32 + (threadIdx.x & 31);
    k1_work<false>(p, par, epoch, low32(p.ctl[W_LIST + 16 * par]), p.ctl + W_TILES + 16 * par, tid,
                   gridDim.x * blockDim.x);
}

/* append the lanes whose predicate holds to list/count (warp-aggregated);
 * a 64-bit counter counts in its low 32 bits */
static __device__ __forceinline__ int count_add(int* count, int v) { return atomicAdd(count, v); }
static __device__ __forceinline__ int count_add(unsigned long long* count, int v)
{
    return low32(atomicAdd(count, (unsigned long long)v));
}
template <typename C>
static __device__ __forceinline__ void warp_append(bool pred, int value, int* list, C* count)
{
    const unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0)
        return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0)
        base = count_add(count, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (pred)
        list[base + __popc(mask & ((1u << lane) - 1u))] = value;
}

/* Block-wide append of up to 4 items per thread to the next list, one
 * atomicAdd per block: item q as value[q] when want[q] (a wet cell) and as
 * ~value[q] when dried[q] (a cell whose outflows K1 must clear). */
static __device__ __forceinline__ void block_append4(const bool want[4], const bool dried[4], const int value[4],
                                                     int* list, unsigned long long* count)
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
    if (threadIdx.x == 0) {
        int tw = 0, td = 0;
        for (int w = 0; w < THREADS / 32; w++) {
            tw += s_warp[0][w];
            td += s_warp[1][w];
        }
        const int base = (tw + td) ? count_add(count, tw + td) : 0;
        s_base[0] = base;      /* wet entries first, */
        s_base[1] = base + tw; /* then the dried ones */
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
            list[bd + __popc(md[q] & below)] = ~value[q];
        bw += __popc(mw[q]);
        bd += __popc(md[q]);
    }
}

/* one flagged tile: h += inflows - outflows in place, then the wet test */
template <bool CO>
static __device__ __forceinline__ void k2_tile(const K2Params& p, int tile, int* list, unsigned long long* count)
{
    const int ty = tile / p.tiles_x, tx = tile - ty * p.tiles_x;
    /* CPT consecutive cells of a row per thread: 4 when the tile has 4
     * cells per thread or more, else 2 or 1 (32 x 16: 2, every thread busy,
     * half the serial FP64 chain per thread) */
    constexpr int CPT = (TW * TH >= 4 * THREADS) ? 4 : ((TW * TH >= 2 * THREADS) ? 2 : 1);
    static_assert((TW / CPT) * TH <= THREADS && TW % CPT == 0, "one group of CPT cells per thread at most");
    const int r = threadIdx.x / (TW / CPT);         /* the tile's row; r >= TH: no cells */
    const int j4 = (threadIdx.x % (TW / CPT)) * CPT; /* 0, CPT, ..., TW - CPT */
    const bool has = r < TH;
    const int i = ty * TH + r;
    const int jb = tx * TW + j4;
    const long long c0 = (long long)i * p.cols + jb;
    double hv[4] = {0.0, 0.0, 0.0, 0.0};
    bool cell[4] = {false, false, false, false};
    const bool full = CPT > 1 && has && i < p.rows && jb + CPT - 1 < p.cols && (p.cols & 1) == 0;
    if (full) {
        /* c0 is a multiple of 2 (jb and cols even): 16-byte loads */
        const double2 a = ldm<CO>(reinterpret_cast<const double2*>(p.h + c0));
        hv[0] = a.x;
        hv[1] = a.y;
        if (CPT == 4) {
            const double2 b = ldm<CO>(reinterpret_cast<const double2*>(p.h + c0 + 2));
            hv[2] = b.x;
            hv[3] = b.y;
        }
#pragma unroll
        for (int q = 0; q < CPT; q++)
            cell[q] = true;
    } else {
#pragma unroll
        for (int q = 0; q < CPT; q++) {
            cell[q] = has && i < p.rows && jb + q < p.cols;
            if (cell[q])
                hv[q] = ldm<CO>(p.h + c0 + q);
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
            const double o0 = ldm<CO>(p.f + c), o1 = ldm<CO>(p.f + p.n + c), o2 = ldm<CO>(p.f + 2 * p.n + c),
                         o3 = ldm<CO>(p.f + 3 * p.n + c);
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
                in1 = ldm<CO>(p.f + 3 * p.n + (long long)a * p.cols + j);
            if ((unsigned)b < (unsigned)p.cols)
                in2 = ldm<CO>(p.f + 2 * p.n + (long long)i * p.cols + b);
            if ((unsigned)d < (unsigned)p.cols)
                in3 = ldm<CO>(p.f + 1 * p.n + (long long)i * p.cols + d);
            if ((unsigned)e < (unsigned)p.rows)
                in4 = ldm<CO>(p.f + (long long)e * p.cols + j);
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
                p.zh[c] = __ldg(p.z + c) + x; /* the u K1 will read next step */
            }
        }
        const bool wb = cell[q] && sdt::is_wet(hv[q], p.eps_bits);
        want[q] = cell[q] && sdt::is_wet(hn, p.eps_bits);
        dried[q] = wb && !want[q];
        value[q] = (int)c;
    }
    block_append4(want, dried, value, list, count);
}

/* K2's work for blocks block, block + nblocks, ...: the flagged tiles, then
 * the current wet list in chunks of THREADS entries (carrying over the wet
 * cells of unflagged tiles, whose h did not change) */
template <bool CO>
static __device__ __forceinline__ void k2_work(const K2Params& p, int par, int epoch, int ntiles, int nlist,
                                               unsigned long long* count, int block, int nblocks)
{
    const int* cur = par ? p.list1 : p.list0;
    int* list = par ? p.list0 : p.list1; /* next step's list */
    const int items = ntiles + (nlist + THREADS - 1) / THREADS;
    for (int item = block; item < items; item += nblocks) {
        if (item < ntiles) {
            k2_tile<CO>(p, ldm<CO>(p.tlist + item), list, count);
            __syncthreads(); /* block_append4's shared words are reused */
        } else {
            const int k = (item - ntiles) * THREADS + threadIdx.x;
            bool carry = false;
            int c = 0;
            if (k < nlist) {
                c = ldm<CO>(cur + k);
                if (c >= 0) { /* a dried entry's outflows were cleared this step */
                    const int i = c / p.cols, j = c - i * p.cols;
                    carry = ldm<CO>(p.tflag + tile_of(i, j, p.tiles_x)) != epoch;
                }
            }
            /* one atomic on the step's counter per block, not per warp:
             * every block of the phase appends to that one word */
            const bool want[4] = {carry, false, false, false};
            const bool none[4] = {false, false, false, false};
            const int value[4] = {c, 0, 0, 0};
            block_append4(want, none, value, list, count);
            __syncthreads(); /* block_append4's shared words are reused */
        }
    }
}

__global__ void __launch_bounds__(THREADS) k2_update(const __grid_constant__ K2Params p)
{
    const bool host = p.hpar >= 0;
    const int par = host ? p.hpar : p.counts[4];
    const int epoch = host ? p.hepoch : p.counts[6];
    k2_work<false>(p, par, epoch, low32(p.ctl[W_TILES + 16 * par]), low32(p.ctl[W_LIST + 16 * par]),
                   p.ctl + W_LIST + 16 * (1 - par), blockIdx.x, gridDim.x);
    if (host) {
        /* nobody reads the device words during this launch */
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            p.counts[4] = 1 - par;
            p.counts[6] = epoch + 1;
        }
    } else if (threadIdx.x == 0) {
        /* every block read parity, epoch and counts at its start; the last
         * one to finish advances them for the next step (no block waits for
         * another) */
        __threadfence();
        if (atomicAdd(reinterpret_cast<unsigned*>(p.counts + C_TICKET), 1u) == gridDim.x - 1) {
            p.counts[4] = 1 - par;
            p.counts[C_TICKET] = 0;
            p.counts[6] = epoch + 1;
        }
    }
}

/* ---- persistent form: every step of a run in one cooperative launch ----
 * The two phases of each step (K1's and K2's work) are separated by a grid
 * barrier on the 64-bit word that counts what the phase appended (packed
 * barrier below), so that the poll that ends the wait also returns the count
 * the next phase needs.  counts[C_ARRIVED] is the arrival counter of the
 * one-off barrier of the placement census (zeroed before the launch),
 * counts[C_ERROR] the error flag.  Only one thread per block touches the
 * shared words: it arrives, waits, and hands the count to its block through
 * shared memory, so that no L2 line is read by every thread of the grid. */
constexpr unsigned BARRIER_SPIN_LIMIT = 1u << 22;
/* pause between two polls of a barrier word: fewer polls leave the word's
 * L2 slice to the arrivals.  2048^2 x 4000 steps per run (same box, two
 * runs each): 32 ns 60.37 ms, 96 ns 59.70, 192 ns 59.46, 320 ns 60.19 */
constexpr unsigned BARRIER_POLL_NS = 192;

static __device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

/* An arrival: an atomic add with release semantics at GPU scope.  Issued by
 * thread 0 after the block barrier, it orders every write the block made
 * before that barrier ahead of the arrival (the block barrier orders the
 * other threads' writes before thread 0's release; release is cumulative),
 * and the acquire poll of a waiting block orders its later reads after it;
 * no separate fence.sc on either side (measured on an empty 608-block grid:
 * 5.2-5.5 us per barrier against 5.6-5.8 us with a fence.sc before a
 * relaxed add and after the poll). */
static __device__ __forceinline__ void red_release_gpu(unsigned* p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

static __device__ __forceinline__ void red_release_gpu(unsigned long long* p, unsigned long long v)
{
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

/* Grid barrier for a cooperative launch (all blocks resident).  Round r
 * (1, 2, ...) is complete when the monotonic arrival counter counts[C_ARRIVED]
 * reaches r * nblocks.  Every wait is bounded: after BARRIER_SPIN_LIMIT
 * polls the error flag is set and the block returns false, and so does
 * every block that finds the flag set.  After the wait, thread 0 reads *r0
 * and *r1 into out[0..1] for the whole block. */
static __device__ __forceinline__ bool grid_barrier(int* counts, unsigned nblocks, unsigned& round, const int* r0,
                                                    const int* r1, int* out)
{
    __shared__ int s_ok;
    __syncthreads();
    round++;
    if (threadIdx.x == 0) {
        unsigned* arrived = reinterpret_cast<unsigned*>(counts + C_ARRIVED);
        const unsigned target = round * nblocks;
        int ok = 1;
        red_release_gpu(arrived, 1u);
        unsigned polls = 0;
        while ((int)(ld_acquire_gpu(arrived) - target) < 0) {
            if (++polls > BARRIER_SPIN_LIMIT) {
                atomicExch(counts + C_ERROR, 1);
                ok = 0;
                break;
            }
            __nanosleep(BARRIER_POLL_NS);
        }
        if (ok && __ldcg(counts + C_ERROR) != 0)
            ok = 0;
        out[0] = __ldcg(r0);
        out[1] = __ldcg(r1);
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

/* The order in which a persistent kernel deals work to its blocks:
 * v = (rank of the block on its SM) * SMs + SM, so that consecutive work
 * items go to different SMs first (a cooperative launch places its first
 * blocks several to an SM).  v is a permutation of the blocks when every
 * block finds its SM id below nsm and its rank below nb / nsm (nb distinct
 * pairs in nb places); if one does not, every block keeps its launch index.
 * Needs counts[C_PLACE_BAD] and counts[C_SMRANK ...] zeroed before the
 * launch; one grid barrier.  Returns -1 when that barrier gave up. */
static __device__ int placement_order(int* counts, unsigned nb, int nsm, unsigned& round, int* s_tmp)
{
    __shared__ int s_v;
    if (threadIdx.x == 0) {
        unsigned smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        int v = -1;
        if (nsm > 0 && smid < (unsigned)nsm && smid < (unsigned)MAX_SM && nb % (unsigned)nsm == 0) {
            const int rank = atomicAdd(counts + C_SMRANK + smid, 1);
            if (rank < (int)(nb / (unsigned)nsm))
                v = rank * nsm + (int)smid;
        }
        if (v < 0)
            atomicExch(counts + C_PLACE_BAD, 1);
        s_v = v;
    }
    if (!grid_barrier(counts, nb, round, counts + C_PLACE_BAD, counts + C_PLACE_BAD, s_tmp))
        return -1;
    const int vb = s_tmp[0] ? (int)blockIdx.x : s_v;
    __syncthreads(); /* s_tmp is free again */
    return vb;
}

static __device__ __forceinline__ unsigned long long ld_acquire_gpu_u64(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

/* Grid barrier on a counter word (W_PT / W_PL): every block adds one
 * arrival to its high 32 bits after the phase's appends, which went to its
 * low 32 bits; the barrier is complete when the arrivals reach nblocks, and
 * the value that shows it carries the phase's final count (the appends of
 * every block precede that block's arrival in the word's order), which
 * thread 0 hands to the block in *out.  Bounded like grid_barrier: after
 * BARRIER_SPIN_LIMIT polls the error flag is set and false returned; a
 * block that gave up stops arriving, so the others give up at their next
 * barrier. */
static __device__ __forceinline__ bool packed_barrier(unsigned long long* word, unsigned nblocks, int* counts, int* out)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        red_release_gpu(word, 1ull << 32);
        unsigned polls = 0;
        unsigned long long v;
        while ((unsigned)((v = ld_acquire_gpu_u64(word)) >> 32) < nblocks) {
            if (++polls > BARRIER_SPIN_LIMIT) {
                atomicExch(counts + C_ERROR, 1);
                ok = 0;
                break;
            }
            __nanosleep(BARRIER_POLL_NS);
        }
        *out = low32(v);
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

#ifndef SDT2_PERSIST_MINB
#define SDT2_PERSIST_MINB 4 /* resident blocks per SM (5 measured slower: 78.4 against 72.8 ms per run) */
#endif
__global__ void __launch_bounds__(THREADS, SDT2_PERSIST_MINB) k_persist(const __grid_constant__ K1Params a,
                                                     const __grid_constant__ K2Params b, int nsteps, int nsm)
{
    __shared__ int s_cnt[2];
    __shared__ int s_state[3];
    const unsigned nb = gridDim.x;
    unsigned round = 0;
    const int vb = placement_order(a.counts, nb, nsm, round, s_cnt);
    if (vb < 0)
        return;
    if (threadIdx.x == 0) {
        s_state[0] = __ldcg(a.counts + 4);
        s_state[1] = __ldcg(a.counts + 6);
        s_state[2] = low32(__ldcg(a.ctl + W_LIST + 16 * s_state[0]));
    }
    __syncthreads();
    int par = s_state[0];
    int epoch = s_state[1];
    int nlist = s_state[2]; /* entries of the current step's list */
    /* K1's list entries in chunks of 32 (one per warp), consecutive chunks
     * on consecutive blocks in the order v, so that the wet cells' FP64 work
     * spreads over every SM whatever their number */
    const int tid = ((threadIdx.x >> 5) * (int)nb + vb) * 32 + (threadIdx.x & 31);
    for (int s = 0; s < nsteps; s++) {
        const int w = 16 * (s % 3);
        unsigned long long* tword = a.ctl + W_PT + w;
        unsigned long long* lword = a.ctl + W_PL + w;
        if (blockIdx.x == 0 && threadIdx.x < 2) {
            /* the words of step s + 1, last polled in step s - 2 */
            const int wn = 16 * ((s + 1) % 3);
            a.ctl[(threadIdx.x ? W_PL : W_PT) + wn] = 0;
        }
        k1_work<true>(a, par, epoch, nlist, tword, tid, nb * THREADS);
        /* then: the flagged tiles of this step */
        if (!packed_barrier(tword, nb, a.counts, s_cnt))
            return;
        k2_work<true>(b, par, epoch, s_cnt[0], nlist, lword, vb, nb);
        par = 1 - par;
        epoch++;
        /* then: the entries of the next step's list */
        if (!packed_barrier(lword, nb, a.counts, s_cnt + 1))
            return;
        nlist = s_cnt[1];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        /* the state the per-step kernels expect */
        a.counts[4] = par;
        a.counts[C_TICKET] = 0;
        a.counts[6] = epoch;
        a.ctl[W_LIST + 16 * par] = (unsigned long long)(unsigned)nlist;
        a.ctl[W_TILES] = 0;
        a.ctl[W_TILES + 16] = 0;
    }
}

/* -0 -> +0 in h, z + h and z + eps of every cell, and the first wet list
 * (its counter must be 0) */
__global__ void __launch_bounds__(THREADS) k_prime(double* h, const double* __restrict__ z, double* zh, double* zeps,
                                                  double eps, long long n, long long eps_bits, int* list,
                                                  unsigned long long* count, int* counts)
{
    if (blockIdx.x == 0 && threadIdx.x == 0)
        counts[6] = 1; /* first epoch (tile stamps start at 0) */
    for (long long c0 = (long long)blockIdx.x * blockDim.x; c0 < n; c0 += (long long)gridDim.x * blockDim.x) {
        const long long c = c0 + threadIdx.x;
        bool wet = false;
        if (c < n) {
            double hv = h[c];
            if (__double_as_longlong(hv) == (long long)0x8000000000000000ULL) {
                hv = 0.0;
                h[c] = 0.0;
            }
            const double zv = z[c];
            zh[c] = zv + hv;
            zeps[c] = zv + eps;
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
    cudaFree(s.zh);
    cudaFree(s.zeps);
    for (int k = 0; k < 2; k++)
        cudaFree(s.list[k]);
    cudaFree(s.counts);
    cudaFree(s.ctl);
    cudaFree(s.tflag);
    cudaFree(s.tlist);
    s = State();
}

/* (re)allocate for `ca` and prime from the current h and z */
static bool prime(struct CALModel2D* ca, double* h, const double* z, double eps, long long eps_bits, cudaStream_t st)
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
                  cudaMalloc(&s.zh, n * sizeof(double)) == cudaSuccess &&
                  cudaMalloc(&s.zeps, n * sizeof(double)) == cudaSuccess &&
                  cudaMalloc(&s.counts, NCOUNTS * sizeof(int)) == cudaSuccess &&
                  cudaMalloc(&s.ctl, NCTL * sizeof(unsigned long long)) == cudaSuccess &&
                  cudaMalloc(&s.tflag, sizeof(int) * s.tiles_x * s.tiles_y) == cudaSuccess &&
                  cudaMalloc(&s.tlist, sizeof(int) * s.tiles_x * s.tiles_y) == cudaSuccess;
        for (int k = 0; k < 2 && ok; k++)
            ok = cudaMalloc(&s.list[k], n * sizeof(int)) == cudaSuccess;
        if (!ok) {
            release();
            return false;
        }
    }
    cudaMemsetAsync(s.f, 0, 4 * n * sizeof(double), st);
    cudaMemsetAsync(s.counts, 0, NCOUNTS * sizeof(int), st); /* parity 0, tickets 0 */
    cudaMemsetAsync(s.ctl, 0, NCTL * sizeof(unsigned long long), st); /* empty lists, no flagged tile */
    cudaMemsetAsync(s.tflag, 0, sizeof(int) * s.tiles_x * s.tiles_y, st);
    int blocks = (int)((n + THREADS - 1) / THREADS);
    if (blocks > 152 * 16)
        blocks = 152 * 16;
    k_prime<<<blocks, THREADS, 0, st>>>(h, z, s.zh, s.zeps, eps, n, eps_bits, s.list[0], s.ctl + W_LIST, s.counts);
    s.primed = true;
    s.hpar = 0; /* what k_prime leaves: parity 0, epoch 1 */
    s.hepoch = 1;
    s.hknown = true;
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
    a.zh = s.zh;
    a.zeps = s.zeps;
    a.f = s.f;
    a.list0 = s.list[0];
    a.list1 = s.list[1];
    a.counts = s.counts;
    a.ctl = s.ctl;
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
    b.zh = s.zh;
    b.z = z;
    b.f = s.f;
    b.list0 = s.list[0];
    b.list1 = s.list[1];
    b.counts = s.counts;
    b.ctl = s.ctl;
    b.tflag = s.tflag;
    b.tlist = s.tlist;
    b.rows = ca->rows;
    b.cols = ca->columns;
    b.toroidal = a.toroidal;
    b.tiles_x = s.tiles_x;
    b.n = s.n;
    b.eps_bits = eps_bits;
    /* eager launches carry parity and epoch; a step being recorded reads the
     * device words (its replays must not depend on the host) */
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess)
        cs = cudaStreamCaptureStatusActive;
    a.hpar = b.hpar = -1;
    a.hepoch = b.hepoch = 0;
    if (cs == cudaStreamCaptureStatusNone) {
        if (!s.hknown) {
            int w[8];
            if (cudaMemcpyAsync(w, s.counts, sizeof(w), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                cudaStreamSynchronize(st) == cudaSuccess) {
                s.hpar = w[4];
                s.hepoch = w[6];
                s.hknown = true;
            }
        }
        if (s.hknown) {
            a.hpar = b.hpar = s.hpar;
            a.hepoch = b.hepoch = s.hepoch;
            s.hpar = 1 - s.hpar;
            s.hepoch++;
        }
    } else {
        s.hknown = false;
    }
    if (ev)
        cudaEventRecord(ev[0], st);
    k1_outflows<<<g_k1_blocks, K1_THREADS, 0, st>>>(a);
    if (ev)
        cudaEventRecord(ev[1], st);
    k2_update<<<g_k2_blocks, THREADS, 0, st>>>(b);
    if (ev)
        cudaEventRecord(ev[2], st);
    return cudaGetLastError() == cudaSuccess;
}

/* `nsteps` steps in one cooperative launch of k_persist (one resident grid:
 * SMs x resident blocks per SM); false when the launch is refused or a
 * CUDA error is pending.  A barrier that gave up sets counts[C_ERROR], which
 * persist_failed() reports. */
static bool persist(struct CALModel2D* ca, const double* z, double* h, double eps, double r, long long eps_bits,
                    int nsteps, cudaStream_t st)
{
    State& s = g_state;
    s.hknown = false; /* the kernel advances parity and epoch on the device */
    static int grid = 0, sms_of_device = 0;
    if (!grid) {
        int per_sm = 0, dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persist, THREADS, 0);
#ifdef SDT2_PERSIST_PER_SM /* compile-time cap (2 or 3 per SM measured slower than 4) */
        if (per_sm > SDT2_PERSIST_PER_SM)
            per_sm = SDT2_PERSIST_PER_SM;
#endif
        grid = sms * per_sm;
        sms_of_device = sms;
        if (grid <= 0)
            return false;
    }
    K1Params a;
    K2Params b;
    a.z = z;
    a.h = h;
    a.zh = s.zh;
    a.zeps = s.zeps;
    a.f = s.f;
    a.list0 = b.list0 = s.list[0];
    a.list1 = b.list1 = s.list[1];
    a.counts = b.counts = s.counts;
    a.ctl = b.ctl = s.ctl;
    a.tflag = s.tflag;
    b.tflag = s.tflag;
    a.tlist = s.tlist;
    b.tlist = s.tlist;
    a.rows = b.rows = ca->rows;
    a.cols = b.cols = ca->columns;
    a.toroidal = b.toroidal = ca->T == CAL_SPACE_TOROIDAL;
    a.tiles_x = b.tiles_x = s.tiles_x;
    a.n = b.n = s.n;
    a.eps = eps;
    a.r = r;
    b.h = h;
    b.zh = s.zh;
    b.z = z;
    b.f = s.f;
    b.eps_bits = eps_bits;
    a.hpar = b.hpar = -1;
    a.hepoch = b.hepoch = 0;
    cudaMemsetAsync(s.counts + C_ARRIVED, 0, sizeof(int), st); /* placement barrier counter */
    cudaMemsetAsync(s.counts + C_ERROR, 0, sizeof(int), st);   /* error flag */
    cudaMemsetAsync(s.counts + C_PLACE_BAD, 0, (NCOUNTS - C_PLACE_BAD) * sizeof(int), st); /* placement census */
    cudaMemsetAsync(s.ctl + W_PT, 0, (NCTL - W_PT) * sizeof(unsigned long long), st); /* the steps' counters */
    int nsm = sms_of_device;
    void* args[] = {&a, &b, &nsteps, &nsm};
    return cudaLaunchCooperativeKernel((const void*)k_persist, dim3(grid), dim3(THREADS), args, 0, st) ==
           cudaSuccess;
}

/* Trace of one step of a plain run on a flat grid, launched after K2 (one
 * block): the mass that left the grid in step t (the step's outflows of
 * border cells towards absent neighbours: f[0] north of row 0, f[3] south of
 * the last row, f[1] west of column 0, f[2] east of the last column; K2 does
 * not change f), the step's wet-cell count (the entries c >= 0 of its list;
 * K2 has advanced the parity word, so the step's list is the other one),
 * and whether a cell of the two-cell edge band holds h != 0 after the step
 * (atomicMin of t + 1 into *edge).  Needs rows, cols >= 5. */
__global__ void __launch_bounds__(THREADS) k_trace(const double* __restrict__ f, const double* __restrict__ h,
                                                  const int* __restrict__ counts,
                                                  const unsigned long long* __restrict__ ctl, const int* list0,
                                                  const int* list1, int rows, int cols, long long n, int t,
                                                  double* outflux, int* wet, int* edge)
{
    __shared__ double s_part[THREADS / 32];
    __shared__ int s_any;
    __shared__ int s_wet;
    if (threadIdx.x == 0) {
        s_any = 0;
        s_wet = 0;
    }
    __syncthreads();
    {
        const int par = 1 - counts[4];
        const int* list = par ? list1 : list0;
        const int nlist = low32(ctl[W_LIST + 16 * par]);
        int mine = 0;
        for (int k = threadIdx.x; k < nlist; k += THREADS)
            mine += list[k] >= 0;
        atomicAdd(&s_wet, mine);
    }
    double s = 0.0;
    for (int j = threadIdx.x; j < cols; j += THREADS)
        s += f[j];
    for (int j = threadIdx.x; j < cols; j += THREADS)
        s += f[3 * n + (long long)(rows - 1) * cols + j];
    for (int i = threadIdx.x; i < rows; i += THREADS)
        s += f[n + (long long)i * cols];
    for (int i = threadIdx.x; i < rows; i += THREADS)
        s += f[2 * n + (long long)i * cols + cols - 1];
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0)
        s_part[threadIdx.x >> 5] = s;
    bool any = false;
    const int ring = 4 * cols + 4 * (rows - 4);
    for (int k = threadIdx.x; k < ring; k += THREADS) {
        int i, j;
        if (k < 4 * cols) {
            const int r = k / cols; /* rows 0, 1, rows - 2, rows - 1 */
            i = r < 2 ? r : rows - 4 + r;
            j = k - r * cols;
        } else {
            const int q = k - 4 * cols, c = q & 3; /* columns 0, 1, cols - 2, cols - 1 */
            i = 2 + q / 4;
            j = c < 2 ? c : cols - 4 + c;
        }
        any |= h[(long long)i * cols + j] != 0.0;
    }
    if (any)
        s_any = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < THREADS / 32; w++)
            tot += s_part[w];
        outflux[t] = tot;
        wet[t] = s_wet;
        if (s_any)
            atomicMin(edge, t + 1);
    }
}

/* did the last persistent run give up at a barrier?  (synchronises) */
static int persist_failed(cudaStream_t st)
{
    int flag = 0;
    if (!g_state.counts)
        return 0;
    cudaStreamSynchronize(st);
    cudaMemcpy(&flag, g_state.counts + C_ERROR, sizeof(int), cudaMemcpyDeviceToHost);
    return flag;
}

} // namespace sdt2

/* ======================= 2c. the split step with active cells ===========
 * OpenCAL's active-cells program (flows, width update and removal of dry
 * cells, an update after each, then the steering:
 * OpenCAL/examples/cal_sciddicaT-activecells-glut/source/sciddicaT.c:20-146)
 * as two kernels per step, with the same result bit for bit:
 *  - after a step's steering every active cell has zero outflows and
 *    h > epsilon (the removal took the others out); after the
 *    initialisation every cell with h > 0 is active and all outflows are 0.
 *    So the next flows process overwrites all four outflows of every active
 *    cell that is wet and leaves the dry ones (after the initialisation
 *    only) at 0: the steering never needs to run;
 *  - a removed cell keeps its outflows (the steering zeroes active cells
 *    only), and the width update of its neighbours, and its own if it is
 *    activated again, read those stale values: one outflow array that keeps
 *    them reproduces that;
 *  - the active set is an epoch mark per cell: a cell is active in the step
 *    whose epoch its mark holds.
 *   K1 (flows): over the active list; a wet cell computes its outflows and
 *      activates every neighbour whose flow was not eliminated (the mark set
 *      by an atomic exchange; a newly marked cell is appended after the
 *      list, so that K1 does not process it).
 *   K2 (width update and removal): over the extended list; h receives the
 *      four inflow-minus-outflow terms in the reference's order (an absent
 *      neighbour of a flat grid gives 0), then cells with h > epsilon are
 *      marked for the next step and appended to the next list; the others
 *      drop out.
 * The list order is not the reference's row-major rebuild; no value depends
 * on it, and the active set is returned in row-major order. */
namespace sdtac {

constexpr int THREADS = 256, BLOCKS = 152 * 4;
/* counts[0..1] list lengths by parity, [4] parity, [6] epoch, [8 + parity]
 * cells activated by the step's flows, [32] K2 block ticket (own line); the
 * persistent kernel's barrier and placement words at sdt2's offsets */
constexpr int NCOUNTS = sdt2::NCOUNTS, C_PAR = 4, C_EPOCH = 6, C_EXT = 8, C_TICKET = sdt2::C_TICKET;

struct State {
    struct CALModel2D* ca = nullptr;
    double* f = nullptr; /* 4 * n outflows, SoA */
    int* mark = nullptr; /* epoch of the step in which the cell is (or was last) active */
    int* list[2] = {nullptr, nullptr};
    int* counts = nullptr;
    long long n = 0;
    bool primed = false;
};
static State g_state;

struct Params {
    const double* __restrict__ z;
    double* h;
    double* f;
    int* mark;
    int* list0;
    int* list1;
    int* counts;
    int rows, cols, toroidal;
    long long n;
    double eps, r;
    long long eps_bits;
};

/* neighbour q (von Neumann order: north, west, east, south) of (i, j);
 * false outside a flat grid */
static __device__ __forceinline__ bool nbr(const Params& p, int i, int j, int q, int& a, int& b)
{
    a = q == 0 ? i - 1 : (q == 3 ? i + 1 : i);
    b = q == 1 ? j - 1 : (q == 2 ? j + 1 : j);
    if (p.toroidal) {
        a = a < 0 ? a + p.rows : (a >= p.rows ? a - p.rows : a);
        b = b < 0 ? b + p.cols : (b >= p.cols ? b - p.cols : b);
        return true;
    }
    return (unsigned)a < (unsigned)p.rows && (unsigned)b < (unsigned)p.cols;
}

/* append the lanes whose predicate holds (warp-aggregated; every lane of
 * the warp calls it) */
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

/* The flows process over the na entries of the active list, in chunks of
 * 32 entries (one per warp): chunks g0, g0 + gs, ... */
static __device__ __forceinline__ void flows_work(const Params& p, int par, int epoch, int na, int g0, int gs)
{
    int* list = par ? p.list1 : p.list0;
    const int lane = threadIdx.x & 31;
    for (int g = g0; g * 32 < na; g += gs) {
        const int k = g * 32 + lane;
        if (k >= na)
            continue;
        const int c = list[k];
        const double hc = p.h[c];
        if (!sdt::is_wet(hc, p.eps_bits)) /* the reference returns at h <= epsilon */
            continue;
        const int i = c / p.cols, j = c - i * p.cols;
        double u[4];
        int nc[4];
        bool in[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int a, b;
            in[q] = nbr(p, i, j, q, a, b);
            nc[q] = a * p.cols + b;
            u[q] = in[q] ? __ldg(p.z + nc[q]) + p.h[nc[q]] : 0.0 + 0.0;
        }
        double f[4];
        unsigned elim;
        sdt::outflows(hc, __ldg(p.z + c), u[0], u[1], u[2], u[3], p.eps, p.r, f, &elim);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            p.f[q * p.n + c] = f[q];
            /* calAddActiveCellX2D for every neighbour whose flow is kept */
            if (!(elim & (2u << q)) && in[q] && p.mark[nc[q]] != epoch &&
                atomicExch(p.mark + nc[q], epoch) != epoch)
                list[na + atomicAdd(p.counts + C_EXT + par, 1)] = nc[q];
        }
    }
}

/* The width update and the removal over the n2 entries of the extended
 * list (chunks g0, g0 + gs, ...); survivors go to the next list */
static __device__ __forceinline__ void update_work(const Params& p, int par, int epoch, int n2, int g0, int gs)
{
    const int* list = par ? p.list1 : p.list0;
    int* next = par ? p.list0 : p.list1;
    int* ncount = p.counts + (1 - par);
    const int lane = threadIdx.x & 31;
    for (int g = g0; g * 32 < n2; g += gs) {
        const int k = g * 32 + lane;
        bool keep = false;
        int c = 0;
        if (k < n2) {
            c = list[k];
            const int i = c / p.cols, j = c - i * p.cols;
            double hn = p.h[c];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                /* inflow from neighbour n = q + 1 is its outflow f[3 - q] */
                int a, b;
                const double fin = nbr(p, i, j, q, a, b) ? p.f[(3 - q) * p.n + (long long)a * p.cols + b] : 0.0;
                hn += fin - p.f[q * p.n + c];
            }
            p.h[c] = hn;
            keep = sdt::is_wet(hn, p.eps_bits); /* the removal: h <= epsilon drops out */
            if (keep)
                p.mark[c] = epoch + 1;
        }
        warp_append(keep, c, next, ncount);
    }
}

/* chunks of 32 list entries on consecutive blocks: the warp's first chunk
 * and the stride between its chunks */
static __device__ __forceinline__ int first_chunk(int block, int nblocks)
{
    return (threadIdx.x >> 5) * nblocks + block;
}

__global__ void __launch_bounds__(THREADS) k1_flows(const __grid_constant__ Params p)
{
    const int par = p.counts[C_PAR], epoch = p.counts[C_EPOCH];
    if (blockIdx.x == 0 && threadIdx.x == 0)
        p.counts[1 - par] = 0; /* the list K2 appends to */
    flows_work(p, par, epoch, p.counts[par], first_chunk(blockIdx.x, gridDim.x), gridDim.x * (THREADS / 32));
}

__global__ void __launch_bounds__(THREADS) k2_update(const __grid_constant__ Params p)
{
    const int par = p.counts[C_PAR], epoch = p.counts[C_EPOCH];
    update_work(p, par, epoch, p.counts[par] + p.counts[C_EXT + par], first_chunk(blockIdx.x, gridDim.x),
                gridDim.x * (THREADS / 32));
    if (threadIdx.x == 0) {
        /* the last block to finish advances parity and epoch */
        __threadfence();
        if (atomicAdd(reinterpret_cast<unsigned*>(p.counts + C_TICKET), 1u) == gridDim.x - 1) {
            p.counts[C_PAR] = 1 - par;
            p.counts[C_EPOCH] = epoch + 1;
            p.counts[C_EXT + par] = 0;
            p.counts[C_TICKET] = 0;
        }
    }
}

/* every step of a run in one cooperative launch: the flows phase, a grid
 * barrier, the update phase, a grid barrier; work dealt in the placement
 * order (sdt2::placement_order) */
__global__ void __launch_bounds__(THREADS, 4) k_persist(const __grid_constant__ Params p, int nsteps, int nsm)
{
    __shared__ int s_cnt[2];
    const unsigned nb = gridDim.x;
    unsigned round = 0;
    const int vb = sdt2::placement_order(p.counts, nb, nsm, round, s_cnt);
    if (vb < 0)
        return;
    if (threadIdx.x == 0) {
        s_cnt[0] = __ldcg(p.counts + C_PAR);
        s_cnt[1] = __ldcg(p.counts + C_EPOCH);
    }
    __syncthreads();
    int par = s_cnt[0], epoch = s_cnt[1];
    __syncthreads();
    if (threadIdx.x == 0)
        s_cnt[0] = __ldcg(p.counts + par);
    __syncthreads();
    int na = s_cnt[0];
    const int g0 = first_chunk(vb, (int)nb), gs = (int)nb * (THREADS / 32);
    for (int s = 0; s < nsteps; s++) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            p.counts[1 - par] = 0; /* the list the update phase appends to */
        flows_work(p, par, epoch, na, g0, gs);
        /* then: the extended list's length */
        if (!sdt2::grid_barrier(p.counts, nb, round, p.counts + par, p.counts + C_EXT + par, s_cnt))
            return;
        const int n2 = s_cnt[0] + s_cnt[1];
        if (blockIdx.x == 0 && threadIdx.x == 0)
            p.counts[C_EXT + (1 - par)] = 0; /* next step's (read last by the previous step) */
        update_work(p, par, epoch, n2, g0, gs);
        par = 1 - par;
        epoch++;
        /* then: the next list's length */
        if (!sdt2::grid_barrier(p.counts, nb, round, p.counts + par, p.counts + par, s_cnt))
            return;
        na = s_cnt[0];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        /* the state the per-step kernels expect */
        p.counts[C_PAR] = par;
        p.counts[C_EPOCH] = epoch;
        p.counts[C_EXT] = 0;
        p.counts[C_EXT + 1] = 0;
        p.counts[C_TICKET] = 0;
    }
}

/* the initialisation's active set: every cell with h > 0 (epoch 1) */
__global__ void __launch_bounds__(THREADS) k_prime(const double* __restrict__ h, long long n, int* mark, int* list,
                                                   int* counts)
{
    if (blockIdx.x == 0 && threadIdx.x == 0)
        counts[C_EPOCH] = 1;
    const long long stride = (long long)gridDim.x * THREADS;
    for (long long base = (long long)blockIdx.x * THREADS; base < n; base += stride) {
        const long long c = base + threadIdx.x;
        const bool act = c < n && h[c] > 0.0;
        if (c < n)
            mark[c] = act ? 1 : 0;
        warp_append(act, (int)c, list, counts + 0);
    }
}

static void release()
{
    State& s = g_state;
    cudaFree(s.f);
    cudaFree(s.mark);
    cudaFree(s.list[0]);
    cudaFree(s.list[1]);
    cudaFree(s.counts);
    s = State();
}

/* (re)allocate for `ca` and take the initialisation's state from h */
static bool prime(struct CALModel2D* ca, const double* h, cudaStream_t st)
{
    State& s = g_state;
    const long long n = (long long)ca->rows * ca->columns;
    if (s.ca != ca || s.n != n) {
        release();
        s.ca = ca;
        s.n = n;
        bool ok = n <= 0x7fffffffLL && cudaMalloc(&s.f, 4 * n * sizeof(double)) == cudaSuccess &&
                  cudaMalloc(&s.mark, n * sizeof(int)) == cudaSuccess &&
                  cudaMalloc(&s.list[0], n * sizeof(int)) == cudaSuccess &&
                  cudaMalloc(&s.list[1], n * sizeof(int)) == cudaSuccess &&
                  cudaMalloc(&s.counts, NCOUNTS * sizeof(int)) == cudaSuccess;
        if (!ok) {
            release();
            return false;
        }
    }
    cudaMemsetAsync(s.f, 0, 4 * n * sizeof(double), st);
    cudaMemsetAsync(s.counts, 0, NCOUNTS * sizeof(int), st);
    long long blocks = (n + THREADS - 1) / THREADS;
    if (blocks > 152 * 16)
        blocks = 152 * 16;
    k_prime<<<(int)blocks, THREADS, 0, st>>>(h, n, s.mark, s.list[0], s.counts);
    s.primed = cudaGetLastError() == cudaSuccess;
    return s.primed;
}

static Params params(struct CALModel2D* ca, const double* z, double* h, double eps, double r, long long eps_bits)
{
    State& s = g_state;
    Params p;
    p.z = z;
    p.h = h;
    p.f = s.f;
    p.mark = s.mark;
    p.list0 = s.list[0];
    p.list1 = s.list[1];
    p.counts = s.counts;
    p.rows = ca->rows;
    p.cols = ca->columns;
    p.toroidal = ca->T == CAL_SPACE_TOROIDAL;
    p.n = s.n;
    p.eps = eps;
    p.r = r;
    p.eps_bits = eps_bits;
    return p;
}

/* one step: K1 then K2 on the model's stream */
static bool step(struct CALModel2D* ca, const double* z, double* h, double eps, double r, long long eps_bits,
                 cudaStream_t st)
{
    const Params p = params(ca, z, h, eps, r, eps_bits);
    k1_flows<<<BLOCKS, THREADS, 0, st>>>(p);
    k2_update<<<BLOCKS, THREADS, 0, st>>>(p);
    return cudaGetLastError() == cudaSuccess;
}

/* `nsteps` steps in one cooperative launch of k_persist (SMs x resident
 * blocks per SM); false when the launch is refused or a CUDA error is
 * pending.  A barrier that gave up sets the error word persist_failed()
 * reports. */
static bool persist(struct CALModel2D* ca, const double* z, double* h, double eps, double r, long long eps_bits,
                    int nsteps, cudaStream_t st)
{
    State& s = g_state;
    static int grid = 0, nsm = 0;
    if (!grid) {
        int per_sm = 0, dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persist, THREADS, 0);
        grid = sms * per_sm;
        nsm = sms;
        if (grid <= 0)
            return false;
    }
    Params p = params(ca, z, h, eps, r, eps_bits);
    cudaMemsetAsync(s.counts + sdt2::C_ARRIVED, 0, sizeof(int), st);
    cudaMemsetAsync(s.counts + sdt2::C_ERROR, 0, sizeof(int), st);
    cudaMemsetAsync(s.counts + sdt2::C_PLACE_BAD, 0, (NCOUNTS - sdt2::C_PLACE_BAD) * sizeof(int), st);
    void* args[] = {&p, &nsteps, &nsm};
    return cudaLaunchCooperativeKernel((const void*)k_persist, dim3(grid), dim3(THREADS), args, 0, st) ==
           cudaSuccess;
}

/* did the last persistent run give up at a barrier?  (synchronises) */
static int persist_failed(cudaStream_t st)
{
    int flag = 0;
    if (!g_state.counts)
        return 0;
    cudaStreamSynchronize(st);
    cudaMemcpy(&flag, g_state.counts + sdt2::C_ERROR, sizeof(int), cudaMemcpyDeviceToHost);
    return flag;
}

/* the active cells in row-major order (cells[2k], cells[2k + 1] = i, j;
 * cells may be null) and their number; synchronises */
static long read_active(int rows, int cols, int* cells, cudaStream_t st)
{
    State& s = g_state;
    if (!s.primed)
        return 0;
    int c[NCOUNTS];
    int* mark = (int*)malloc(sizeof(int) * (size_t)s.n);
    if (!mark)
        return 0;
    if (cudaMemcpyAsync(c, s.counts, sizeof(c), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(mark, s.mark, sizeof(int) * (size_t)s.n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        free(mark);
        return 0;
    }
    long m = 0;
    for (long long k = 0; k < s.n; k++)
        if (mark[k] == c[C_EPOCH]) {
            if (cells) {
                cells[2 * m] = (int)(k / cols);
                cells[2 * m + 1] = (int)(k % cols);
            }
            m++;
        }
    free(mark);
    (void)rows;
    return m;
}

} // namespace sdtac

/* ======================= 2c. the sparse fused step ======================
 * One launch per step.  A tile (32 x 16 cells) can only change in a step if
 * it holds a wet cell or borders one, so the step works on the tiles of
 * L_t = dilate(W_{t-1}) u dilate(W_t), W_t the tiles holding a wet cell of
 * h_t and dilate() the 3 x 3 tile neighbourhood (wrapping on a toroidal
 * grid).  Each listed tile runs the fused step of the single-kernel path
 * (sdt::fused_tile: z, h staged with a 2-cell ring in shared memory, the
 * wet cells of tile + ring compacted, EP 1 on them, EP 2 on the tile) from
 * one h buffer into the other, and marks its neighbourhood for step t+1
 * when it held a wet cell before or after the step.  Membership is a flag
 * per tile, double-buffered by step parity: step t reads and clears one
 * buffer (each tile's flag belongs to one block: tile t to block t mod
 * grid), marks go to the other.  The h buffers are the substate's two
 * layers, used alternately; the parity word says which one holds the state.
 * Invariant: the input buffer of step t holds h_t everywhere, because a tile
 * left out of L_t was not changed by steps t-1 and t, so both buffers hold
 * its value.  Resolving (before the host reads h) swaps the layer pointers
 * when the state sits in the second buffer: a pointer exchange, no copy.
 * Every launch of the step is identical (parity and ticket in device
 * memory), so a recorded step replays. */
namespace sdt3 {

constexpr int TW = 32, TH = 16;
constexpr int THREADS = sdt::THREADS;

struct Params {
    const double* __restrict__ z;
    double* h0;
    double* h1;
    int* flags0;
    int* flags1;
    int* ctrl; /* [0] parity: which buffer holds the state, [1] block ticket */
    int rows, cols, toroidal, tiles_x, tiles_y, ntiles;
    double eps, r;
    long long eps_bits;
};

struct State {
    struct CALModel2D* ca = nullptr;
    double* h[2] = {nullptr, nullptr};
    int* flags[2] = {nullptr, nullptr};
    int* ctrl = nullptr;
    int tiles_x = 0, tiles_y = 0;
    long long n = 0;
    bool primed = false;
};
static State g_state;

__global__ void __launch_bounds__(THREADS, 4) k_sparse_step(const __grid_constant__ Params p)
{
    extern __shared__ __align__(16) double smem[];
    __shared__ int s_tiles[THREADS];
    __shared__ int s_count;
    const int par = p.ctrl[0];
    const double* hin = par ? p.h1 : p.h0;
    double* hout = par ? p.h0 : p.h1;
    int* cur = par ? p.flags1 : p.flags0;
    int* nxt = par ? p.flags0 : p.flags1;
    sdt::Params fp;
    fp.z = p.z;
    fp.h = hin;
    fp.h_next = hout;
    fp.rows = p.rows;
    fp.cols = p.cols;
    fp.toroidal = p.toroidal;
    fp.eps = p.eps;
    fp.r = p.r;
    fp.eps_bits = p.eps_bits;
    /* this block's tiles: blockIdx.x + k * gridDim.x, THREADS candidates at a time */
    for (int base = 0; base * (int)gridDim.x < p.ntiles; base += THREADS) {
        if (threadIdx.x == 0)
            s_count = 0;
        __syncthreads();
        const int t = blockIdx.x + (base + (int)threadIdx.x) * (int)gridDim.x;
        bool mine = false;
        if (t < p.ntiles && cur[t]) {
            cur[t] = 0; /* read and cleared by its owner only */
            mine = true;
        }
        const unsigned m = __ballot_sync(0xffffffffu, mine);
        if (m) {
            int b = 0;
            if ((threadIdx.x & 31) == 0)
                b = atomicAdd(&s_count, __popc(m));
            b = __shfl_sync(0xffffffffu, b, 0);
            if (mine)
                s_tiles[b + __popc(m & ((1u << (threadIdx.x & 31)) - 1u))] = t;
        }
        __syncthreads();
        const int nt = s_count;
        for (int k = 0; k < nt; k++) {
            const int tile = s_tiles[k];
            const int ty = tile / p.tiles_x, tx = tile - ty * p.tiles_x;
            const int wet = sdt::fused_tile<TW, TH, true>(fp, ty * TH, tx * TW, smem);
            if (wet && threadIdx.x < 9) {
                int y = ty + (int)threadIdx.x / 3 - 1, x = tx + (int)threadIdx.x % 3 - 1;
                bool ok = true;
                if (p.toroidal) {
                    y = y < 0 ? y + p.tiles_y : (y >= p.tiles_y ? y - p.tiles_y : y);
                    x = x < 0 ? x + p.tiles_x : (x >= p.tiles_x ? x - p.tiles_x : x);
                } else {
                    ok = (unsigned)y < (unsigned)p.tiles_y && (unsigned)x < (unsigned)p.tiles_x;
                }
                if (ok)
                    nxt[y * p.tiles_x + x] = 1;
            }
            __syncthreads(); /* shared memory is reused by the next tile */
        }
    }
    if (threadIdx.x == 0) {
        /* every block read the parity at its start; the last one to finish
         * flips it (no block waits for another) */
        __threadfence();
        if (atomicAdd(reinterpret_cast<unsigned*>(p.ctrl + 1), 1u) == gridDim.x - 1) {
            p.ctrl[0] = 1 - par;
            p.ctrl[1] = 0;
        }
    }
}

/* both buffers = h with -0 made +0 (the first reference step adds 0.0 to
 * every cell); flags0 = the 3 x 3 tiles around every tile with a wet cell */
__global__ void k_prime(double* h0, double* h1, long long n, int cols, int tiles_x, int tiles_y, int toroidal,
                        long long eps_bits, int* flags0)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const double v = sdt::plus_zero(h0[c]);
        h0[c] = v;
        h1[c] = v;
        if (sdt::is_wet(v, eps_bits)) {
            const int i = (int)(c / cols), j = (int)(c - (long long)(c / cols) * cols);
            const int ty = i / TH, tx = j / TW;
            for (int q = 0; q < 9; q++) {
                int y = ty + q / 3 - 1, x = tx + q % 3 - 1;
                if (toroidal) {
                    y = y < 0 ? y + tiles_y : (y >= tiles_y ? y - tiles_y : y);
                    x = x < 0 ? x + tiles_x : (x >= tiles_x ? x - tiles_x : x);
                } else if ((unsigned)y >= (unsigned)tiles_y || (unsigned)x >= (unsigned)tiles_x) {
                    continue;
                }
                flags0[y * tiles_x + x] = 1;
            }
        }
    }
}

static void release()
{
    State& s = g_state;
    cudaFree(s.flags[0]);
    cudaFree(s.flags[1]);
    cudaFree(s.ctrl);
    s = State();
}

static int step_grid()
{
    static int blocks = 0;
    if (!blocks) {
        const int smem = (int)sdt::Tile<TW, TH>::smem_bytes;
        cudaFuncSetAttribute(k_sparse_step, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        int per_sm = 1, dev = 0, sms = 152;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sparse_step, THREADS, smem);
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        blocks = sms * (per_sm > 0 ? per_sm : 1);
    }
    return blocks;
}

/* (re)prime from the substate's current layer; its next layer becomes the
 * second buffer */
static bool prime(struct CALModel2D* ca, double* cur, double* nxt, long long eps_bits, cudaStream_t st)
{
    State& s = g_state;
    const long long n = (long long)ca->rows * ca->columns;
    if (s.ca != ca || s.n != n) {
        release();
        s.ca = ca;
        s.n = n;
        s.tiles_x = (ca->columns + TW - 1) / TW;
        s.tiles_y = (ca->rows + TH - 1) / TH;
        const size_t fb = sizeof(int) * (size_t)s.tiles_x * s.tiles_y;
        if (cudaMalloc(&s.flags[0], fb) != cudaSuccess || cudaMalloc(&s.flags[1], fb) != cudaSuccess ||
            cudaMalloc(&s.ctrl, 4 * sizeof(int)) != cudaSuccess) {
            release();
            return false;
        }
    }
    s.h[0] = cur;
    s.h[1] = nxt;
    const size_t fb = sizeof(int) * (size_t)s.tiles_x * s.tiles_y;
    cudaMemsetAsync(s.flags[0], 0, fb, st);
    cudaMemsetAsync(s.flags[1], 0, fb, st);
    cudaMemsetAsync(s.ctrl, 0, 4 * sizeof(int), st);
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16)
        blocks = 152 * 16;
    k_prime<<<blocks, 256, 0, st>>>(cur, nxt, n, ca->columns, s.tiles_x, s.tiles_y, ca->T == CAL_SPACE_TOROIDAL,
                                    eps_bits, s.flags[0]);
    s.primed = true;
    return cudaGetLastError() == cudaSuccess;
}

static bool step(struct CALModel2D* ca, const double* z, double eps, double r, long long eps_bits, cudaStream_t st)
{
    State& s = g_state;
    Params p;
    p.z = z;
    p.h0 = s.h[0];
    p.h1 = s.h[1];
    p.flags0 = s.flags[0];
    p.flags1 = s.flags[1];
    p.ctrl = s.ctrl;
    p.rows = ca->rows;
    p.cols = ca->columns;
    p.toroidal = ca->T == CAL_SPACE_TOROIDAL;
    p.tiles_x = s.tiles_x;
    p.tiles_y = s.tiles_y;
    p.ntiles = s.tiles_x * s.tiles_y;
    p.eps = eps;
    p.r = r;
    p.eps_bits = eps_bits;
    k_sparse_step<<<step_grid(), THREADS, sdt::Tile<TW, TH>::smem_bytes, st>>>(p);
    return cudaGetLastError() == cudaSuccess;
}

} // namespace sdt3

enum SdtKernel { SDT_SPARSE = 0, SDT_SPLIT = 1, SDT_SINGLE = 2 };

/* the plain-mode step: the split step (outflows of the wet cells spread
 * over the whole GPU, then the update) unless OPENCAL_SDT_KERNEL=sparse |
 * single selects the sparse fused step (one launch per step; its FP64 work
 * stays on the SMs that own the flow's tiles) or the dense single kernel */
static SdtKernel sdt_kernel()
{
    const char* e = getenv("OPENCAL_SDT_KERNEL");
    if (e && !strcmp(e, "sparse"))
        return SDT_SPARSE;
    if (e && !strcmp(e, "single"))
        return SDT_SINGLE;
    return SDT_SPLIT;
}

static bool sdt_use_split() { return sdt_kernel() == SDT_SPLIT; }

/* before the host or another process touches h: if the sparse step left the
 * state in the substate's next layer, exchange the layer pointers (and the
 * step's buffer roles) so that current holds it.  Synchronises. */
static void sciddicaT_sparse_resolve(struct CALModel2D* ca)
{
    sdt3::State& s = sdt3::g_state;
    if (!s.primed || s.ca != ca)
        return;
    cudaStream_t st = (cudaStream_t)calGetStream2D(ca);
    int par = 0;
    cudaStreamSynchronize(st);
    cudaMemcpy(&par, s.ctrl, sizeof(int), cudaMemcpyDeviceToHost);
    if (par) {
        calSwapSubstate2Dr(ca, Q.h);
        double* t = s.h[0];
        s.h[0] = s.h[1];
        s.h[1] = t;
        int* f = s.flags[0];
        s.flags[0] = s.flags[1];
        s.flags[1] = f;
        const int zero = 0;
        cudaMemcpy(s.ctrl, &zero, sizeof(int), cudaMemcpyHostToDevice);
    }
}

static void sciddicaT_sparse_invalidate() { sdt3::g_state.primed = false; }

static void sciddicaT_sparse_prepare(struct CALModel2D* ca)
{
    if (sdt_kernel() != SDT_SPARSE || (sdt3::g_state.ca == ca && sdt3::g_state.primed))
        return;
    long long eps_bits;
    memcpy(&eps_bits, &P.epsilon, sizeof(double));
    double* cur = (double*)calGetDeviceBuffer2Dr(ca, Q.h, 0);
    double* nxt = (double*)calGetDeviceBuffer2Dr(ca, Q.h, 2);
    sdt3::prime(ca, cur, nxt, eps_bits, (cudaStream_t)calGetStream2D(ca));
}

static void sciddicaT_sparse_transition(struct CALModel2D* ca)
{
    long long eps_bits;
    memcpy(&eps_bits, &P.epsilon, sizeof(double));
    if (sdt3::g_state.ca != ca || !sdt3::g_state.primed)
        sciddicaT_sparse_prepare(ca);
    const double* z = (const double*)calGetDeviceBuffer2Dr(ca, Q.z, 0);
    (void)calGetDeviceBuffer2Dr(ca, Q.h, 2); /* both layers change: host copies stale */
    calMarkCurrentWritten2Dr(ca, Q.h);
    sdt3::step(ca, z, P.epsilon, P.r, eps_bits, (cudaStream_t)calGetStream2D(ca));
}

static void sciddicaT_split_prepare_now(struct CALModel2D* ca);

/* the split step as a global transition (h updated in place) */
static void sciddicaT_split_transition_timed(struct CALModel2D* ca, cudaEvent_t* ev)
{
    const double* z = (const double*)calGetDeviceBuffer2Dr(ca, Q.z, 0);
    double* h = (double*)calGetDeviceBuffer2Dr(ca, Q.h, 0);
    cudaStream_t st = (cudaStream_t)calGetStream2D(ca);
    long long eps_bits;
    memcpy(&eps_bits, &P.epsilon, sizeof(double));
    if (sdt2::g_state.ca != ca || !sdt2::g_state.primed || sdt3::g_state.primed) {
        sciddicaT_split_prepare_now(ca);
        h = (double*)calGetDeviceBuffer2Dr(ca, Q.h, 0);
    }
    if (!sdt2::g_state.primed) {
        cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "SCIDDICA-T split step: buffers not allocated");
        return;
    }
    sdt2::step(ca, z, h, P.epsilon, P.r, eps_bits, st, ev);
    calMarkCurrentWritten2Dr(ca, Q.h);
}

/* the split and sparse steps keep device state derived from h; anything
 * that changes h behind their back makes them re-prime */
static void sciddicaT_step_invalidate()
{
    sdt2::g_state.primed = false;
    sdt3::g_state.primed = false;
    sdtac::g_state.primed = false;
}

/* the fused step of a run with active cells is the active-cells split step */
static bool g_fused_ac = false;

/* prime the active-cells split step from the initialised state (its
 * active set: every cell with h > 0) unless it is primed for `ca` */
static void sciddicaT_ac_prepare_now(struct CALModel2D* ca)
{
    if (sdtac::g_state.ca == ca && sdtac::g_state.primed)
        return;
    sdtac::prime(ca, (const double*)calGetDeviceBuffer2Dr(ca, Q.h, 0), (cudaStream_t)calGetStream2D(ca));
}

static void sciddicaT_ac_transition(struct CALModel2D* ca)
{
    sciddicaT_ac_prepare_now(ca);
    if (!sdtac::g_state.primed) {
        cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "SCIDDICA-T active-cells split step: buffers not allocated");
        return;
    }
    long long eps_bits;
    memcpy(&eps_bits, &P.epsilon, sizeof(double));
    const double* z = (const double*)calGetDeviceBuffer2Dr(ca, Q.z, 0);
    double* h = (double*)calGetDeviceBuffer2Dr(ca, Q.h, 0);
    sdtac::step(ca, z, h, P.epsilon, P.r, eps_bits, (cudaStream_t)calGetStream2D(ca));
    calMarkCurrentWritten2Dr(ca, Q.h);
}

/* prime the split step now (eagerly), handing h over from the sparse step
 * if that ran last */
static void sciddicaT_split_prepare_now(struct CALModel2D* ca)
{
    if (sdt3::g_state.primed && sdt3::g_state.ca == ca) {
        sciddicaT_sparse_resolve(ca);
        sciddicaT_sparse_invalidate();
        sdt2::g_state.primed = false;
    }
    if (sdt2::g_state.ca == ca && sdt2::g_state.primed)
        return;
    long long eps_bits;
    memcpy(&eps_bits, &P.epsilon, sizeof(double));
    sdt2::prime(ca, (double*)calGetDeviceBuffer2Dr(ca, Q.h, 0), (const double*)calGetDeviceBuffer2Dr(ca, Q.z, 0),
                P.epsilon, eps_bits, (cudaStream_t)calGetStream2D(ca));
}

/* prime the selected plain-mode step now if its next step would: keeps the
 * priming out of a step that is being recorded as a graph */
static void sciddicaT_step_prepare(struct CALModel2D* ca)
{
    if (g_fused_ac) {
        sciddicaT_ac_prepare_now(ca);
        return;
    }
    const SdtKernel k = sdt_kernel();
    if (k == SDT_SPLIT) {
        sciddicaT_split_prepare_now(ca);
    } else if (k == SDT_SPARSE) {
        if (sdt2::g_state.primed && sdt2::g_state.ca == ca) /* h is current after split steps */
            sdt2::g_state.primed = false;
        sciddicaT_sparse_prepare(ca);
    }
}

/* host side of the fused step: queue the kernel, then exchange the h layers */
static void sciddicaT_fused_transition(struct CALModel2D* ca)
{
    if (g_fused_ac) {
        sciddicaT_ac_transition(ca);
        return;
    }
    if (sdt_kernel() == SDT_SPARSE) {
        sciddicaT_sparse_transition(ca);
        return;
    }
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
    /* the init's z -= h is in the next layer until the run's update; the
     * split step's priming reads z (z + h, z + epsilon per cell), so the
     * update runs here (the run's own update after the init then finds
     * nothing written and copies nothing) */
    calUpdate2D(sciddicaT);
    sciddicaT_step_invalidate();
    sciddicaT_step_prepare(sciddicaT);
}

/* ======================= driver entry points ============================ */

/* The two processes of the plain program read only z, h and the outflows
 * over the von Neumann neighbourhood and the run's constant parameters:
 * pure in the sense of calSetElementaryProcessPure2D.  Declared when
 * cal_sciddicaT_set_pure(1) was called (off by default: the reference
 * program as it stands). */
static int g_sdt_pure = 0;
static int g_sdt_staged = 0;
static int g_sdt_guard = 0;

/* the declarations cal_sciddicaT_set_pure / _set_staged asked for; called
 * once the processes and the substates exist */
static void sciddicaT_declare_pure(struct CALModel2D* ca)
{
    if (g_sdt_pure) {
        calSetElementaryProcessPure2D(ca, sciddicaT_flows_computation, CAL_TRUE);
        calSetElementaryProcessPure2D(ca, sciddicaT_width_update, CAL_TRUE);
    }
    if (g_sdt_staged) {
        const void* flows_reads[2] = {Q.z, Q.h};
        const void* width_reads[5] = {Q.h, Q.f[0], Q.f[1], Q.f[2], Q.f[3]};
        calSetElementaryProcessReads2D(ca, sciddicaT_flows_computation, flows_reads, 2);
        calSetElementaryProcessReads2D(ca, sciddicaT_width_update, width_reads, 5);
    }
    /* the flows process starts with `if (h <= epsilon) return;` */
    if (g_sdt_guard)
        calSetElementaryProcessGuard2Dr(ca, sciddicaT_flows_computation, Q.h, CAL_GUARD_LE, P.epsilon);
}

extern "C" int cal_sciddicaT_set_pure(int on)
{
    g_sdt_pure = on != 0;
    return 0;
}

/* 1: models created afterwards (processes mode) declare the flows
 * process's early return on dry cells (calSetElementaryProcessGuard2Dr), so
 * that its kernel runs it on the wet cells of each tile packed into
 * consecutive threads; 0 (default): every cell's thread runs it */
extern "C" int cal_sciddicaT_set_guard(int on)
{
    g_sdt_guard = on != 0;
    return 0;
}

/* 1: models created afterwards (processes mode) declare what the two plain
 * processes read (calSetElementaryProcessReads2D), so that the process
 * kernels stage z, h and the outflows by TMA; 0 (default): global reads */
extern "C" int cal_sciddicaT_set_staged(int on)
{
    g_sdt_staged = on != 0;
    return 0;
}

enum { SDT_MODE_PROCESSES = 0, SDT_MODE_FUSED = 1 };

/* The reference example's main() as it stands (OpenCAL-OMP/examples/
 * calomp_sciddicaT/source/sciddicaT.c:140-180): the model, its two device
 * processes and six substates, z and h loaded from text files with
 * calLoadSubstate2Dr, the run (init, steering, IMPLICIT updates) with
 * calRun2D, and h saved with calSaveSubstate2Dr.  graph: 1 replays the
 * recorded step.  Returns a CALError code (CAL_ERROR_IO when a file cannot
 * be read or written). */
extern "C" int cal_sciddicaT_run_files(int rows, int cols, int toroidal, int steps, double p_r, double p_eps,
                                       const char* dem_path, const char* source_path, const char* output_path,
                                       int graph)
{
    sdt2::g_state.hknown = false;
    calClearError();
    sciddicaT_step_invalidate();
    g_fused_ac = false;
    struct CALModel2D* ca = calCADef2D(rows, cols, CAL_VON_NEUMANN_NEIGHBORHOOD_2D,
                                       toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    if (!ca)
        return calGetLastError();
    struct CALRun2D* run = calRunDef2D(ca, 1, steps, CAL_UPDATE_IMPLICIT);
    P.epsilon = p_eps;
    P.r = p_r;
    P.active = 0;
    calAddElementaryProcess2D(ca, sciddicaT_flows_computation);
    calAddElementaryProcess2D(ca, sciddicaT_width_update);
    Q.z = calAddSubstate2Dr(ca);
    Q.h = calAddSubstate2Dr(ca);
    for (int q = 0; q < NUMBER_OF_OUTFLOWS; q++)
        Q.f[q] = calAddSubstate2Dr(ca);
    int err = CAL_SUCCESS;
    if (!calLoadSubstate2Dr(ca, Q.z, (char*)dem_path) || !calLoadSubstate2Dr(ca, Q.h, (char*)source_path)) {
        err = CAL_ERROR_IO;
    } else {
        calRunAddInitFunc2D(run, sciddicaT_simulation_init);
        calRunAddSteeringFunc2D(run, sciddicaT_steering_plain);
        calRunSetGraph2D(run, graph ? CAL_TRUE : CAL_FALSE);
        calRun2D(run);
        if (!calSaveSubstate2Dr(ca, Q.h, (char*)output_path) && calGetLastError() == CAL_SUCCESS)
            err = CAL_ERROR_IO;
    }
    if (err == CAL_SUCCESS)
        err = calGetLastError();
    calRunFinalize2D(run);
    calFinalize2D(ca);
    return err;
}

/* how many device-loop runs had to fall back to a launch sequence per step */
static int g_fallbacks = 0;
static void cal_note_fallback() { g_fallbacks++; }
extern "C" int cal_sciddicaT_device_loop_fallbacks(void) { return g_fallbacks; }

/* every one of `steps` steps in one cooperative launch: the persistent
 * split step (plain) or the persistent active-cells split step; the state
 * must be initialised.  Returns a CALError code (CAL_ERROR_CUDA also when a
 * grid barrier gave up, which synchronises). */
static int sciddicaT_persist_steps(struct CALModel2D* ca, int steps, bool fused_ac)
{
    long long eps_bits;
    memcpy(&eps_bits, &P.epsilon, sizeof(double));
    cudaStream_t st = (cudaStream_t)calGetStream2D(ca);
    if (fused_ac) {
        sciddicaT_ac_prepare_now(ca);
        if (!sdtac::g_state.primed)
            return CAL_ERROR_OUT_OF_MEMORY;
    } else {
        sciddicaT_split_prepare_now(ca);
        if (!sdt2::g_state.primed)
            return CAL_ERROR_OUT_OF_MEMORY;
    }
    const double* z = (const double*)calGetDeviceBuffer2Dr(ca, Q.z, 0);
    double* h = (double*)calGetDeviceBuffer2Dr(ca, Q.h, 0);
    const bool ok = fused_ac ? sdtac::persist(ca, z, h, P.epsilon, P.r, eps_bits, steps, st)
                             : sdt2::persist(ca, z, h, P.epsilon, P.r, eps_bits, steps, st);
    if (!ok)
        return CAL_ERROR_CUDA;
    calMarkCurrentWritten2Dr(ca, Q.h);
    return calGetLastError();
}

/* Runs SCIDDICA-T for `steps` steps on (z0, h0) and returns the final z, h
 * and active list -- the same contract as the oracle's orc_sciddicaT.
 * mode 0 runs the reference program (device processes); mode 1 the fused
 * step (plain mode: the split step; with active cells: the active-cells
 * split step).  graph != 0 replays the step as a CUDA graph.
 * *ms receives the device time of the step loop (CUDA events).  Returns 0
 * on success, else the CALError code. */
extern "C" int cal_sciddicaT_run(int rows, int cols, int toroidal, int ac, int steps, double p_r, double p_eps,
                                 const double* z0, const double* h0, double* z_out, double* h_out, long* n_active,
                                 int* cells_out, int mode, int graph, double* ms)
{
    sdt2::g_state.hknown = false; /* launches this library did not see may have run since */
    calClearError();
    /* with active cells, the fused mode keeps its own active set (epoch
     * marks) on a model without the active-cells option */
    const bool fused_ac = mode == SDT_MODE_FUSED && ac;
    sciddicaT_step_invalidate();
    g_fused_ac = fused_ac;
    struct CALModel2D* ca = calCADef2D(rows, cols, CAL_VON_NEUMANN_NEIGHBORHOOD_2D,
                                       toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT,
                                       (ac && !fused_ac) ? CAL_OPT_ACTIVE_CELLS : CAL_NO_OPT);
    if (!ca) {
        g_fused_ac = false;
        return calGetLastError();
    }
    struct CALRun2D* run = calRunDef2D(ca, 1, steps, CAL_UPDATE_IMPLICIT);
    P.epsilon = p_eps;
    P.r = p_r;
    P.active = ac && !fused_ac;
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
    if (mode == SDT_MODE_PROCESSES)
        sciddicaT_declare_pure(ca);
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
    } else if (graph == 4 && mode == SDT_MODE_FUSED) {
        /* every step in one cooperative launch (the persistent split step) */
        if (steps > 0 && sciddicaT_persist_steps(ca, steps, fused_ac) == CAL_SUCCESS &&
            (fused_ac ? sdtac::persist_failed(s) : sdt2::persist_failed(s)) != 0)
            cal::set_error(CAL_ERROR_CUDA, "SCIDDICA-T persistent step: a grid barrier gave up");
    } else {
        for (run->step = run->initial_step; run->step <= run->final_step; run->step++)
            if (!calRunCAStep2D(run))
                break;
    }
    cudaEventRecord(e1, s);
    sciddicaT_sparse_resolve(ca);
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
    if (fused_ac) {
        const long m = sdtac::read_active(rows, cols, cells_out, s);
        if (n_active)
            *n_active = m;
    } else {
        if (n_active)
            *n_active = ac ? ca->A.size_current : 0;
        if (cells_out && ac)
            memcpy(cells_out, ca->A.cells, sizeof(int) * 2 * (size_t)ca->A.size_current);
    }
    int err = calGetLastError();
    sdt2::release();
    sdtac::release();
    g_fused_ac = false;
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
    int fused_ac; /* active cells in fused mode: the active-cells split step */
    size_t bytes;
    double* snap[6][2]; /* device copies of z, h, f0..f3 (both layers) after init */
    CALbyte* snap_flags;
};

static struct CALSubstate2Dr* sdt_sub(int k) { return k == 0 ? Q.z : (k == 1 ? Q.h : Q.f[k - 2]); }

extern "C" void* cal_sciddicaT_open(int rows, int cols, int toroidal, int ac, double p_r, double p_eps,
                                    const double* z0, const double* h0, int mode)
{
    calClearError();
    sciddicaT_step_invalidate();
    SdtSession* s = (SdtSession*)calloc(1, sizeof(SdtSession));
    s->mode = mode;
    s->ac = ac;
    s->fused_ac = mode == SDT_MODE_FUSED && ac;
    g_fused_ac = s->fused_ac;
    s->bytes = sizeof(double) * (size_t)rows * cols;
    s->ca = calCADef2D(rows, cols, CAL_VON_NEUMANN_NEIGHBORHOOD_2D, toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT,
                       (ac && !s->fused_ac) ? CAL_OPT_ACTIVE_CELLS : CAL_NO_OPT);
    if (!s->ca) {
        g_fused_ac = false;
        free(s);
        return nullptr;
    }
    s->run = calRunDef2D(s->ca, 1, CAL_RUN_LOOP, CAL_UPDATE_IMPLICIT);
    P.epsilon = p_eps;
    P.r = p_r;
    P.active = ac && !s->fused_ac;
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
    if (mode == SDT_MODE_PROCESSES)
        sciddicaT_declare_pure(s->ca);
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
            if (mode == SDT_MODE_PROCESSES) {
                /* through the API, so that the substates keep their change
                 * tracking (after the init's update both layers are equal) */
                if (l == 0)
                    calCopySubstateToHost2Dr(s->ca, sdt_sub(k), (double*)s->snap[k][0]);
                continue;
            }
            cudaMemcpyAsync(s->snap[k][l], calGetDeviceBuffer2Dr(s->ca, sdt_sub(k), l), s->bytes,
                            cudaMemcpyDeviceToDevice, st);
        }
    if (ac && !s->fused_ac) {
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
    sdt2::g_state.hknown = false; /* launches this library did not see may have run since */
    SdtSession* s = (SdtSession*)handle;
    sciddicaT_step_invalidate();
    cudaStream_t st = (cudaStream_t)calGetStream2D(s->ca);
    if (s->mode == SDT_MODE_PROCESSES) {
        for (int k = 0; k < 6; k++)
            calCopySubstateFromHost2Dr(s->ca, sdt_sub(k), (const double*)s->snap[k][0]);
    } else {
        for (int k = 0; k < 6; k++)
            for (int l = 0; l < 2; l++)
                cudaMemcpyAsync(calGetDeviceBuffer2Dr(s->ca, sdt_sub(k), l == 0 ? 0 : 2), s->snap[k][l], s->bytes,
                                cudaMemcpyDeviceToDevice, st);
    }
    if (s->ac && !s->fused_ac) {
        CALbyte* flags;
        calGetDeviceActiveCells2D(s->ca, &flags, nullptr, nullptr);
        cudaMemcpyAsync(flags, s->snap_flags, (size_t)s->ca->rows * s->ca->columns, cudaMemcpyDeviceToDevice, st);
        calUpdateActiveCells2D(s->ca);
    }
    if (s->mode != SDT_MODE_PROCESSES)
        calMarkDeviceWritten2D(s->ca);
    return calGetLastError();
}

/* queue `steps` steps; graph != 0 replays a recorded step */
extern "C" int cal_sciddicaT_steps(void* handle, int steps, int graph)
{
    sdt2::g_state.hknown = false; /* launches this library did not see may have run since */
    SdtSession* s = (SdtSession*)handle;
    if (graph == 4) {
        if (s->mode != SDT_MODE_FUSED)
            return CAL_ERROR_INVALID_ARGUMENT;
        return sciddicaT_persist_steps(s->ca, steps, s->fused_ac);
    }
    if (s->mode == SDT_MODE_FUSED)
        sciddicaT_step_prepare(s->ca);
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
    if (s->mode == SDT_MODE_PROCESSES)
        sciddicaT_declare_pure(s->ca); /* the guard holds epsilon's value */
    calRunSetGraph2D(s->run, CAL_FALSE);
    return calGetLastError();
}

/* launch grids of the split step's two kernels (256-thread blocks; 0
 * restores the default 608 / 608); a recorded
 * step, which bakes them into its launches, is dropped */
extern "C" int cal_sciddicaT_set_split_grid(void* handle, int k1_blocks, int k2_blocks)
{
    SdtSession* s = (SdtSession*)handle;
    if (k1_blocks < 0 || k2_blocks < 0)
        return CAL_ERROR_INVALID_ARGUMENT;
    sdt2::g_k1_blocks = k1_blocks ? k1_blocks : 152 * 4;
    sdt2::g_k2_blocks = k2_blocks ? k2_blocks : sdt2::K2_BLOCKS;
    calRunSetGraph2D(s->run, CAL_FALSE);
    return calGetLastError();
}

/* the dense step's TMA form: launches queued by this library's SCIDDICA-T
 * programs so far, and tiles whose copies did not complete in time
 * (synchronises the device) */
extern "C" int cal_sciddicaT_tma_stats(long long* launches, int* timeouts)
{
    if (launches)
        *launches = sdt::g_tma_launches;
    if (timeouts) {
        *timeouts = 0;
        if (cudaDeviceSynchronize() != cudaSuccess ||
            cudaMemcpyFromSymbol(timeouts, sdt::g_tma_timeouts, sizeof(int)) != cudaSuccess)
            return CAL_ERROR_CUDA;
    }
    return CAL_SUCCESS;
}

extern "C" void* cal_sciddicaT_stream(void* handle) { return calGetStream2D(((SdtSession*)handle)->ca); }

/* 1 when a barrier of the last persistent run gave up (the run stopped
 * early and the state is not that of the requested step); synchronises */
extern "C" int cal_sciddicaT_persist_failed(void* handle)
{
    SdtSession* s = (SdtSession*)handle;
    cudaStream_t st = (cudaStream_t)calGetStream2D(s->ca);
    return s->fused_ac ? sdtac::persist_failed(st) : sdt2::persist_failed(st);
}

/* host-buffer round trip through the API: z and h from the caller's arrays
 * into the model (calCopySubstateFromHost2Dr), the program's init and
 * `steps` steps (graph: as for cal_sciddicaT_steps), h back into the
 * caller's array (calCopySubstateToHost2Dr) */
extern "C" int cal_sciddicaT_host_run(void* handle, const double* z_host, const double* h_host, int steps, int graph,
                                      double* h_out)
{
    sdt2::g_state.hknown = false; /* launches this library did not see may have run since */
    SdtSession* s = (SdtSession*)handle;
    /* the inputs go straight from the caller's arrays to the device (both
     * layers, as the program's file loader leaves them); the outflows are
     * reset by the program's init */
    calCopySubstateFromHost2Dr(s->ca, Q.z, z_host);
    calCopySubstateFromHost2Dr(s->ca, Q.h, h_host);
    sciddicaT_step_invalidate();
    calRunInitSimulation2D(s->run); /* the program's init: z -= h at the source, f = 0 */
    cal_sciddicaT_steps(handle, steps, graph);
    sciddicaT_sparse_resolve(s->ca);
    calCopySubstateToHost2Dr(s->ca, Q.h, h_out);
    return calGetLastError();
}

/* device time of each of n steps' kernels, events around every launch:
 * split step -> ms_a[k] = K1 (outflows), ms_b[k] = K2 (update);
 * single fused kernel -> ms_a[k] = the kernel, ms_b[k] = 0 */
extern "C" int cal_sciddicaT_kernel_times(void* handle, int n, float* ms_a, float* ms_b)
{
    sdt2::g_state.hknown = false; /* launches this library did not see may have run since */
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
    if (!sdt2::g_state.counts)
        return -1;
    /* the model's stream does not synchronise with the legacy stream */
    cudaStreamSynchronize((cudaStream_t)calGetStream2D(s->ca));
    int c[6] = {0, 0, 0, 0, 0, 0};
    cudaMemcpy(c, sdt2::g_state.counts, sizeof(c), cudaMemcpyDeviceToHost);
    const int par = c[4] & 1;
    unsigned long long w = 0;
    cudaMemcpy(&w, sdt2::g_state.ctl + sdt2::W_LIST + 16 * par, sizeof(w), cudaMemcpyDeviceToHost);
    std::vector<int> list(sdt2::low32(w));
    if (!list.empty())
        cudaMemcpy(list.data(), sdt2::g_state.list[par], list.size() * sizeof(int), cudaMemcpyDeviceToHost);
    int wet = 0;
    for (int e : list)
        wet += e >= 0;
    return wet;
}

extern "C" int cal_sciddicaT_read(void* handle, double* h_out)
{
    SdtSession* s = (SdtSession*)handle;
    sciddicaT_sparse_resolve(s->ca);
    calSyncSubstate2Dr(s->ca, Q.h);
    memcpy(h_out, Q.h->current, s->bytes);
    return calGetLastError();
}

/* `steps` plain steps from the current state, one split step (K1, K2) at a
 * time, each followed by sdt2::k_trace: outflux[t] = mass that left the grid
 * in step t + 1, wet[t] = wet cells processed in it, *edge_step = first step
 * after which the two-cell edge band holds h != 0 (-1: none).  Host arrays;
 * flat grids of at least 5 x 5 cells, plain split-step sessions only.  A
 * measurement aid, not a timed path (two extra launches per step). */
extern "C" int cal_sciddicaT_trace(void* handle, int steps, double* outflux, int* wet, int* edge_step)
{
    sdt2::g_state.hknown = false;
    SdtSession* s = (SdtSession*)handle;
    struct CALModel2D* ca = s ? s->ca : nullptr;
    if (!s || s->mode != SDT_MODE_FUSED || s->fused_ac || steps < 0 || !outflux || !wet || !edge_step ||
        ca->T == CAL_SPACE_TOROIDAL || ca->rows < 5 || ca->columns < 5) {
        cal::set_error(CAL_ERROR_INVALID_ARGUMENT, "cal_sciddicaT_trace: plain split-step session on a flat grid");
        return CAL_ERROR_INVALID_ARGUMENT;
    }
    cudaStream_t st = (cudaStream_t)calGetStream2D(ca);
    sciddicaT_split_prepare_now(ca);
    if (!sdt2::g_state.primed)
        return CAL_ERROR_OUT_OF_MEMORY;
    double* d_out = nullptr;
    int* d_wet = nullptr;
    if (!cal_cuda(cudaMalloc(&d_out, sizeof(double) * (steps + 1)), "cudaMalloc trace") ||
        !cal_cuda(cudaMalloc(&d_wet, sizeof(int) * (steps + 2)), "cudaMalloc trace")) {
        cudaFree(d_out);
        return CAL_ERROR_CUDA;
    }
    int* d_edge = d_wet + steps + 1;
    const int never = 0x7fffffff;
    cudaMemcpyAsync(d_edge, &never, sizeof(int), cudaMemcpyHostToDevice, st);
    long long eps_bits;
    memcpy(&eps_bits, &P.epsilon, sizeof(double));
    const double* z = (const double*)calGetDeviceBuffer2Dr(ca, Q.z, 0);
    double* h = (double*)calGetDeviceBuffer2Dr(ca, Q.h, 0);
    for (int t = 0; t < steps; t++) {
        if (!sdt2::step(ca, z, h, P.epsilon, P.r, eps_bits, st, nullptr))
            break;
        sdt2::k_trace<<<1, sdt2::THREADS, 0, st>>>(sdt2::g_state.f, h, sdt2::g_state.counts, sdt2::g_state.ctl,
                                                   sdt2::g_state.list[0], sdt2::g_state.list[1], ca->rows,
                                                   ca->columns, sdt2::g_state.n, t, d_out, d_wet, d_edge);
    }
    calMarkCurrentWritten2Dr(ca, Q.h);
    int edge = never;
    if (cal_cuda(cudaGetLastError(), "trace launches") &&
        cal_cuda(cudaMemcpyAsync(outflux, d_out, sizeof(double) * steps, cudaMemcpyDeviceToHost, st), "trace") &&
        cal_cuda(cudaMemcpyAsync(wet, d_wet, sizeof(int) * steps, cudaMemcpyDeviceToHost, st), "trace") &&
        cal_cuda(cudaMemcpyAsync(&edge, d_edge, sizeof(int), cudaMemcpyDeviceToHost, st), "trace"))
        cal_cuda(cudaStreamSynchronize(st), "trace");
    *edge_step = edge == never ? -1 : edge;
    cudaFree(d_out);
    cudaFree(d_wet);
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
    sdtac::release();
    g_fused_ac = false;
    calRunFinalize2D(s->run);
    calFinalize2D(s->ca);
    free(s);
}
