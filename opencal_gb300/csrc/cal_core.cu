/*
 * cal_core.cu -- engine shared by the 2D and 3D C APIs: device buffers and
 * host mirrors of the substates, the update (next -> current) kernel, the
 * substate fill kernel and the active-cell compaction.
 *
 * Reference behaviour restated here:
 *   calUpdate2D            OpenCAL-OMP/source/cal2D.c:758-776
 *   calUpdateActiveCells2D OpenCAL-OMP/source/cal2D.c:382-440 (row-major list)
 *   calUpdateActiveCells3D OpenCAL-OMP/source/cal3D.c:313-370 (i, j, k order)
 *   calCopyBuffer2D* / calCopyActiveCellsBuffer2D*  cal2DBuffer.c:44-160
 *   calSetBuffer2D* / calSetActiveCellsBuffer2D*    cal2DBuffer.c:223-259
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>

#include "cal_core.cuh"

namespace cal {

/* ======================= errors ========================================= */

static thread_local CALError g_err = CAL_SUCCESS;
static thread_local char g_msg[512] = "";

void set_error(CALError code, const std::string& msg)
{
    g_err = code;
    snprintf(g_msg, sizeof(g_msg), "%s", msg.c_str());
    static const char* verbose = getenv("OPENCAL_VERBOSE_ERRORS");
    if (code != CAL_SUCCESS && (verbose == nullptr || verbose[0] != '0'))
        fprintf(stderr, "opencal-gb300: %s\n", g_msg);
    const char* ab = getenv("OPENCAL_ABORT_ON_ERROR");
    if (code != CAL_SUCCESS && ab && ab[0] == '1')
        abort();
}

bool cuda_ok(cudaError_t e, const char* what)
{
    if (e == cudaSuccess)
        return true;
    set_error(CAL_ERROR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

/* ======================= kernels ======================================== */

static const int kThreads = 256;

static int grid_for(long long work)
{
    long long b = (work + kThreads - 1) / kThreads;
    const long long cap = 152LL * 8;
    if (b < 1)
        b = 1;
    return (int)(b < cap ? b : cap);
}

/* every cell, or the listed cells when the list is non-empty */
template <typename T>
__global__ void k_fill(T* buf, T v, long long n, const int* lin, const int* count, int at_active)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int listed = at_active ? *count : 0;
    if (listed > 0) {
        for (long long c = t; c < listed; c += stride)
            buf[lin[c]] = v;
    } else {
        for (long long c = t; c < n; c += stride)
            buf[c] = v;
    }
}

#define CAL_UPDATE_MAX (CAL_NTYPES * CAL_MAX_SUBSTATES_CORE)

struct UpdateParams {
    const void* src[CAL_UPDATE_MAX];
    void* dst[CAL_UPDATE_MAX];
    unsigned char elem[CAL_UPDATE_MAX];
    unsigned char type[CAL_UPDATE_MAX];
    unsigned char slot[CAL_UPDATE_MAX];
    int n_entries;
    long long ncells;
    const unsigned* dirty;
    unsigned forced[CAL_NTYPES];
    int use_dirty;
    int at_active;
    const int* lin;
    const int* count;
};

/* next -> current of the selected substates.  Whole-grid copies move 16-byte
 * vectors (device buffers are 256-byte aligned); active-cell copies move one
 * element per listed cell (calCopyActiveCellsBuffer2D*). */
__global__ void k_update(const __grid_constant__ UpdateParams p)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int listed = p.at_active ? *p.count : 0;
    for (int e = 0; e < p.n_entries; e++) {
        if (p.use_dirty && !(((p.dirty[p.type[e]] | p.forced[p.type[e]]) >> p.slot[e]) & 1u))
            continue;
        const int es = p.elem[e];
        if (listed > 0) {
            for (long long c = t0; c < listed; c += stride) {
                const long long o = (long long)__ldg(p.lin + c);
                if (es == 8)
                    ((unsigned long long*)p.dst[e])[o] = __ldg((const unsigned long long*)p.src[e] + o);
                else if (es == 4)
                    ((unsigned*)p.dst[e])[o] = __ldg((const unsigned*)p.src[e] + o);
                else
                    ((unsigned char*)p.dst[e])[o] = __ldg((const unsigned char*)p.src[e] + o);
            }
        } else {
            const long long bytes = p.ncells * es;
            const long long vecs = bytes >> 4;
            const uint4* s = (const uint4*)p.src[e];
            uint4* d = (uint4*)p.dst[e];
            for (long long c = t0; c < vecs; c += stride)
                d[c] = s[c];
            for (long long c = (vecs << 4) + t0; c < bytes; c += stride)
                ((unsigned char*)p.dst[e])[c] = ((const unsigned char*)p.src[e])[c];
        }
    }
}

/* ---- change tracking: tile-sparse update and fill ----------------------
 * A tile is CAL_TILE_W x CAL_TILE_H cells (the process kernels' tiles);
 * tile index = tile row * tiles_x + tile column; one bit per tile. */
struct TileGeom {
    int rows, cols, tiles_x, tile_words, ntiles;
    int toroidal;
    unsigned* run; /* must-run bitmaps of the processes (NULL: no skipping) */
    int nrun;
};

/* tile `tile`'s current layer changed: every process must run again on it
 * and on the eight tiles around it (wrapping on toroidal grids); thread k <
 * 9 of the caller takes neighbour k */
static __device__ __forceinline__ void mark_run(const TileGeom& g, int tile, int k)
{
    if (!g.run || k >= 9)
        return;
    const int tiles_y = g.ntiles / g.tiles_x;
    const int ty = tile / g.tiles_x, tx = tile - ty * g.tiles_x;
    int y = ty + k / 3 - 1, x = tx + k % 3 - 1;
    if (g.toroidal) {
        y = y < 0 ? y + tiles_y : (y >= tiles_y ? y - tiles_y : y);
        x = x < 0 ? x + g.tiles_x : (x >= g.tiles_x ? x - g.tiles_x : x);
    } else if (y < 0 || y >= tiles_y || x < 0 || x >= g.tiles_x) {
        return;
    }
    const int t = y * g.tiles_x + x;
    for (int p = 0; p < g.nrun; p++)
        atomicOr(&g.run[(long long)p * g.tile_words + (t >> 5)], 1u << (t & 31));
}

/* the cells of `tile`, one per thread of a 256-thread block */
static __device__ __forceinline__ bool tile_cell(const TileGeom& g, int tile, long long* c)
{
    const int ty = tile / g.tiles_x;
    const int i = ty * CAL_TILE_H + (int)(threadIdx.x >> 5);
    const int j = (tile - ty * g.tiles_x) * CAL_TILE_W + (int)(threadIdx.x & 31);
    *c = (long long)i * g.cols + j;
    return i < g.rows && j < g.cols;
}

template <typename T>
static __device__ __forceinline__ void copy_tile(const TileGeom& g, int tile, const void* src, void* dst)
{
    long long c;
    if (tile_cell(g, tile, &c))
        static_cast<T*>(dst)[c] = static_cast<const T*>(src)[c];
}

struct TileUpdateParams {
    const void* src[CAL_UPDATE_MAX];
    void* dst[CAL_UPDATE_MAX];
    unsigned char elem[CAL_UPDATE_MAX];
    unsigned char type[CAL_UPDATE_MAX];
    unsigned char slot[CAL_UPDATE_MAX];
    int n_entries;
    TileGeom g;
    const unsigned* dirty;
    unsigned forced[CAL_NTYPES];
    int use_dirty;
    unsigned* chg;
    unsigned* dev;
    unsigned* untracked; /* [3] per type, [3] the ticket */
};

/* next -> current of the tracked substates, tile by tile: the tiles whose
 * chg bit is set (every tile of a substate written by unsafe operations);
 * the copied tiles' bits move from chg to dev.  Work items are (entry,
 * bitmap word), grid-stride; the last block to finish clears the unsafe
 * marks (a ticket, reset by that block). */
__global__ void __launch_bounds__(kThreads) k_update_tiles(const __grid_constant__ TileUpdateParams p)
{
    __shared__ unsigned s_bits;
    __shared__ int s_last;
    const int items = p.n_entries * p.g.tile_words;
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int e = item / p.g.tile_words, w = item - e * p.g.tile_words;
        const int t = p.type[e], sl = p.slot[e];
        if (p.use_dirty && !(((p.dirty[t] | p.forced[t]) >> sl) & 1u))
            continue;
        const long long row = (long long)(t * CAL_MAX_SUBSTATES_CORE + sl) * p.g.tile_words;
        if (threadIdx.x == 0) {
            unsigned b = p.chg[row + w];
            if ((p.untracked[t] >> sl) & 1u) {
                const int left = p.g.ntiles - w * 32;
                b = left >= 32 ? 0xffffffffu : ((1u << left) - 1u);
            }
            s_bits = b;
        }
        __syncthreads();
        unsigned bits = s_bits;
        while (bits) {
            const int tile = w * 32 + __ffs(bits) - 1;
            bits &= bits - 1;
            switch (p.elem[e]) {
            case 8: copy_tile<unsigned long long>(p.g, tile, p.src[e], p.dst[e]); break;
            case 4: copy_tile<unsigned>(p.g, tile, p.src[e], p.dst[e]); break;
            default: copy_tile<unsigned char>(p.g, tile, p.src[e], p.dst[e]); break;
            }
            mark_run(p.g, tile, threadIdx.x);
        }
        if (threadIdx.x == 0 && s_bits) {
            p.chg[row + w] = 0;
            p.dev[row + w] |= s_bits;
        }
        __syncthreads(); /* s_bits is reused */
    }
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(p.untracked + 3, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x < 4)
        p.untracked[threadIdx.x] = 0; /* the unsafe marks (read by every block) and the ticket */
}

/* both layers of one substate to `value` on the tiles of dev | chg, whose
 * bits are then cleared (the layers are equal and uniform again) */
template <typename T>
__global__ void __launch_bounds__(kThreads) k_fill_tiles(TileGeom g, T* l0, T* l1, T value, unsigned* chg,
                                                          unsigned* dev)
{
    __shared__ unsigned s_bits;
    for (int w = blockIdx.x; w < g.tile_words; w += gridDim.x) {
        if (threadIdx.x == 0)
            s_bits = chg[w] | dev[w];
        __syncthreads();
        unsigned bits = s_bits;
        while (bits) {
            const int tile = w * 32 + __ffs(bits) - 1;
            bits &= bits - 1;
            long long c;
            if (tile_cell(g, tile, &c)) {
                l0[c] = value;
                if (l1)
                    l1[c] = value;
            }
            mark_run(g, tile, threadIdx.x);
        }
        if (threadIdx.x == 0 && s_bits) {
            chg[w] = 0;
            dev[w] = 0;
        }
        __syncthreads();
    }
}

/* ---- active-cell compaction -------------------------------------------
 * The list order is the reference's:
 *   2D: memory order (row-major);
 *   3D: i, then j, then k, while memory is slice-major (k*rows*cols + ...).
 * Positions v = 0 .. n-1 of that order are cut into chunks of kChunk per
 * block and kWarpSpan per warp; a warp takes kRounds rounds of 32
 * consecutive positions, one per lane, and sees each round's flags as one
 * __ballot_sync word.
 *   Pass 1 (k_compact_count): every warp counts its set flags (__popc of the
 *   ballots), the block sums its warps and stores its count; the last block
 *   to finish (a ticket) turns the counts into exclusive offsets in place (a
 *   block-wide prefix scan), writes the total to *count and puts the ticket
 *   back to 0 for the next call.
 *   Pass 2 (k_compact_scatter): every block reads its offset, scans its
 *   warps' counts, and each warp writes its cells round by round: a lane's
 *   slot is the running offset plus the set lanes below it in the round's
 *   ballot, so the list comes out in order with coalesced stores.
 * Scratch (compact_scratch_ints): kScratchHead ints holding the ticket on a
 * 128-byte line of its own, then one int per block.  Flags are read one
 * byte per lane, so the flags pointer needs no alignment; cells, lin and
 * count need 4-byte alignment. */
static const int kRounds = 16;
static const int kWarpSpan = 32 * kRounds;                 /* 512 positions per warp */
static const int kChunk = (kThreads / 32) * kWarpSpan;     /* 4096 positions per block */
static const int kScratchHead = 32;                        /* ticket line */

struct CompactGeom {
    int dim, rows, cols, slices;
    long long n;
    /* non-NULL: a word that the process kernels set when they changed a
     * flag; while it is 0 the list of the previous compaction (still in
     * cells, lin, count and the block offsets in scratch) is the answer and
     * both passes keep it.  The count pass's last block records its decision
     * in scratch[1] for the scatter pass and clears the word. */
    unsigned* dirty;
};

static __device__ __forceinline__ long long order_to_mem(const CompactGeom& g, long long v)
{
    if (g.dim == 2)
        return v;
    const long long k = v % g.slices;
    const long long ij = v / g.slices; /* i*cols + j */
    return k * (long long)g.rows * g.cols + ij;
}

static __device__ __forceinline__ bool flag_at(const unsigned char* __restrict__ flags, const CompactGeom& g,
                                               long long v)
{
    return v < g.n && flags[order_to_mem(g, v)] != 0;
}

/* exclusive prefix sums of a[0..n) in place by one block; the total goes to
 * *total.  Each thread owns a contiguous segment, so the result is in order. */
static __device__ void block_exclusive_scan(int* a, int n, int* total)
{
    __shared__ int s_warp[kThreads / 32];
    const int per = (n + kThreads - 1) / kThreads;
    const int lo = threadIdx.x * per;
    const int hi = min(lo + per, n);
    int sum = 0;
    for (int b = lo; b < hi; b++)
        sum += __ldcg(a + b);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o)
            incl += y;
    }
    if (lane == 31)
        s_warp[warp] = incl;
    __syncthreads();
    int run = incl - sum;
    for (int w = 0; w < warp; w++)
        run += s_warp[w];
    for (int b = lo; b < hi; b++) {
        const int c = __ldcg(a + b);
        a[b] = run;
        run += c;
    }
    if (threadIdx.x == kThreads - 1)
        *total = run;
}

__global__ void __launch_bounds__(kThreads) k_compact_count(const unsigned char* __restrict__ flags, CompactGeom g,
                                                              int* scratch, int* count)
{
    __shared__ int s_warp[kThreads / 32];
    __shared__ int s_last, s_go;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0)
        s_go = g.dirty ? (*(volatile const unsigned*)g.dirty != 0) : 1; /* the same for every block */
    __syncthreads();
    const int go = s_go;
    if (go) {
        const long long base = (long long)blockIdx.x * kChunk + (long long)warp * kWarpSpan + lane;
        int c = 0;
#pragma unroll
        for (int q = 0; q < kRounds; q++)
            c += __popc(__ballot_sync(0xffffffffu, flag_at(flags, g, base + 32 * q)));
        if (lane == 0)
            s_warp[warp] = c;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (go) {
            int s = 0;
            for (int w = 0; w < kThreads / 32; w++)
                s += s_warp[w];
            scratch[kScratchHead + blockIdx.x] = s;
        }
        __threadfence(); /* the count is visible before the ticket is taken */
        s_last = atomicAdd(reinterpret_cast<unsigned*>(scratch), 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last)
        return;
    __threadfence();
    if (go)
        block_exclusive_scan(scratch + kScratchHead, gridDim.x, count);
    if (threadIdx.x == 0) {
        scratch[1] = go;      /* the scatter pass's decision */
        if (g.dirty)
            *g.dirty = 0;     /* every block has read it */
        scratch[0] = 0;       /* every ticket of this call has been taken */
    }
}

/* next -> current at the listed cells, fused into the scatter pass of the
 * compaction that lists them (CalGrid::update_all with active cells): the
 * substates to copy, and the list's length (an empty list copies every
 * cell, calUpdateSubstate2D* in cal2D.c) */
struct ActiveCopy {
    const void* src[CAL_UPDATE_MAX];
    void* dst[CAL_UPDATE_MAX];
    unsigned char elem[CAL_UPDATE_MAX];
    int n;
    const int* count;
};

/* next -> current of substate e at cell o; next is not written during the
 * kernel, so it is read through the non-coherent path and the loads of
 * successive calls can be in flight together */
static __device__ __forceinline__ void copy_elem(const ActiveCopy& u, int e, long long o)
{
    const int es = u.elem[e];
    if (es == 8)
        ((unsigned long long*)u.dst[e])[o] = __ldg((const unsigned long long*)u.src[e] + o);
    else if (es == 4)
        ((unsigned*)u.dst[e])[o] = __ldg((const unsigned*)u.src[e] + o);
    else
        ((unsigned char*)u.dst[e])[o] = __ldg((const unsigned char*)u.src[e] + o);
}

template <bool UPD>
static __device__ __forceinline__ void compact_scatter(const unsigned char* __restrict__ flags, const CompactGeom& g,
                                                       const int* __restrict__ scratch, int* cells, int* lin,
                                                       const ActiveCopy* u)
{
    __shared__ int s_warp[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long base = (long long)blockIdx.x * kChunk + (long long)warp * kWarpSpan;
    unsigned m[kRounds];
    int c = 0;
#pragma unroll
    for (int q = 0; q < kRounds; q++) {
        m[q] = __ballot_sync(0xffffffffu, flag_at(flags, g, base + 32 * q + lane));
        c += __popc(m[q]);
    }
    if (lane == 0)
        s_warp[warp] = c;
    __syncthreads();
    int pos = scratch[kScratchHead + blockIdx.x];
    for (int w = 0; w < warp; w++)
        pos += s_warp[w];
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int q = 0; q < kRounds; q++) {
        if ((m[q] >> lane) & 1u) {
            const long long v = base + 32 * q + lane;
            const int slot = pos + __popc(m[q] & below);
            const long long mem = order_to_mem(g, v);
            if (g.dim == 2) {
                const unsigned i = (unsigned)v / (unsigned)g.cols;
                cells[2 * slot] = (int)i;
                cells[2 * slot + 1] = (int)((unsigned)v - i * (unsigned)g.cols);
            } else {
                const unsigned ij = (unsigned)v / (unsigned)g.slices;
                const unsigned i = ij / (unsigned)g.cols;
                cells[3 * slot] = (int)i;
                cells[3 * slot + 1] = (int)(ij - i * (unsigned)g.cols);
                cells[3 * slot + 2] = (int)((unsigned)v - ij * (unsigned)g.slices);
            }
            lin[slot] = (int)mem;
        }
        pos += __popc(m[q]);
    }
    if (UPD) {
        /* the block's listed cells, slots [first, pos of the last warp),
         * one per thread, substate by substate */
        __shared__ int s_range[2];
        if (threadIdx.x == kThreads - 1) {
            s_range[0] = scratch[kScratchHead + blockIdx.x];
            s_range[1] = pos; /* the last warp's end: the block's end */
        }
        __syncthreads(); /* this block's lin[] entries are visible to it */
        const int first = s_range[0], last = s_range[1];
        for (int e = 0; e < u->n; e++)
            for (int k = first + threadIdx.x; k < last; k += kThreads)
                copy_elem(*u, e, lin[k]);
    }
}

__global__ void __launch_bounds__(kThreads) k_compact_scatter(const unsigned char* __restrict__ flags, CompactGeom g,
                                                                const int* __restrict__ scratch, int* cells, int* lin)
{
    if (scratch[1])
        compact_scatter<false>(flags, g, scratch, cells, lin, nullptr);
}

__global__ void __launch_bounds__(kThreads) k_compact_scatter_update(const unsigned char* __restrict__ flags,
                                                                       CompactGeom g, const int* __restrict__ scratch,
                                                                       int* cells, int* lin,
                                                                       const __grid_constant__ ActiveCopy u)
{
    const int listed = *u.count;
    if (listed > 0 && scratch[1]) {
        compact_scatter<true>(flags, g, scratch, cells, lin, &u);
        return;
    }
    if (listed > 0) {
        /* the flags did not change: the previous list, this block's slots */
        const int first = scratch[kScratchHead + blockIdx.x];
        const int last = blockIdx.x + 1 < gridDim.x ? scratch[kScratchHead + blockIdx.x + 1] : listed;
        for (int e = 0; e < u.n; e++)
            for (int k = first + threadIdx.x; k < last; k += kThreads)
                copy_elem(u, e, lin[k]);
        return;
    }
    /* no active cell: every cell of this block's range (linear memory) */
    const long long lo = (long long)blockIdx.x * kChunk;
    const long long hi = lo + kChunk < g.n ? lo + kChunk : g.n;
    for (int e = 0; e < u.n; e++)
        for (long long c = lo + threadIdx.x; c < hi; c += kThreads)
            copy_elem(u, e, c);
}

int compact_blocks_needed(long long ncells)
{
    return (int)((ncells + kChunk - 1) / kChunk);
}

long long compact_scratch_ints(long long ncells)
{
    return kScratchHead + (long long)compact_blocks_needed(ncells);
}

cudaError_t compact_flags(const unsigned char* flags, int dim, int rows, int cols, int slices, int* cells, int* lin,
                          int* count, int* scratch, long long scratch_ints, cudaStream_t stream, unsigned* dirty)
{
    CompactGeom g;
    g.dirty = dirty;
    g.dim = dim;
    g.rows = rows;
    g.cols = cols;
    g.slices = dim == 3 ? slices : 1;
    g.n = (long long)rows * cols * g.slices;
    if (g.n <= 0 || g.n > 0x7fffffffLL || scratch_ints < compact_scratch_ints(g.n))
        return cudaErrorInvalidValue;
    const int nb = compact_blocks_needed(g.n);
    k_compact_count<<<nb, kThreads, 0, stream>>>(flags, g, scratch, count);
    k_compact_scatter<<<nb, kThreads, 0, stream>>>(flags, g, scratch, cells, lin);
    return cudaGetLastError();
}

/* the compaction, then next -> current of the listed substates at the new
 * list's cells (every cell when the list is empty) in its scatter pass */
static cudaError_t compact_and_copy(const unsigned char* flags, int dim, int rows, int cols, int slices, int* cells,
                                    int* lin, int* count, int* scratch, long long scratch_ints, const ActiveCopy& u,
                                    cudaStream_t stream, unsigned* dirty)
{
    CompactGeom g;
    g.dirty = dirty;
    g.dim = dim;
    g.rows = rows;
    g.cols = cols;
    g.slices = dim == 3 ? slices : 1;
    g.n = (long long)rows * cols * g.slices;
    if (g.n <= 0 || g.n > 0x7fffffffLL || scratch_ints < compact_scratch_ints(g.n))
        return cudaErrorInvalidValue;
    const int nb = compact_blocks_needed(g.n);
    k_compact_count<<<nb, kThreads, 0, stream>>>(flags, g, scratch, count);
    k_compact_scatter_update<<<nb, kThreads, 0, stream>>>(flags, g, scratch, cells, lin, u);
    return cudaGetLastError();
}

/* ======================= CalGrid ======================================== */

static size_t type_size(int t)
{
    return t == 0 ? sizeof(CALbyte) : (t == 1 ? sizeof(CALint) : sizeof(CALreal));
}

bool CalGrid::init(int dim_, int rows_, int cols_, int slices_, int toroidal_, int active_)
{
    dim = dim_;
    rows = rows_;
    cols = cols_;
    slices = dim == 3 ? slices_ : 1;
    toroidal = toroidal_;
    active = active_;
    ncells = (long long)rows * cols * slices;
    if (rows <= 0 || cols <= 0 || slices <= 0 || ncells > 0x7fffffffLL) {
        set_error(CAL_ERROR_INVALID_ARGUMENT, "grid dimensions must be positive and hold < 2^31 cells");
        return false;
    }
    if (!cuda_ok(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate"))
        return false;
    for (int t = 0; t < CAL_NTYPES; t++) {
        /* handle pool: one 32-byte record per slot, addresses stable */
        pool[t] = calloc(CAL_MAX_SUBSTATES_CORE, 32);
        if (!pool[t]) {
            set_error(CAL_ERROR_OUT_OF_MEMORY, "handle pool");
            return false;
        }
    }
    if (!cuda_ok(cudaMalloc(&d_dirty, 4 * sizeof(unsigned)), "cudaMalloc dirty") ||
        !cuda_ok(cudaMemsetAsync(d_dirty, 0, 4 * sizeof(unsigned), stream), "memset dirty"))
        return false;
    if (!cuda_ok(cudaMalloc(&d_step, 2 * sizeof(int)), "cudaMalloc step") ||
        !cuda_ok(cudaMemsetAsync(d_step, 0, 2 * sizeof(int), stream), "memset step"))
        return false;
    if (!cuda_ok(cudaMalloc(&d_count, sizeof(int)), "cudaMalloc count") ||
        !cuda_ok(cudaMemsetAsync(d_count, 0, sizeof(int), stream), "memset count"))
        return false;
    /* reduction scratch (512 per-block partials of up to 8 bytes, plus the
     * result word), allocated here so that a reduction queued while a step
     * is being recorded as a graph never has to allocate */
    if (!cuda_ok(cudaMalloc(&d_reduce_partial, 512 * sizeof(double) + 64), "cudaMalloc reduction") ||
        !cuda_ok(cudaMalloc(&d_reduce_result, 64), "cudaMalloc reduction result"))
        return false;
    /* change tracking for 2D models without active cells (every substate
     * starts zero in both layers: equal and uniform) */
    tracking = dim == 2 && !active;
    if (tracking) {
        tiles_x = (cols + CAL_TILE_W - 1) / CAL_TILE_W;
        tiles_y = (rows + CAL_TILE_H - 1) / CAL_TILE_H;
        tile_words = (int)(((long long)tiles_x * tiles_y + 31) / 32);
        const size_t bm = (size_t)CAL_NTYPES * CAL_MAX_SUBSTATES_CORE * tile_words * sizeof(unsigned);
        if (!cuda_ok(cudaMalloc(&d_chg, bm), "cudaMalloc change bitmaps") ||
            !cuda_ok(cudaMalloc(&d_dev, bm), "cudaMalloc change bitmaps") ||
            !cuda_ok(cudaMalloc(&d_untracked, 4 * sizeof(unsigned)), "cudaMalloc change bitmaps") ||
            !cuda_ok(cudaMemsetAsync(d_chg, 0, bm, stream), "memset change bitmaps") ||
            !cuda_ok(cudaMemsetAsync(d_dev, 0, bm, stream), "memset change bitmaps") ||
            !cuda_ok(cudaMemsetAsync(d_untracked, 0, 4 * sizeof(unsigned), stream), "memset change bitmaps") ||
            !cuda_ok(cudaMalloc(&d_run, (size_t)CAL_MAX_PROCESSES_CORE * tile_words * sizeof(unsigned)),
                     "cudaMalloc skipping bitmaps") ||
            !cuda_ok(cudaMalloc(&d_quiet, (size_t)(tile_words + 32) * sizeof(unsigned)), "cudaMalloc skipping bitmaps") ||
            !cuda_ok(cudaMemsetAsync(d_quiet, 0, (size_t)(tile_words + 32) * sizeof(unsigned), stream),
                     "memset skipping bitmaps") ||
            !arm_runs())
            return false;
        d_ticket = d_quiet + tile_words + 16; /* a line of its own past the bitmap */
    }
    if (active) {
        scratch_ints = compact_scratch_ints(ncells);
        if (!cuda_ok(cudaMalloc(&d_flags, (size_t)ncells), "cudaMalloc flags") ||
            !cuda_ok(cudaMalloc(&d_cells, (size_t)ncells * dim * sizeof(int)), "cudaMalloc cells") ||
            !cuda_ok(cudaMalloc(&d_lin, (size_t)ncells * sizeof(int)), "cudaMalloc lin") ||
            !cuda_ok(cudaMalloc(&d_block_counts, (size_t)scratch_ints * sizeof(int)), "cudaMalloc scratch") ||
            !cuda_ok(cudaMemsetAsync(d_block_counts, 0, (size_t)scratch_ints * sizeof(int), stream),
                     "memset scratch") ||
            !cuda_ok(cudaMemsetAsync(d_flags, 0, (size_t)ncells, stream), "memset flags"))
            return false;
        if (dim == 2 && (!cuda_ok(cudaMalloc(&d_flags_dirty, sizeof(unsigned)), "cudaMalloc flags word") ||
                         !cuda_ok(cudaMemsetAsync(d_flags_dirty, 0xff, sizeof(unsigned), stream), "set flags word")))
            return false;
        if (!cuda_ok(cudaMallocHost(&h_flags, (size_t)ncells), "cudaMallocHost flags"))
            return false;
        memset(h_flags, 0, (size_t)ncells);
    }
    return true;
}

void CalGrid::destroy()
{
    if (stream)
        cudaStreamSynchronize(stream);
    for (int t = 0; t < CAL_NTYPES; t++) {
        for (int s = 0; s < nslot[t]; s++) {
            Sub& q = sub[t][s];
            for (int l = 0; l < 2; l++) {
                if (q.layer[l].dev)
                    cudaFree(q.layer[l].dev);
                if (q.host[l])
                    cudaFreeHost(q.host[l]);
            }
        }
        free(pool[t]);
        pool[t] = nullptr;
    }
    cudaFree(d_flags);
    cudaFree(d_flags_dirty);
    cudaFree(d_cells);
    cudaFree(d_lin);
    cudaFree(d_count);
    cudaFree(d_block_counts);
    cudaFree(d_dirty);
    cudaFree(d_chg);
    cudaFree(d_dev);
    cudaFree(d_untracked);
    cudaFree(d_run);
    cudaFree(d_quiet);
    cudaFree(d_step);
    cudaFree(d_reduce_partial);
    cudaFree(d_reduce_result);
    if (h_flags)
        cudaFreeHost(h_flags);
    if (stream)
        cudaStreamDestroy(stream);
    stream = nullptr;
}

int CalGrid::add_sub(int type, bool single, void** cur_mirror, void** next_mirror)
{
    if (nslot[type] >= CAL_MAX_SUBSTATES_CORE) {
        set_error(CAL_ERROR_LIMIT, "too many substates of one type (limit 32)");
        return -1;
    }
    const int slot = nslot[type];
    Sub& q = sub[type][slot];
    q.used = true;
    q.single = single;
    q.type = type;
    q.elem = type_size(type);
    const size_t bytes = (size_t)ncells * q.elem;
    const int layers = single ? 1 : 2;
    for (int l = 0; l < layers; l++) {
        if (!cuda_ok(cudaMalloc(&q.layer[l].dev, bytes), "cudaMalloc substate"))
            return -1;
        if (!cuda_ok(cudaMemsetAsync(q.layer[l].dev, 0, bytes, stream), "memset substate"))
            return -1;
        if (!cuda_ok(cudaMallocHost(&q.host[l], bytes), "cudaMallocHost substate mirror"))
            return -1;
        memset(q.host[l], 0, bytes);
        q.layer[l].host_valid = true;
        q.layer[l].dev_valid = true;
    }
    *cur_mirror = q.host[0];
    *next_mirror = single ? nullptr : q.host[1];
    nslot[type]++;
    return slot;
}

/* ---- coherence ---------------------------------------------------------- */

bool CalGrid::to_device_all()
{
    for (int t = 0; t < CAL_NTYPES; t++)
        for (int s = 0; s < nslot[t]; s++) {
            Sub& q = sub[t][s];
            for (int l = 0; l < (q.single ? 1 : 2); l++) {
                if (q.layer[l].dev_valid)
                    continue;
                if (capturing) {
                    set_error(CAL_ERROR_NOT_CAPTURABLE, "host data must be uploaded during graph capture");
                    return false;
                }
                if (!cuda_ok(cudaMemcpyAsync(q.layer[l].dev, q.host[l], (size_t)ncells * q.elem,
                                             cudaMemcpyHostToDevice, stream), "upload substate"))
                    return false;
                q.layer[l].dev_valid = true;
                transfers++;
            }
        }
    if (active && !flags_dev_valid) {
        if (capturing) {
            set_error(CAL_ERROR_NOT_CAPTURABLE, "active flags must be uploaded during graph capture");
            return false;
        }
        if (!cuda_ok(cudaMemcpyAsync(d_flags, h_flags, (size_t)ncells, cudaMemcpyHostToDevice, stream),
                     "upload flags"))
            return false;
        if (d_flags_dirty &&
            !cuda_ok(cudaMemsetAsync(d_flags_dirty, 0xff, sizeof(unsigned), stream), "set flags word"))
            return false;
        flags_dev_valid = true;
        transfers++;
    }
    return true;
}

bool CalGrid::to_host(int type, int slot, int layer)
{
    Sub& q = sub[type][slot];
    if (q.layer[layer].host_valid)
        return true;
    if (capturing) {
        set_error(CAL_ERROR_NOT_CAPTURABLE, "host read of device data during graph capture");
        return false;
    }
    if (layer == 1 && q.next_stale && !repair_stale(type, slot))
        return false;
    if (!cuda_ok(cudaMemcpyAsync(q.host[layer], q.layer[layer].dev, (size_t)ncells * q.elem,
                                 cudaMemcpyDeviceToHost, stream), "download substate") ||
        !cuda_ok(cudaStreamSynchronize(stream), "sync"))
        return false;
    q.layer[layer].host_valid = true;
    transfers++;
    return true;
}

bool CalGrid::flags_to_host()
{
    if (!active || flags_host_valid)
        return true;
    if (capturing) {
        set_error(CAL_ERROR_NOT_CAPTURABLE, "host read of active flags during graph capture");
        return false;
    }
    if (!cuda_ok(cudaMemcpyAsync(h_flags, d_flags, (size_t)ncells, cudaMemcpyDeviceToHost, stream), "download flags") ||
        !cuda_ok(cudaStreamSynchronize(stream), "sync"))
        return false;
    flags_host_valid = true;
    transfers++;
    return true;
}

/* the caller's array (rows*cols[*slices] elements) becomes both layers of
 * a substate on the device: one host-to-device copy into the current
 * layer, one device copy into the next; the host mirrors become stale.
 * From pinned host memory the copy is asynchronous on the model's stream. */
bool CalGrid::load_from_host(int type, int slot, const void* src)
{
    Sub& q = sub[type][slot];
    if (!q.used) {
        set_error(CAL_ERROR_INVALID_ARGUMENT, "copy from host: not a substate of this model");
        return false;
    }
    if (capturing) {
        set_error(CAL_ERROR_NOT_CAPTURABLE, "host copy during graph capture");
        return false;
    }
    const size_t bytes = (size_t)ncells * q.elem;
    /* cudaMemcpyDefault: the caller's array may be in host or device memory */
    if (!cuda_ok(cudaMemcpyAsync(q.layer[0].dev, src, bytes, cudaMemcpyDefault, stream), "copy from host"))
        return false;
    q.layer[0].dev_valid = true;
    q.layer[0].host_valid = false;
    if (!q.single) {
        if (!cuda_ok(cudaMemcpyAsync(q.layer[1].dev, q.layer[0].dev, bytes, cudaMemcpyDeviceToDevice, stream),
                     "copy current to next"))
            return false;
        q.layer[1].dev_valid = true;
        q.layer[1].host_valid = false;
        q.next_stale = false;
    }
    q.forced_dirty = false;
    q.uval_valid = false;
    inval_epoch++;
    if (tracking && !q.single) {
        /* both layers are equal: no tile differs */
        const size_t row = (size_t)(type * CAL_MAX_SUBSTATES_CORE + slot) * tile_words;
        if (!cuda_ok(cudaMemsetAsync(d_chg + row, 0, tile_words * sizeof(unsigned), stream), "clear change bits"))
            return false;
        q.track = true;
    }
    return true;
}

/* the current layer into the caller's array (from the host mirror when it
 * is up to date, else straight from the device); synchronises */
bool CalGrid::store_to_host(int type, int slot, void* dst)
{
    Sub& q = sub[type][slot];
    if (!q.used) {
        set_error(CAL_ERROR_INVALID_ARGUMENT, "copy to host: not a substate of this model");
        return false;
    }
    if (capturing) {
        set_error(CAL_ERROR_NOT_CAPTURABLE, "host copy during graph capture");
        return false;
    }
    const size_t bytes = (size_t)ncells * q.elem;
    /* cudaMemcpyDefault: the caller's array may be in host or device memory */
    const void* from = q.layer[0].host_valid ? q.host[0] : q.layer[0].dev;
    return cuda_ok(cudaMemcpyAsync(dst, from, bytes, cudaMemcpyDefault, stream), "copy to host") &&
           cuda_ok(cudaStreamSynchronize(stream), "sync");
}

void CalGrid::host_wrote(int type, int slot, int layer)
{
    Sub& q = sub[type][slot];
    q.layer[layer].dev_valid = false;
    q.forced_dirty = true; /* the next update copies the whole substate, after which tracking resumes */
    q.track = false;
    q.uval_valid = false;
    inval_epoch++;
}

void CalGrid::untrack(int type, int slot)
{
    if (sub[type][slot].trackable) {
        sub[type][slot].trackable = false;
        inval_epoch++;
    }
}

void CalGrid::device_wrote_all()
{
    written_since_update = true;
    for (int t = 0; t < CAL_NTYPES; t++)
        for (int s = 0; s < nslot[t]; s++) {
            sub[t][s].layer[0].host_valid = false;
            sub[t][s].layer[1].host_valid = false;
        }
    if (active)
        flags_host_valid = false;
}

bool CalGrid::repair_stale(int type, int slot)
{
    Sub& q = sub[type][slot];
    if (!q.next_stale)
        return true;
    if (!cuda_ok(cudaMemcpyAsync(q.layer[1].dev, q.layer[0].dev, (size_t)ncells * q.elem, cudaMemcpyDeviceToDevice,
                                 stream), "repair next layer"))
        return false;
    q.next_stale = false;
    q.layer[1].host_valid = false;
    q.layer[1].dev_valid = true;
    return true;
}

bool CalGrid::repair_all_stale()
{
    for (int t = 0; t < CAL_NTYPES; t++)
        for (int s = 0; s < nslot[t]; s++)
            if (!repair_stale(t, s))
                return false;
    return true;
}

/* ---- device operations ----------------------------------------------- */

bool CalGrid::fill(int type, int slot, int layer, const void* value, bool at_active)
{
    Sub& q = sub[type][slot];
    if (!q.used || (layer == 1 && q.single))
        return true;
    if (layer == 1 && !repair_stale(type, slot))
        return false;
    if (!to_device_all())
        return false;
    const int use = (at_active && active) ? 1 : 0;
    const int g = grid_for(ncells);
    void* buf = q.layer[layer].dev;
    switch (type) {
    case 0: k_fill<CALbyte><<<g, kThreads, 0, stream>>>((CALbyte*)buf, *(const CALbyte*)value, ncells, d_lin, d_count, use); break;
    case 1: k_fill<CALint><<<g, kThreads, 0, stream>>>((CALint*)buf, *(const CALint*)value, ncells, d_lin, d_count, use); break;
    default: k_fill<CALreal><<<g, kThreads, 0, stream>>>((CALreal*)buf, *(const CALreal*)value, ncells, d_lin, d_count, use); break;
    }
    if (!cuda_ok(cudaGetLastError(), "fill kernel") || !arm_runs())
        return false;
    q.layer[layer].host_valid = false;
    q.forced_dirty = true;
    q.track = false; /* one layer only: the layers differ; the next update copies the whole substate */
    q.uval_valid = false;
    if (tracking)
        inval_epoch++;
    return true;
}

/* calInitSubstate*: both layers.  With change tracking the layers stay
 * equal (no update copy is needed afterwards), and when the substate
 * already holds this value outside the tiles of its dev and chg bitmaps,
 * only those tiles are filled. */
bool CalGrid::fill_both(int type, int slot, const void* value)
{
    Sub& q = sub[type][slot];
    if (!tracking || !q.trackable || q.single || !q.used) {
        if (!fill(type, slot, 0, value, true))
            return false;
        return fill(type, slot, 1, value, true);
    }
    if (!repair_stale(type, slot) || !to_device_all())
        return false;
    unsigned long long v = 0;
    memcpy(&v, value, q.elem);
    const size_t row = (size_t)(type * CAL_MAX_SUBSTATES_CORE + slot) * tile_words;
    void* l0 = q.layer[0].dev;
    void* l1 = q.layer[1].dev;
    if (q.track && q.uval_valid && q.uval == v) {
        TileGeom tg;
        tg.rows = rows;
        tg.cols = cols;
        tg.tiles_x = tiles_x;
        tg.tile_words = tile_words;
        tg.ntiles = tiles_x * tiles_y;
        tg.toroidal = toroidal;
        tg.run = nrun > 0 ? d_run : nullptr;
        tg.nrun = nrun;
        const int g = tile_words < 152 * 8 ? tile_words : 152 * 8;
        switch (type) {
        case 0: k_fill_tiles<CALbyte><<<g, kThreads, 0, stream>>>(tg, (CALbyte*)l0, (CALbyte*)l1, *(const CALbyte*)value, d_chg + row, d_dev + row); break;
        case 1: k_fill_tiles<CALint><<<g, kThreads, 0, stream>>>(tg, (CALint*)l0, (CALint*)l1, *(const CALint*)value, d_chg + row, d_dev + row); break;
        default: k_fill_tiles<CALreal><<<g, kThreads, 0, stream>>>(tg, (CALreal*)l0, (CALreal*)l1, *(const CALreal*)value, d_chg + row, d_dev + row); break;
        }
        if (!cuda_ok(cudaGetLastError(), "tile fill kernel"))
            return false;
    } else {
        const int g = grid_for(ncells);
        for (int l = 0; l < 2; l++) {
            void* buf = q.layer[l].dev;
            switch (type) {
            case 0: k_fill<CALbyte><<<g, kThreads, 0, stream>>>((CALbyte*)buf, *(const CALbyte*)value, ncells, d_lin, d_count, 0); break;
            case 1: k_fill<CALint><<<g, kThreads, 0, stream>>>((CALint*)buf, *(const CALint*)value, ncells, d_lin, d_count, 0); break;
            default: k_fill<CALreal><<<g, kThreads, 0, stream>>>((CALreal*)buf, *(const CALreal*)value, ncells, d_lin, d_count, 0); break;
            }
        }
        if (!cuda_ok(cudaGetLastError(), "fill kernel") || !arm_runs() ||
            !cuda_ok(cudaMemsetAsync(d_chg + row, 0, tile_words * sizeof(unsigned), stream), "clear change bits") ||
            !cuda_ok(cudaMemsetAsync(d_dev + row, 0, tile_words * sizeof(unsigned), stream), "clear change bits"))
            return false;
        q.uval = v;
        q.uval_valid = true;
        q.track = true;
    }
    /* the layers are equal: whatever a process wrote into next before is gone */
    q.layer[0].host_valid = false;
    q.layer[1].host_valid = false;
    q.forced_dirty = false;
    return true;
}

bool CalGrid::copy_next_to_current(const std::vector<std::pair<int, int>>& which, bool use_dirty, bool at_active)
{
    /* tracked substates go tile by tile (k_update_tiles), the others whole
     * (k_update); a substate whose bitmap was not exact becomes tracked again
     * once its whole copy is queued */
    UpdateParams p;
    memset(&p, 0, sizeof(p));
    TileUpdateParams tp;
    memset(&tp, 0, sizeof(tp));
    std::vector<std::pair<int, int>> retrack;
    for (size_t w = 0; w < which.size(); w++) {
        const int t = which[w].first, sl = which[w].second;
        Sub& q = sub[t][sl];
        if (!q.used || q.single || q.next_stale)
            continue;
        const bool tiles = tracking && q.trackable && q.track;
        if (tiles) {
            const int e = tp.n_entries++;
            tp.src[e] = q.layer[1].dev;
            tp.dst[e] = q.layer[0].dev;
            tp.elem[e] = (unsigned char)q.elem;
            tp.type[e] = (unsigned char)t;
            tp.slot[e] = (unsigned char)sl;
            if (q.forced_dirty)
                tp.forced[t] |= 1u << sl;
            continue;
        }
        const int e = p.n_entries++;
        p.src[e] = q.layer[1].dev;
        p.dst[e] = q.layer[0].dev;
        p.elem[e] = (unsigned char)q.elem;
        p.type[e] = (unsigned char)t;
        p.slot[e] = (unsigned char)sl;
        if (q.forced_dirty)
            p.forced[t] |= 1u << sl;
        if (tracking && q.trackable)
            retrack.push_back(which[w]);
    }
    if (p.n_entries > 0) {
        p.ncells = ncells;
        p.dirty = d_dirty;
        p.use_dirty = use_dirty ? 1 : 0;
        p.at_active = (at_active && active) ? 1 : 0;
        p.lin = d_lin;
        p.count = d_count;
        const long long work = p.at_active ? ncells : (ncells * 8) / 16;
        k_update<<<grid_for(work), kThreads, 0, stream>>>(p);
        if (!cuda_ok(cudaGetLastError(), "update kernel"))
            return false;
        if (!arm_runs()) /* whole copies: no tile-by-tile record of what changed */
            return false;
        for (size_t r = 0; r < retrack.size(); r++) {
            /* copied whole only if written or forced: a substate that lost
             * its tracking was forced (host write, one-layer fill), so the
             * layers are equal after this copy */
            Sub& q = sub[retrack[r].first][retrack[r].second];
            if (!q.forced_dirty && use_dirty)
                continue;
            const size_t row = (size_t)(retrack[r].first * CAL_MAX_SUBSTATES_CORE + retrack[r].second) * tile_words;
            if (!cuda_ok(cudaMemsetAsync(d_chg + row, 0, tile_words * sizeof(unsigned), stream),
                         "clear change bits"))
                return false;
            q.track = true;
            q.uval_valid = false;
        }
    }
    if (tp.n_entries > 0) {
        tp.g.rows = rows;
        tp.g.cols = cols;
        tp.g.tiles_x = tiles_x;
        tp.g.tile_words = tile_words;
        tp.g.ntiles = tiles_x * tiles_y;
        tp.g.toroidal = toroidal;
        tp.g.run = nrun > 0 ? d_run : nullptr;
        tp.g.nrun = nrun;
        tp.dirty = d_dirty;
        tp.use_dirty = use_dirty ? 1 : 0;
        tp.chg = d_chg;
        tp.dev = d_dev;
        tp.untracked = d_untracked;
        const long long items = (long long)tp.n_entries * tile_words;
        const int g = (int)(items < 152 * 8 ? items : 152 * 8);
        k_update_tiles<<<g, kThreads, 0, stream>>>(tp);
        if (!cuda_ok(cudaGetLastError(), "tile update kernel"))
            return false;
    }
    for (size_t w = 0; w < which.size(); w++) {
        Sub& q = sub[which[w].first][which[w].second];
        if (!q.used || q.single || q.next_stale)
            continue;
        q.layer[0].host_valid = false;
        q.forced_dirty = false;
    }
    return true;
}

bool CalGrid::mark_flags_changed()
{
    return !d_flags_dirty ||
           cuda_ok(cudaMemsetAsync(d_flags_dirty, 0xff, sizeof(unsigned), stream), "set flags word");
}

/* calUpdateActiveCells2D: always a full compaction (flags may have been
 * written through the device pointer) */
bool CalGrid::compact()
{
    if (!active)
        return true;
    if (!to_device_all() || !mark_flags_changed())
        return false;
    return cuda_ok(compact_flags(d_flags, dim, rows, cols, slices, d_cells, d_lin, d_count, d_block_counts,
                                 scratch_ints, stream, flags_dirty_word()),
                   "active-cell compaction");
}

bool CalGrid::arm_runs()
{
    run_epoch = inval_epoch;
    if (!d_run)
        return true;
    return cuda_ok(cudaMemsetAsync(d_run, 0xff, (size_t)CAL_MAX_PROCESSES_CORE * tile_words * sizeof(unsigned), stream),
                   "arm tile skipping");
}

bool CalGrid::clear_dirty()
{
    return cuda_ok(cudaMemsetAsync(d_dirty, 0, 4 * sizeof(unsigned), stream), "clear written bits");
}

bool CalGrid::update_all()
{
    if (!to_device_all())
        return false;
    if (active) {
        /* calUpdateActiveCells2D, then every registered substate's next ->
         * current at the new list's cells: one compaction whose scatter
         * pass does the copy */
        ActiveCopy u;
        memset(&u, 0, sizeof(u));
        for (int t = 0; t < CAL_NTYPES; t++)
            for (int sl = 0; sl < nslot[t]; sl++) {
                Sub& q = sub[t][sl];
                if (!q.used || q.single || q.next_stale)
                    continue;
                u.src[u.n] = q.layer[1].dev;
                u.dst[u.n] = q.layer[0].dev;
                u.elem[u.n] = (unsigned char)q.elem;
                u.n++;
            }
        u.count = d_count;
        if (!cuda_ok(compact_and_copy(d_flags, dim, rows, cols, slices, d_cells, d_lin, d_count, d_block_counts,
                                      scratch_ints, u, stream, flags_dirty_word()),
                     "active-cell compaction and update"))
            return false;
        for (int t = 0; t < CAL_NTYPES; t++)
            for (int sl = 0; sl < nslot[t]; sl++) {
                Sub& q = sub[t][sl];
                if (!q.used || q.single || q.next_stale)
                    continue;
                q.layer[0].host_valid = false;
                q.forced_dirty = false;
            }
        written_since_update = false;
        return clear_dirty();
    }
    std::vector<std::pair<int, int>> all;
    for (int t = 0; t < CAL_NTYPES; t++)
        for (int s = 0; s < nslot[t]; s++)
            if (!sub[t][s].single)
                all.push_back(std::make_pair(t, s));
    /* without active cells, untouched substates are skipped (next == current
     * everywhere); with them, every registered substate is copied */
    if (!active && !written_since_update) {
        bool forced = false;
        for (size_t w = 0; w < all.size(); w++)
            forced = forced || sub[all[w].first][all[w].second].forced_dirty;
        if (!forced)
            return true; /* nothing was written since the last update */
    }
    if (!copy_next_to_current(all, !active, true))
        return false;
    written_since_update = false;
    return clear_dirty();
}

bool CalGrid::swap(int type, int slot)
{
    Sub& q = sub[type][slot];
    if (!q.used || q.single)
        return true;
    Layer tmp = q.layer[0];
    q.layer[0] = q.layer[1];
    q.layer[1] = tmp;
    q.layer[0].host_valid = false;
    q.layer[1].host_valid = false;
    q.next_stale = true;
    if (q.trackable) {
        q.trackable = false; /* the layers were written outside the tracked path */
        inval_epoch++;
    }
    swaps++;
    return true;
}

bool CalGrid::sync()
{
    return cuda_ok(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
}

void CalGrid::save(GridState* st) const
{
    memcpy(st->sub, sub, sizeof(sub));
    st->flags_host_valid = flags_host_valid;
    st->flags_dev_valid = flags_dev_valid;
    st->transfers = transfers;
    st->swaps = swaps;
}

void CalGrid::restore(const GridState* st)
{
    memcpy(sub, st->sub, sizeof(sub));
    flags_host_valid = st->flags_host_valid;
    flags_dev_valid = st->flags_dev_valid;
    transfers = st->transfers;
    swaps = st->swaps;
}

void CalGrid::launch_grid(int* gx, int* gy) const
{
    int x = (cols + 255) / 256;
    if (x > 16)
        x = 16;
    const long long lines = (long long)rows * slices;
    long long y = (152LL * 8 * 2) / x;
    if (y > lines)
        y = lines;
    if (y > 65535)
        y = 65535;
    if (y < 1)
        y = 1;
    *gx = x;
    *gy = (int)y;
}

} // namespace cal

/* ======================= error API ====================================== */

extern "C" enum CALError calGetLastError(void)
{
    return cal::g_err;
}

extern "C" const char* calGetErrorString(void)
{
    return cal::g_err == CAL_SUCCESS ? "no error" : cal::g_msg;
}

extern "C" void calClearError(void)
{
    cal::g_err = CAL_SUCCESS;
    cal::g_msg[0] = 0;
}
