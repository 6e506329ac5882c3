/*
 * cal2DDevice.cuh -- device side of the 2D API (included by cal2D.h when the
 * translation unit is compiled by nvcc).
 *
 * Writing an elementary process for the GPU:
 *
 *     #include <opencal/cal2D.h>
 *     __managed__ struct { struct CALSubstate2Dr *z, *h; } Q;   // handles
 *     __managed__ struct { CALreal eps; } P;                     // parameters
 *
 *     CAL_ELEMENTARY_PROCESS_2D(flows)(struct CALModel2D* ca, int i, int j)
 *     {
 *         if (calGet2Dr(ca, Q.h, i, j) <= P.eps) return;
 *         ... calGetX2Dr(ca, Q.z, i, j, n) ... calSet2Dr(ca, Q.h, i, j, v);
 *     }
 *     ...
 *     calAddElementaryProcess2D(model, flows);   // host, same call as OpenCAL
 *
 * The body is the reference's per-cell callback; it runs as one GPU thread
 * per cell (or per active cell).  Globals it reads (substate handles,
 * parameters) must be visible from the device: declare them __managed__.
 *
 * How the accessors find a substate: every model allocates the handles of
 * one type from a single 32-byte-stride pool, so a handle's slot is
 * (handle - pool) >> 5.  The launch descriptor (a __grid_constant__ kernel
 * parameter, i.e. constant-cache resident) maps slots to device buffers.
 * Nothing is looked up in memory per access besides the cell itself.
 */
#ifndef cal2DDevice_cuh
#define cal2DDevice_cuh

#include <cuda.h> /* CUtensorMap */
#include <cuda_runtime.h>
#include <stdint.h>

#define CAL_TYPE_B 0
#define CAL_TYPE_I 1
#define CAL_TYPE_R 2
#define CAL_HANDLE_SHIFT 5 /* log2(sizeof(struct CALSubstate2Dr)) */
#define CAL_EP_THREADS 256
#ifndef CAL_MAX_STAGED
#define CAL_MAX_STAGED 8 /* substates a process may declare it reads (calSetElementaryProcessReads2D) */
#endif

/* Launch descriptor of one elementary-process kernel. */
struct CALDevModel2D {
    struct CALModel2D model; /* public fields for user code: rows, columns, sizeof_X, X (device copy) */
    unsigned long long pool[3]; /* host address of the handle pool of each type */
    void* cur[3][CAL_MAX_SUBSTATES];
    void* nxt[3][CAL_MAX_SUBSTATES];
    unsigned int* dirty;         /* [3] bitmasks: substates whose next layer was written */
    unsigned int* flags_dirty;   /* set when a process changed an active-cell flag (NULL: not kept) */
    int* step;                   /* current step of a device-driven run (calRunDevice2D) */
    CALbyte* flags;              /* active-cell flags, NULL without the optimisation */
    struct CALCell2D* cells;     /* compacted active list */
    int* count;                  /* its length */
    int rows, cols;
    int toroidal;
    int hex;      /* 0: none; 1: shift on odd columns; 2: shift on odd rows */
    int use_list; /* iterate the active list when it is non-empty */
    int nx;
    int xi[CAL_MAX_NEIGHBORS];
    int xj[CAL_MAX_NEIGHBORS];
    /* change tracking (models without active cells): the grid is cut into
     * CAL_TILE_W x CAL_TILE_H tiles; a process that stores into next a value
     * whose bits differ from current sets the tile's bit in chg (one bitmap
     * of tile_words words per substate slot, index type * CAL_MAX_SUBSTATES
     * + slot), so that the update copies only those tiles; writes the tile
     * bitmaps cannot follow (unsafe operations) set the substate's bit in
     * untracked[type] and the update copies all of it */
    int track;
    int tiles_x, tiles_y, tile_words;
    unsigned int* chg;
    unsigned int* untracked;
    /* tile skipping of a process declared pure (calSetElementaryProcessPure2D),
     * NULL otherwise: one bit per tile, set where the process must run (its
     * neighbourhood changed since it last changed nothing there); the kernel
     * skips the other tiles and clears the bit of every tile where it
     * changed nothing */
    unsigned int* run;
    /* with quiet (skipping launches whose busy tiles are dealt over the
     * blocks): run stays unchanged during the launch, every block computes
     * the same compaction of it, block b takes busy tiles b, b + nblocks, ...
     * (the lowest blocks, which the hardware places on different SMs, get
     * the work), the tiles where the process changed nothing are gathered in
     * quiet and the last block to finish (ticket) clears them from run */
    unsigned int* quiet;
    unsigned int* ticket;
    /* guard of the process (calSetElementaryProcessGuard2Dr): it returns at
     * once where the current layer of real slot guard_slot compares true
     * with guard_value under guard_op; 0: none */
    int guard_op, guard_slot;
    double guard_value;
    /* TMA staging of the substates a process declared it reads
     * (calSetElementaryProcessReads2D); nstage == 0: none.  On every tile
     * that the process runs on (in toroidal grids only tiles off the grid's
     * border), box k -- (CAL_TILE_W + 2 * hx) x (CAL_TILE_H + 2 * stage_r)
     * elements from (j0 - hx, i0 - stage_r), hx = 16 / element size, so
     * that the box starts on a 16-byte boundary -- is loaded into the
     * dynamic shared memory at stage_off[k] bytes by one
     * cp.async.bulk.tensor.2d through stage_map[k] (zero fill outside the
     * grid: the flat boundary's "absent neighbours read 0"), and the
     * accessors read the staged substates there.  stage_of[type][slot] = k
     * or -1; stage_tx: the bytes the boxes bring (the mbarrier's
     * transaction count); stage_bytes: the dynamic shared memory. */
    int nstage, stage_r, stage_tx, stage_bytes, stage_hxmax;
    int stage_off[CAL_MAX_STAGED];
    int stage_hx[CAL_MAX_STAGED]; /* 16 / element size: 16, 4, 2 (x stays 16-byte aligned) */
    signed char stage_of[3][CAL_MAX_SUBSTATES];
    int* stage_err; /* set when a box did not arrive in time (the tile then reads global memory) */
    CUtensorMap stage_map[CAL_MAX_STAGED];
};


#if defined(__CUDACC__)

/* per-block record of which substates a process wrote (plain byte stores:
 * every writer stores 1, so concurrent writers cannot lose an update) */
static __shared__ unsigned char cal_written2D[3 * CAL_MAX_SUBSTATES];
/* per warp: substates whose next layer this warp changed in the current
 * tile (flushed into the chg bitmaps after each tile row), and per block:
 * substates written by unsafe operations */
static __shared__ unsigned char cal_chg2D[CAL_EP_THREADS / 32][3 * CAL_MAX_SUBSTATES];
static __shared__ unsigned char cal_untracked2D[3 * CAL_MAX_SUBSTATES];
/* per block: a process changed an active-cell flag */
static __shared__ unsigned char cal_flagchg2D;
/* per block: the current tile is staged, its origin, the staging barrier */
static __shared__ int cal_stage_on2D, cal_stage_i02D, cal_stage_j02D, cal_stage_pad2D, cal_stage_buf2D;
static __shared__ __align__(8) unsigned long long cal_stage_bar2D[2];
/* per block: the cells of the current tile that pass the process's guard
 * (thread index in the tile: row * 32 + column) and each warp's count */
static __shared__ unsigned char cal_gcell2D[CAL_EP_THREADS];
static __shared__ int cal_gcount2D[CAL_EP_THREADS / 32];
/* per block: the busy tiles dealt to it (skipping launches with quiet) */
#define CAL_DEAL_MAX 64
static __shared__ int cal_dtile2D[CAL_DEAL_MAX];
static __shared__ int cal_dlast2D;
extern __shared__ __align__(128) unsigned char cal_stage_mem2D[];

/* ---- TMA: mbarrier with a transaction count, tiled 2D loads, bounded wait */
static __device__ __forceinline__ uint32_t cal_smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}
static __device__ __forceinline__ void cal_bar_init(unsigned long long* bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(cal_smem_u32(bar)) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
static __device__ __forceinline__ void cal_bar_expect(unsigned long long* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(cal_smem_u32(bar)), "r"(bytes)
                 : "memory");
}
static __device__ __forceinline__ void cal_tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                                       unsigned long long* bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];" ::"r"(cal_smem_u32(dst)),
                 "l"(map), "r"(x), "r"(y), "r"(cal_smem_u32(bar))
                 : "memory");
}
static __device__ __forceinline__ bool cal_bar_wait(unsigned long long* bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t k = 0; k < limit; k++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(cal_smem_u32(bar)), "r"(parity)
                     : "memory");
        if (done)
            return true;
    }
    return false;
}
#define CAL_STAGE_WAIT_LIMIT (1u << 20)

template <typename T>
static __device__ __forceinline__ bool cal_same_bits(T a, T b)
{
    return a == b;
}
template <>
__device__ __forceinline__ bool cal_same_bits<double>(double a, double b)
{
    return __double_as_longlong(a) == __double_as_longlong(b);
}

/* The model a device process receives is a copy of the descriptor's public
 * part made by the kernel (cal_model_view2D): its `gpu` field points at the
 * launch descriptor, where the accessors find the buffers. */
static __device__ __forceinline__ const struct CALDevModel2D* cal_dm2D(const struct CALModel2D* ca)
{
    return reinterpret_cast<const struct CALDevModel2D*>(ca->gpu);
}

/* The kernel-local model handed to user code.  NX > 0: the launch is for a
 * model whose neighbourhood has NX cells, and the copy says so as a
 * compile-time constant, so that a process's loops over ca->sizeof_X have a
 * fixed count and arrays indexed by the neighbour (u[n], eliminated[n], ...)
 * live in registers instead of local memory.  The copy is only read; once
 * the process is inlined its fields are the descriptor's, in registers. */
template <int NX>
static __device__ __forceinline__ struct CALModel2D cal_model_view2D(const struct CALDevModel2D& m)
{
    struct CALModel2D v = m.model;
    if (NX > 0)
        v.sizeof_X = NX;
    v.gpu = reinterpret_cast<struct CALGpuModel2D*>(const_cast<struct CALDevModel2D*>(&m));
    return v;
}

static __device__ __forceinline__ int cal_slot2D(const struct CALDevModel2D* m, int t, const void* q)
{
    return (int)(((unsigned long long)(uintptr_t)q - m->pool[t]) >> CAL_HANDLE_SHIFT);
}

static __device__ __forceinline__ long long cal_lin2D(const struct CALDevModel2D* m, int i, int j)
{
    return (long long)i * m->cols + j;
}

/* neighbour n of (i, j): cal2D.c:859-870 semantics, FLAT = absent outside */
static __device__ __forceinline__ bool cal_nbr2D(const struct CALDevModel2D* m, int i, int j, int n, int& ni, int& nj)
{
    if ((m->hex == 1 && (j & 1)) || (m->hex == 2 && (i & 1)))
        n += CAL_HEXAGONAL_SHIFT;
    ni = i + m->xi[n];
    nj = j + m->xj[n];
    if (m->toroidal) {
        ni = ni < 0 ? ni + m->rows : (ni >= m->rows ? ni - m->rows : ni);
        nj = nj < 0 ? nj + m->cols : (nj >= m->cols ? nj - m->cols : nj);
        return true;
    }
    return (unsigned)ni < (unsigned)m->rows && (unsigned)nj < (unsigned)m->cols;
}

/* the staged copy of substate (t, slot) at (a, b), when the current tile is
 * staged and the substate is one of the declared reads; NULL otherwise */
template <typename T>
static __device__ __forceinline__ const T* cal_staged2D(const struct CALDevModel2D* m, int t, int s, int a, int b)
{
    if (!m->nstage || !cal_stage_on2D)
        return nullptr;
    const int k = m->stage_of[t][s];
    if (k < 0)
        return nullptr;
    constexpr int hx = 16 / (int)sizeof(T);
    constexpr int bw = CAL_TILE_W + 2 * hx;
    const int y = a - cal_stage_i02D + m->stage_r, x = b - cal_stage_j02D + hx;
    /* a cell outside the box (calGet at other coordinates) reads global memory */
    if ((unsigned)y >= (unsigned)(CAL_TILE_H + 2 * m->stage_r) || (unsigned)x >= (unsigned)bw)
        return nullptr;
    const T* box = reinterpret_cast<const T*>(cal_stage_mem2D + cal_stage_pad2D + cal_stage_buf2D + m->stage_off[k]);
    return box + y * bw + x;
}

template <typename T>
static __device__ __forceinline__ T cal_get2D(const struct CALModel2D* ca, int t, const void* q, int i, int j)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    const int s = cal_slot2D(m, t, q);
    if (const T* p = cal_staged2D<T>(m, t, s, i, j))
        return *p;
    return static_cast<const T*>(m->cur[t][s])[cal_lin2D(m, i, j)];
}

template <typename T>
static __device__ __forceinline__ T cal_getx2D(const struct CALModel2D* ca, int t, const void* q, int i, int j, int n)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    const int s = cal_slot2D(m, t, q);
    if (m->nstage && cal_stage_on2D) {
        /* a staged tile lies inside a toroidal grid or the box's zero fill
         * is the flat boundary: the neighbour is read without wrapping */
        const int nn = ((m->hex == 1 && (j & 1)) || (m->hex == 2 && (i & 1))) ? n + CAL_HEXAGONAL_SHIFT : n;
        if (const T* p = cal_staged2D<T>(m, t, s, i + m->xi[nn], j + m->xj[nn]))
            return *p;
    }
    int a, b;
    if (!cal_nbr2D(m, i, j, n, a, b))
        return (T)0;
    return static_cast<const T*>(m->cur[t][s])[cal_lin2D(m, a, b)];
}

/* the tile of a tracked process changed substate (t, s): flagged for the
 * calling warp (a process writes only its own cell, which lies in the
 * block's current tile) */
static __device__ __forceinline__ void cal_mark_chg2D(int t, int s)
{
    cal_chg2D[threadIdx.x >> 5][t * CAL_MAX_SUBSTATES + s] = 1;
}

template <typename T>
static __device__ __forceinline__ void cal_set2D(const struct CALModel2D* ca, int t, const void* q, int i, int j, T v)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    int s = cal_slot2D(m, t, q);
    const long long c = cal_lin2D(m, i, j);
    static_cast<T*>(m->nxt[t][s])[c] = v;
    cal_written2D[t * CAL_MAX_SUBSTATES + s] = 1;
    if (m->track && !cal_same_bits(static_cast<const T*>(m->cur[t][s])[c], v))
        cal_mark_chg2D(t, s);
}

template <typename T>
static __device__ __forceinline__ void cal_setcur2D(const struct CALModel2D* ca, int t, const void* q, int i, int j, T v)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    int s = cal_slot2D(m, t, q);
    static_cast<T*>(m->cur[t][s])[cal_lin2D(m, i, j)] = v;
    /* the next update copies next over it, as in the reference */
    cal_written2D[t * CAL_MAX_SUBSTATES + s] = 1;
    if (m->track)
        cal_mark_chg2D(t, s);
}

template <typename T>
static __device__ __forceinline__ void cal_init2D(const struct CALModel2D* ca, int t, const void* q, int i, int j, T v)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    int s = cal_slot2D(m, t, q);
    long long c = cal_lin2D(m, i, j);
    static_cast<T*>(m->cur[t][s])[c] = v;
    if (m->nxt[t][s])
        static_cast<T*>(m->nxt[t][s])[c] = v;
    cal_written2D[t * CAL_MAX_SUBSTATES + s] = 1;
    if (m->track)
        cal_mark_chg2D(t, s); /* the tile no longer holds the substate's uniform value */
}

/* flag writes: only a changed flag is stored, and the block notes it (the
 * compaction after the process keeps the list when no block did) */
static __device__ __forceinline__ void cal_setflag2D(const struct CALDevModel2D* m, long long c, CALbyte v)
{
    if (!m->flags) /* a model without active cells: nothing to record */
        return;
    if (m->flags[c] != v) {
        m->flags[c] = v;
        cal_flagchg2D = 1;
    }
}

static __device__ __forceinline__ void cal_addactive2D(const struct CALModel2D* ca, int i, int j)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    if ((unsigned)i < (unsigned)m->rows && (unsigned)j < (unsigned)m->cols)
        cal_setflag2D(m, cal_lin2D(m, i, j), 1);
}

static __device__ __forceinline__ void cal_addactivex2D(const struct CALModel2D* ca, int i, int j, int n)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    int a, b;
    if (cal_nbr2D(m, i, j, n, a, b))
        cal_setflag2D(m, cal_lin2D(m, a, b), 1);
}

static __device__ __forceinline__ void cal_removeactive2D(const struct CALModel2D* ca, int i, int j)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    cal_setflag2D(m, cal_lin2D(m, i, j), 0);
}

/* the step number a device-driven run is executing (calRunDevice2D); the
 * device counterpart of reading CALRun2D::step in a stop condition */
static __device__ __forceinline__ int calRunGetStep2D(const struct CALModel2D* ca)
{
    return *cal_dm2D(ca)->step;
}

/* number of active cells after the last update (device counterpart of
 * A.size_current) */
static __device__ __forceinline__ int calGetActiveCellCountDevice2D(const struct CALModel2D* ca)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    return m->count ? *m->count : 0;
}

/* One elementary process over every cell, or over the active list when the
 * optimisation is on and the list is non-empty (cal2D.c:717-734).  The grid
 * is sized by the host to a few waves of the GPU; both loops are
 * grid-stride.  Without the list the blocks take CAL_TILE_W x CAL_TILE_H
 * tiles (one cell per thread, a warp per tile row); with change tracking
 * each warp then adds its tile to the chg bitmap of every substate whose
 * next layer it changed.  At the end each block publishes which substates
 * it wrote (and which it wrote by unsafe operations). */
template <void (*EP)(struct CALModel2D*, int, int), int NX, int MODE>
__global__ void __launch_bounds__(CAL_EP_THREADS) cal_ep2D_kernel(const __grid_constant__ struct CALDevModel2D m)
{
    /* MODE 0: tile by tile; 1: declared reads staged by TMA; 2: tile
     * skipping, the block's run bits fetched 32 tiles at a time; 3: a
     * guarded process, the tile's passing cells packed into consecutive
     * threads (with or without tile skipping) */
    constexpr bool STAGED = MODE == 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int t = threadIdx.x; t < 3 * CAL_MAX_SUBSTATES; t += blockDim.x) {
        cal_written2D[t] = 0;
        cal_untracked2D[t] = 0;
    }
    for (int t = lane; t < 3 * CAL_MAX_SUBSTATES; t += 32)
        cal_chg2D[warp][t] = 0;
    if (threadIdx.x == 0) {
        cal_flagchg2D = 0;
        cal_stage_on2D = 0;
        /* the boxes start on a 128-byte boundary of the shared window (the
         * launch adds 128 bytes for this) */
        cal_stage_pad2D = (int)((128u - (cal_smem_u32(cal_stage_mem2D) & 127u)) & 127u);
        cal_stage_buf2D = 0;
        if (STAGED && m.nstage) {
            cal_bar_init(&cal_stage_bar2D[0]);
            cal_bar_init(&cal_stage_bar2D[1]);
        }
    }
    __syncthreads();
    struct CALModel2D view = cal_model_view2D<NX>(m);
    struct CALModel2D* ca = &view;
    int nstage = STAGED ? m.nstage : 0; /* 0 after a box failed to arrive: global reads for the rest */
    const int listed = m.use_list ? *m.count : 0;
    const int nblocks = gridDim.x * gridDim.y, bid = blockIdx.y * gridDim.x + blockIdx.x;
    if (listed > 0) {
        const int stride = nblocks * blockDim.x;
        for (int n = bid * blockDim.x + threadIdx.x; n < listed; n += stride) {
            const struct CALCell2D c = m.cells[n];
            EP(ca, c.i, c.j);
        }
    } else {
        const int ntiles = m.tiles_x * m.tiles_y;
        /* skipping launches with quiet: every block ranks the busy tiles
         * (the set bits of run, in tile order: each thread counts a run of
         * words, then a block scan) and takes ranks bid, bid + nblocks, ...
         * into cal_dtile2D (at most CAL_DEAL_MAX: the host deals only when
         * the tiles allow it); -1 when the launch does not deal */
        auto deal_tiles = [&]() -> int {
            const int W = m.tile_words;
            const int per = (W + CAL_EP_THREADS - 1) / CAL_EP_THREADS;
            const int w0 = (int)threadIdx.x * per, w1 = min(W, w0 + per);
            int cnt = 0;
            for (int w = w0; w < w1; w++)
                cnt += __popc(m.run[w]);
            int incl = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o)
                    incl += y;
            }
            if (lane == 31)
                cal_gcount2D[warp] = incl;
            __syncthreads();
            int pre = incl - cnt, total = 0;
            for (int w = 0; w < CAL_EP_THREADS / 32; w++) {
                const int v = cal_gcount2D[w];
                pre += w < warp ? v : 0;
                total += v;
            }
            if (cnt) {
                int r = bid >= pre ? bid : bid + (pre - bid + nblocks - 1) / nblocks * nblocks;
                int seen = pre;
                for (int w = w0; w < w1 && r < pre + cnt; w++) {
                    const unsigned bits = m.run[w];
                    const int n = __popc(bits);
                    for (; r < seen + n; r += nblocks) {
                        unsigned b = bits;
                        for (int k = r - seen; k > 0; k--)
                            b &= b - 1; /* drop the lowest set bits below rank r */
                        cal_dtile2D[(r - bid) / nblocks] = w * 32 + __ffs(b) - 1;
                    }
                    seen += n;
                }
            }
            __syncthreads();
            return total > bid ? (total - bid + nblocks - 1) / nblocks : 0;
        };
        const int ntodo = (MODE != 0 && m.run && m.quiet) ? deal_tiles() : -1;
        if (!STAGED) {
        /* one tile, one cell per thread; with change tracking each warp
         * records which substates it changed in the tile, and with tile
         * skipping a tile where the process changed nothing has its bit
         * cleared (or, when the launch deals its tiles, gathered in quiet for
         * the last block to clear) */
        auto run_tile = [&](int tile) {
            const unsigned tbit = 1u << (tile & 31);
            const int ty = tile / m.tiles_x;
            const int i = ty * CAL_TILE_H + warp, j = (tile - ty * m.tiles_x) * CAL_TILE_W + lane;
            if (MODE == 3) {
                /* the cells that pass the guard, in tile order, onto threads
                 * 0, 1, ... (the counting barrier comes first: the previous
                 * tile's list is read until every thread has taken its cell) */
                bool pass = false;
                if (i < m.rows && j < m.cols) {
                    const double v = ((const double*)m.cur[CAL_TYPE_R][m.guard_slot])[(long long)i * m.cols + j];
                    const double w = m.guard_value;
                    switch (m.guard_op) {
                    case 1: pass = !(v <= w); break;
                    case 2: pass = !(v < w); break;
                    case 3: pass = !(v >= w); break;
                    case 4: pass = !(v > w); break;
                    case 5: pass = !(v == w); break;
                    case 6: pass = !(v != w); break;
                    default: pass = true; break;
                    }
                }
                /* one barrier settles a tile where no cell or every cell
                 * passes; the others are packed */
                const int total = __syncthreads_count(pass);
                if (total == CAL_EP_THREADS) {
                    EP(ca, i, j);
                } else if (total > 0) {
                    const unsigned bal = __ballot_sync(0xffffffffu, pass);
                    if (lane == 0)
                        cal_gcount2D[warp] = __popc(bal);
                    __syncthreads();
                    int off = 0;
                    for (int w = 0; w < warp; w++)
                        off += cal_gcount2D[w];
                    if (pass)
                        cal_gcell2D[off + __popc(bal & ((1u << lane) - 1u))] = (unsigned char)threadIdx.x;
                    __syncthreads();
                    if ((int)threadIdx.x < total) {
                        const int q = cal_gcell2D[threadIdx.x];
                        EP(ca, ty * CAL_TILE_H + (q >> 5), (tile - ty * m.tiles_x) * CAL_TILE_W + (q & 31));
                    }
                }
            } else if (i < m.rows && j < m.cols) {
                EP(ca, i, j);
            }
            if (m.track) {
                bool changed = false;
                __syncwarp();
                for (int t = lane; t < 3 * CAL_MAX_SUBSTATES; t += 32)
                    if (cal_chg2D[warp][t]) {
                        cal_chg2D[warp][t] = 0;
                        changed = true;
                        atomicOr(&m.chg[(long long)t * m.tile_words + (tile >> 5)], tbit);
                    }
                __syncwarp();
                if (m.run && !__syncthreads_or(changed) && threadIdx.x == 0) {
                    if (m.quiet)
                        atomicOr(&m.quiet[tile >> 5], tbit);
                    else
                        atomicAnd(&m.run[tile >> 5], ~tbit);
                }
            }
        };
        if (ntodo >= 0) {
            for (int k = 0; k < ntodo; k++)
                run_tile(cal_dtile2D[k]);
        } else if (MODE == 2 || (MODE == 3 && m.run)) {
            /* the block's tiles bid, bid + nblocks, ..., only those whose run
             * bit is set.  The bits of 32 of them come in one load per lane
             * and a ballot (the same in every warp: a bit is cleared only by
             * the block that owns the tile, after every warp has taken its
             * ballot), so that a block with nothing to run leaves after one
             * round trip instead of one per tile.  Its own instantiation:
             * the loop's state costs registers the plain loop does not pay. */
            for (int base = bid; base < ntiles; base += 32 * nblocks) {
                const int t = base + lane * nblocks;
                bool need = t < ntiles;
                if (need && m.run)
                    need = (m.run[t >> 5] >> (t & 31)) & 1u;
                for (unsigned todo = __ballot_sync(0xffffffffu, need); todo; todo &= todo - 1)
                    run_tile(base + (__ffs(todo) - 1) * nblocks);
            }
        } else {
            for (int tile = bid; tile < ntiles; tile += nblocks)
                if (!m.run || (m.run[tile >> 5] >> (tile & 31)) & 1u)
                    run_tile(tile);
        }
        } else {
        /* staged: the tiles dealt to the block, or the block's tiles bid,
         * bid + nblocks, ... (with tile skipping only those whose bit is set:
         * a bit is cleared only by the block that owns the tile, after
         * processing it, so every thread finds the same next tile).  With
         * staging, the next tile's boxes are loaded into the other of two
         * buffers while the current tile computes.  next_tile(from, k): the
         * tile after the k-th of the block. */
        auto next_tile = [&](int from, int k) {
            if (ntodo >= 0)
                return k < ntodo ? cal_dtile2D[k] : ntiles;
            int t = from;
            while (t < ntiles && m.run && !(m.run[t >> 5] & (1u << (t & 31))))
                t += nblocks;
            return t;
        };
        auto staged_tile = [&](int t) {
            /* toroidal grids: only tiles whose boxes lie inside the grid (no
             * neighbour read needs a wrap); flat grids: every tile */
            const int ty = t / m.tiles_x;
            const int i0 = ty * CAL_TILE_H, j0 = (t - ty * m.tiles_x) * CAL_TILE_W;
            return !m.toroidal || (i0 - m.stage_r >= 0 && i0 + CAL_TILE_H + m.stage_r <= m.rows &&
                                   j0 - m.stage_hxmax >= 0 && j0 + CAL_TILE_W + m.stage_hxmax <= m.cols);
        };
        /* thread 0: the boxes of tile t into buffer b */
        auto issue = [&](int t, int b) {
            const int ty = t / m.tiles_x, tx = t - ty * m.tiles_x;
            /* earlier reads of the buffer (generic proxy, ordered by the
             * block barrier) before the copies (async proxy) overwrite it */
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            cal_bar_expect(&cal_stage_bar2D[b], (uint32_t)m.stage_tx);
            for (int k = 0; k < nstage; k++)
                cal_tma_load_2d(cal_stage_mem2D + cal_stage_pad2D + b * m.stage_bytes + m.stage_off[k],
                                &m.stage_map[k], tx * CAL_TILE_W - m.stage_hx[k], ty * CAL_TILE_H - m.stage_r,
                                &cal_stage_bar2D[b]);
        };
        uint32_t phases = 0;  /* bit b: parity of buffer b's next phase */
        uint32_t pending = 0; /* bit b: copies issued into buffer b and not yet waited for */
        int buf = 0;
        int nk = 0; /* the block's tiles taken so far */
        int tile = next_tile(bid, nk++);
        if (nstage && tile < ntiles && staged_tile(tile)) {
            if (threadIdx.x == 0)
                issue(tile, 0);
            pending = 1u;
        }
        while (tile < ntiles) {
            const unsigned tbit = 1u << (tile & 31);
            const int nxt = next_tile(tile + nblocks, nk++);
            const int ty = tile / m.tiles_x, tx = tile - ty * m.tiles_x;
            const int i = ty * CAL_TILE_H + warp, j = tx * CAL_TILE_W + lane;
            if (nstage) {
                if (nxt < ntiles && staged_tile(nxt)) { /* prefetch */
                    if (threadIdx.x == 0)
                        issue(nxt, buf ^ 1);
                    pending |= 1u << (buf ^ 1);
                }
                bool arrived = true;
                if ((pending >> buf) & 1u) {
                    arrived = cal_bar_wait(&cal_stage_bar2D[buf], (phases >> buf) & 1u, CAL_STAGE_WAIT_LIMIT);
                    phases ^= 1u << buf;
                    pending &= ~(1u << buf);
                }
                if (threadIdx.x == 0) {
                    cal_stage_on2D = staged_tile(tile) && arrived;
                    cal_stage_i02D = ty * CAL_TILE_H;
                    cal_stage_j02D = tx * CAL_TILE_W;
                    cal_stage_buf2D = buf * m.stage_bytes;
                }
                if (!__syncthreads_and(arrived)) {
                    /* a box did not arrive: record it, wait (bounded) for the
                     * copies still in flight into this block's shared memory,
                     * and read global memory from here on */
                    if (threadIdx.x == 0) {
                        if (m.stage_err)
                            atomicExch(m.stage_err, 1);
                        cal_bar_wait(&cal_stage_bar2D[buf], ((phases >> buf) & 1u) ^ 1u, CAL_STAGE_WAIT_LIMIT);
                        if ((pending >> (buf ^ 1)) & 1u)
                            cal_bar_wait(&cal_stage_bar2D[buf ^ 1], (phases >> (buf ^ 1)) & 1u, CAL_STAGE_WAIT_LIMIT);
                        cal_stage_on2D = 0;
                    }
                    __syncthreads();
                    nstage = 0;
                }
            }
            if (i < m.rows && j < m.cols)
                EP(ca, i, j);
            if (nstage)
                __syncthreads(); /* every read of this buffer done before it is refilled */
            if (m.track) {
                bool changed = false;
                __syncwarp();
                for (int t = lane; t < 3 * CAL_MAX_SUBSTATES; t += 32)
                    if (cal_chg2D[warp][t]) {
                        cal_chg2D[warp][t] = 0;
                        changed = true;
                        atomicOr(&m.chg[(long long)t * m.tile_words + (tile >> 5)], tbit);
                    }
                __syncwarp();
                if (m.run && !__syncthreads_or(changed) && threadIdx.x == 0) {
                    if (m.quiet)
                        atomicOr(&m.quiet[tile >> 5], tbit);
                    else
                        atomicAnd(&m.run[tile >> 5], ~tbit);
                }
            }
            tile = nxt;
            buf ^= 1;
        }
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 3 * CAL_MAX_SUBSTATES; t += blockDim.x) {
        /* every block of a dense launch writes the same bits: the atomic only
         * where the bit is not already set, so that the blocks do not queue
         * on one word */
        const unsigned bit = 1u << (t % CAL_MAX_SUBSTATES);
        if (cal_written2D[t] && !(*(volatile const unsigned*)&m.dirty[t / CAL_MAX_SUBSTATES] & bit))
            atomicOr(&m.dirty[t / CAL_MAX_SUBSTATES], bit);
        if (cal_untracked2D[t] && m.untracked)
            atomicOr(&m.untracked[t / CAL_MAX_SUBSTATES], 1u << (t % CAL_MAX_SUBSTATES));
    }
    if (threadIdx.x == 0 && cal_flagchg2D && m.flags_dirty)
        *m.flags_dirty = 1;
    if (MODE != 0 && m.run && m.quiet && !listed) {
        /* the last block to finish clears the quiet tiles from run */
        if (threadIdx.x == 0) {
            __threadfence();
            cal_dlast2D = atomicAdd(m.ticket, 1u) == (unsigned)(gridDim.x * gridDim.y) - 1u;
        }
        __syncthreads();
        if (cal_dlast2D) {
            __threadfence();
            for (int w = threadIdx.x; w < m.tile_words; w += blockDim.x) {
                const unsigned q = __ldcg(m.quiet + w);
                if (q) {
                    m.run[w] &= ~q;
                    m.quiet[w] = 0;
                }
            }
            if (threadIdx.x == 0)
                *m.ticket = 0;
        }
    }
}

/* one kernel per common neighbourhood size (von Neumann 5, hexagonal 7,
 * Moore 9) and a generic one for the others, each plain, with the staging
 * of declared reads, with tile skipping, and for a guarded process (the
 * staging, skipping and packing loops cost registers and barriers that the
 * plain loop does not pay) */
template <void (*EP)(struct CALModel2D*, int, int)>
static int cal_launch_ep2D(const struct CALDevModel2D* m, int gx, int gy, void* stream)
{
    const dim3 grid(gx, gy);
    cudaStream_t st = (cudaStream_t)stream;
    /* two buffers of boxes, + alignment */
    const size_t smem = m->nstage ? 2 * (size_t)m->stage_bytes + 128 : 0;
    if (m->nstage) {
        switch (m->model.sizeof_X) {
        case 5: cal_ep2D_kernel<EP, 5, 1><<<grid, CAL_EP_THREADS, smem, st>>>(*m); break;
        case 7: cal_ep2D_kernel<EP, 7, 1><<<grid, CAL_EP_THREADS, smem, st>>>(*m); break;
        case 9: cal_ep2D_kernel<EP, 9, 1><<<grid, CAL_EP_THREADS, smem, st>>>(*m); break;
        default: cal_ep2D_kernel<EP, 0, 1><<<grid, CAL_EP_THREADS, smem, st>>>(*m); break;
        }
    } else if (m->guard_op) {
        switch (m->model.sizeof_X) {
        case 5: cal_ep2D_kernel<EP, 5, 3><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        case 7: cal_ep2D_kernel<EP, 7, 3><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        case 9: cal_ep2D_kernel<EP, 9, 3><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        default: cal_ep2D_kernel<EP, 0, 3><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        }
    } else if (m->run) {
        switch (m->model.sizeof_X) {
        case 5: cal_ep2D_kernel<EP, 5, 2><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        case 7: cal_ep2D_kernel<EP, 7, 2><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        case 9: cal_ep2D_kernel<EP, 9, 2><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        default: cal_ep2D_kernel<EP, 0, 2><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        }
    } else {
        switch (m->model.sizeof_X) {
        case 5: cal_ep2D_kernel<EP, 5, 0><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        case 7: cal_ep2D_kernel<EP, 7, 0><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        case 9: cal_ep2D_kernel<EP, 9, 0><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        default: cal_ep2D_kernel<EP, 0, 0><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
        }
    }
    return (int)cudaGetLastError();
}

/* Device stop condition of a device-driven run: one thread evaluates STOP
 * after each step.  The run continues while STOP is false and, with a
 * final step, while the step number has not passed it (cal2DRun.c:125-139);
 * the decision drives the graph's conditional WHILE node.  `flag` receives
 * the decision too, for the step-by-step fallback. */
/* the largest step a device-driven run executes: past it the loop ends and
 * the second word of the step counter is set (the host reports an error) */
#ifndef CAL_DEVICE_LOOP_MAX_STEP
#define CAL_DEVICE_LOOP_MAX_STEP (1 << 26)
#endif

template <CALbyte (*STOP)(struct CALModel2D*)>
__global__ void cal_stop2D_kernel(const __grid_constant__ struct CALDevModel2D m, cudaGraphConditionalHandle h,
                                  int use_handle, int final_step, int* flag)
{
    struct CALModel2D view = cal_model_view2D<0>(m);
    cal_flagchg2D = 0;
    const bool stop = STOP(&view) != 0;
    if (cal_flagchg2D && m.flags_dirty)
        *m.flags_dirty = 1;
    int again = 0;
    if (!stop) {
        const int next = *m.step + 1;
        *m.step = next;
        again = (final_step == CAL_RUN_LOOP || next <= final_step) ? 1 : 0;
        if (again && next > CAL_DEVICE_LOOP_MAX_STEP) {
            again = 0; /* a device-driven run never loops without bound */
            m.step[1] = 1;
        }
    }
    *flag = again;
    if (use_handle)
        cudaGraphSetConditional(h, (unsigned)again);
}

template <CALbyte (*STOP)(struct CALModel2D*)>
static int cal_launch_stop2D(const struct CALDevModel2D* m, unsigned long long handle, int use_handle, int final_step,
                             int* flag, void* stream)
{
    cal_stop2D_kernel<STOP><<<1, 1, 0, (cudaStream_t)stream>>>(*m, (cudaGraphConditionalHandle)handle, use_handle,
                                                                final_step, flag);
    return (int)cudaGetLastError();
}

/* Defines a device stop condition NAME, registered for
 * calRunAddDeviceStopConditionFunc2D.  Usage:
 *   CAL_DEVICE_STOP_CONDITION_2D(NAME)(struct CALModel2D* ca) { return ...; } */
#define CAL_DEVICE_STOP_CONDITION_2D(NAME)                                                              \
    static __device__ __forceinline__ CALbyte NAME##_cal_device_(struct CALModel2D*);                 \
    extern "C" CALbyte NAME(struct CALModel2D* ca2D_)                                                   \
    {                                                                                                   \
        (void)ca2D_;                                                                                    \
        calHostCallOfDeviceProcess2D(#NAME);                                                            \
        return CAL_FALSE;                                                                               \
    }                                                                                                   \
    static const int NAME##_cal_registered_ =                                                           \
        calRegisterDeviceStopCondition2D(NAME, cal_launch_stop2D<NAME##_cal_device_>, #NAME);           \
    static __device__ __forceinline__ CALbyte NAME##_cal_device_

/* Defines the device elementary process NAME and its host-side name, which
 * is what calAddElementaryProcess2D / calApplyElementaryProcess2D take.
 * Usage: CAL_ELEMENTARY_PROCESS_2D(NAME)(struct CALModel2D* ca, int i, int j) { body } */
#define CAL_ELEMENTARY_PROCESS_2D(NAME)                                                                 \
    static __device__ __forceinline__ void NAME##_cal_device_(struct CALModel2D*, int, int);          \
    extern "C" void NAME(struct CALModel2D* ca2D_, int i_, int j_)                                      \
    {                                                                                                   \
        (void)ca2D_; (void)i_; (void)j_;                                                                \
        calHostCallOfDeviceProcess2D(#NAME);                                                            \
    }                                                                                                   \
    static const int NAME##_cal_registered_ =                                                           \
        calRegisterElementaryProcess2D(NAME, cal_launch_ep2D<NAME##_cal_device_>, #NAME);               \
    static __device__ __forceinline__ void NAME##_cal_device_

#ifndef CAL_BUILDING_LIBRARY
/* Accessors callable from both host code and device processes.  In device
 * code they touch the cell in device memory; in host code they call the
 * library's exported C functions of the same name. */
#ifdef __CUDA_ARCH__
#define CAL_HD_BODY(dev, host) return dev
#else
#define CAL_HD_BODY(dev, host) return host
#endif

#define CAL_HD_ACCESSORS_2D(S, T, TC)                                                                       \
    static __host__ __device__ __forceinline__ T cal_hd_get2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j) \
    { CAL_HD_BODY((cal_get2D<T>(ca, TC, q, i, j)), (calGet2D##S(ca, q, i, j))); }                           \
    static __host__ __device__ __forceinline__ T cal_hd_getx2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j, int n) \
    { CAL_HD_BODY((cal_getx2D<T>(ca, TC, q, i, j, n)), (calGetX2D##S(ca, q, i, j, n))); }                   \
    static __host__ __device__ __forceinline__ void cal_hd_set2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j, T v) \
    { CAL_HD_BODY((cal_set2D<T>(ca, TC, q, i, j, v)), (calSet2D##S(ca, q, i, j, v))); }                     \
    static __host__ __device__ __forceinline__ void cal_hd_setcur2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j, T v) \
    { CAL_HD_BODY((cal_setcur2D<T>(ca, TC, q, i, j, v)), (calSetCurrent2D##S(ca, q, i, j, v))); }           \
    static __host__ __device__ __forceinline__ void cal_hd_init2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j, T v) \
    { CAL_HD_BODY((cal_init2D<T>(ca, TC, q, i, j, v)), (calInit2D##S(ca, q, i, j, v))); }

CAL_HD_ACCESSORS_2D(b, CALbyte, CAL_TYPE_B)
CAL_HD_ACCESSORS_2D(i, CALint, CAL_TYPE_I)
CAL_HD_ACCESSORS_2D(r, CALreal, CAL_TYPE_R)

static __host__ __device__ __forceinline__ void cal_hd_addactive2D(struct CALModel2D* ca, int i, int j)
{ CAL_HD_BODY(cal_addactive2D(ca, i, j), calAddActiveCell2D(ca, i, j)); }
static __host__ __device__ __forceinline__ void cal_hd_addactivex2D(struct CALModel2D* ca, int i, int j, int n)
{ CAL_HD_BODY(cal_addactivex2D(ca, i, j, n), calAddActiveCellX2D(ca, i, j, n)); }
static __host__ __device__ __forceinline__ void cal_hd_removeactive2D(struct CALModel2D* ca, int i, int j)
{ CAL_HD_BODY(cal_removeactive2D(ca, i, j), calRemoveActiveCell2D(ca, i, j)); }

#define calGet2Db cal_hd_get2Db
#define calGet2Di cal_hd_get2Di
#define calGet2Dr cal_hd_get2Dr
#define calGetX2Db cal_hd_getx2Db
#define calGetX2Di cal_hd_getx2Di
#define calGetX2Dr cal_hd_getx2Dr
#define calSet2Db cal_hd_set2Db
#define calSet2Di cal_hd_set2Di
#define calSet2Dr cal_hd_set2Dr
#define calSetCurrent2Db cal_hd_setcur2Db
#define calSetCurrent2Di cal_hd_setcur2Di
#define calSetCurrent2Dr cal_hd_setcur2Dr
#define calInit2Db cal_hd_init2Db
#define calInit2Di cal_hd_init2Di
#define calInit2Dr cal_hd_init2Dr
#define calAddActiveCell2D cal_hd_addactive2D
#define calAddActiveCellX2D cal_hd_addactivex2D
#define calRemoveActiveCell2D cal_hd_removeactive2D
#endif /* CAL_BUILDING_LIBRARY */

#endif /* __CUDACC__ */
#endif
