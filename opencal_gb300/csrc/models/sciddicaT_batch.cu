/*
 * sciddicaT_batch.cu -- an ensemble of independent SCIDDICA-T instances
 * (calibration ensembles, scenarios) advanced together, forward and adjoint.
 * Every instance is the plain program of OpenCAL/examples/cal_sciddicaT
 * (flat boundary, von Neumann, EP 1 outflows + EP 2 width update,
 * OpenCAL-OMP/examples/calomp_sciddicaT/source/sciddicaT.c), each with its
 * own grid size, DEM, source, p_r and p_epsilon.
 *
 * Layout.  The fields of all instances are packed back to back, one
 * allocation per field; instance b occupies [off_b, off_b + rows_b*cols_b)
 * with off_b a multiple of 32 cells (256 bytes), so every instance's rows
 * start 16-byte aligned when its column count is even.  A device table holds
 * per-instance dimensions and parameters.  Each instance is cut into
 * TW x TH tiles; the tiles of all instances are numbered in one range.
 *
 * Forward.  One launch per step over a packed tile WORK-LIST L_t spanning
 * every instance: a fixed grid of blocks takes tiles from the list, looks up
 * the tile's instance and origin, and runs the fused step on it (the device
 * function of the single-model fused kernel, so every instance stays
 * bit-identical to a run of its own).  h ping-pongs between two buffers.  A
 * tile can only change in a step if it holds a wet cell or borders one, so
 * L_t = dilate(W_{t-1}) u dilate(W_t), with W_t the tiles holding a wet cell
 * of h_t and dilate() the 3 x 3 tile neighbourhood: a tile that processed
 * step t marks its neighbourhood for step t+1 when it held a wet cell before
 * or after the step (an epoch stamp per tile keeps each tile once per list).
 * Invariant: the input buffer of step t holds h_t everywhere, because a tile
 * left out of L_t was unchanged by steps t-1 and t, so both buffers hold its
 * value.  Dry tiles far from the flow cost nothing.
 *
 * Adjoint.  The forward TAPES each processed tile's input values, step
 * after step at offsets the steps chain on the device; the backward walks
 * the rollout in reverse, restoring the taped tiles of step t into the
 * state (turning h_{t+1} into h_t in place: the other tiles did not change)
 * and running the adjoint kernels on the tiles of L_t only (lambda changes
 * only within one cell of a wet cell).  The tape holds every tile a step
 * processed, so it grows with the flow's area times T; when it would not
 * fit in device memory the ensemble falls back to sqrt(T) checkpointing: h
 * is stored every K = ceil(sqrt(T)) steps and the backward recomputes one
 * segment at a time from its checkpoint with the stored work-lists, taping
 * that segment only.  The adjoint of one step is
 * the single-model one (sciddicaT_adjoint.cu): elimination sets recomputed
 * bit-identically from h_t and frozen; lambda is updated in place; per-
 * instance dL/dp_r and dL/dp_eps are block-reduced per tile and added with
 * one atomic per tile (so their summation order is not fixed).
 *
 * Tile shape is chosen by a small autotuner (cal_sdt_batch_autotune): each
 * candidate shape times a forward probe with CUDA events and the fastest is
 * kept for the ensemble.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "sciddicaT_kernels.cuh"

namespace sdtb {

constexpr int T = 256;
constexpr int MAX_INST = 4096;
constexpr long long ALIGN = 32; /* cells */

struct Inst {
    int rows, cols;
    long long off;
    double r, eps;
    long long eps_bits;
    int tiles_x, tiles_y, tile0, pad;
};

struct Shape {
    int tw, th;
};
constexpr int NSHAPES = 5;
static const Shape kShapes[NSHAPES] = {{32, 16}, {64, 16}, {64, 32}, {16, 8}, {32, 8}};

struct Batch {
    int B = 0, steps = 0, K = 0, nseg = 0, shape = 1;
    long long N = 0; /* padded cells */
    int ntiles = 0;
    std::vector<Inst> inst;
    std::vector<long long> offs; /* B + 1 (offs[B] = N) */
    Inst* d_inst = nullptr;
    long long* d_offs = nullptr;
    int* d_tile_inst = nullptr;
    int* stamps = nullptr;
    int* lists = nullptr;  /* (steps + 1) x ntiles */
    int* counts = nullptr; /* steps + 1 */
    std::vector<int> h_counts;
    double *z_dem = nullptr, *z = nullptr, *h0 = nullptr;
    double* hbuf[2] = {nullptr, nullptr};
    double* ckpt = nullptr; /* nseg x N */
    double* tape = nullptr;
    unsigned char* etape = nullptr; /* elimination sets, one byte per taped cell */
    size_t tape_cap = 0;    /* cells (doubles of tape, bytes of etape) */
    double *lam = nullptr, *lamz = nullptr, *g = nullptr, *gz = nullptr, *w = nullptr;
    double* grad = nullptr; /* 2B: dL/dr[0..B), dL/deps[B..2B) */
    double* loss = nullptr; /* B */
    cudaStream_t st = nullptr;
    /* the loss + gradient evaluation recorded once as a CUDA graph and
     * replayed every call: tape offsets computed on the device (toff: the
     * offset of each step's tiles within its segment's tape, need: the
     * largest segment), results copied into pinned host memory (h_out: B
     * losses, 2B gradients, then `need`); valid for the target, dL/dh0
     * buffer, tile shape and tape it was recorded with */
    long long* toff = nullptr;  /* steps + 1 offsets, then need */
    double* h_out = nullptr;    /* pinned: 3B doubles + one long long */
    cudaGraphExec_t gexec = nullptr;
    const double* g_target = nullptr;
    const double* g_gh0 = nullptr;
    const double* g_tape = nullptr;
    const unsigned char* g_etape = nullptr;
    int g_shape = -1;
    long long graph_launches = 0;
    long long graph_nodes = 0;  /* kernel and copy nodes of the recorded evaluation */
    bool use_graph = true;
    /* what the tape holds: the whole rollout (run_full: the backward
     * recomputes nothing) or one sqrt(T) segment at a time.  tape_mode -1
     * chooses by memory: the whole rollout while its tape (plus a quarter)
     * fits in half of the device memory free for it, else segments; 0
     * always segments, 1 always the whole rollout */
    int tape_mode = -1;
    bool run_full = true;
    bool g_full = true;
    long long last_need = 0; /* doubles of tape the last evaluation needed */
};

static int tile_cells(const Batch& bt) { return kShapes[bt.shape].tw * kShapes[bt.shape].th; }

/* a tape (and elimination tape) for `cap` cells; false when out of memory */
static bool grow_tape(Batch& bt, size_t cap)
{
    cudaFree(bt.tape);
    cudaFree(bt.etape);
    bt.tape = nullptr;
    bt.etape = nullptr;
    bt.tape_cap = 0;
    if (cudaMalloc(&bt.tape, cap * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&bt.etape, cap) != cudaSuccess) {
        (void)cudaGetLastError();
        cudaFree(bt.tape);
        bt.tape = nullptr;
        bt.etape = nullptr;
        return false;
    }
    bt.tape_cap = cap;
    return true;
}

/* re-tile every instance for the current shape */
static void drop_graph(Batch& bt)
{
    if (bt.gexec)
        cudaGraphExecDestroy(bt.gexec);
    bt.gexec = nullptr;
}

static bool tiles_for(Batch& bt)
{
    const int tw = kShapes[bt.shape].tw, th = kShapes[bt.shape].th;
    drop_graph(bt); /* the work-list buffers are reallocated */
    std::vector<int> tinst;
    for (int b = 0; b < bt.B; b++) {
        Inst& I = bt.inst[b];
        I.tiles_x = (I.cols + tw - 1) / tw;
        I.tiles_y = (I.rows + th - 1) / th;
        I.tile0 = (int)tinst.size();
        tinst.insert(tinst.end(), (size_t)I.tiles_x * I.tiles_y, b);
    }
    bt.ntiles = (int)tinst.size();
    cudaStreamSynchronize(bt.st);
    cudaFree(bt.d_tile_inst);
    cudaFree(bt.stamps);
    cudaFree(bt.lists);
    bt.d_tile_inst = nullptr;
    bt.stamps = nullptr;
    bt.lists = nullptr;
    bool ok = cudaMalloc(&bt.d_tile_inst, sizeof(int) * tinst.size()) == cudaSuccess &&
              cudaMalloc(&bt.stamps, sizeof(int) * tinst.size()) == cudaSuccess &&
              cudaMalloc(&bt.lists, sizeof(int) * (size_t)bt.ntiles * (bt.steps + 1)) == cudaSuccess;
    if (!ok)
        return false;
    cudaMemcpy(bt.d_tile_inst, tinst.data(), sizeof(int) * tinst.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(bt.d_inst, bt.inst.data(), sizeof(Inst) * bt.B, cudaMemcpyHostToDevice);
    return true;
}

static __device__ __forceinline__ sdt::Params params_of(const Inst& I, const double* z, const double* h, double* hn)
{
    sdt::Params p;
    p.z = z + I.off;
    p.h = h + I.off;
    p.h_next = hn + I.off;
    p.rows = I.rows;
    p.cols = I.cols;
    p.toroidal = 0;
    p.eps = I.eps;
    p.r = I.r;
    p.eps_bits = I.eps_bits;
    return p;
}

/* instance of packed cell c (offsets in shared memory); false on padding */
static __device__ __forceinline__ bool locate(const long long* s_offs, const Inst* inst, int B, long long c, int* b)
{
    int lo = 0, hi = B - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_offs[mid] <= c)
            lo = mid;
        else
            hi = mid - 1;
    }
    *b = lo;
    return c - s_offs[lo] < (long long)inst[lo].rows * inst[lo].cols;
}

/* put tile t into list `list`/`count` for the step whose stamp is `stamp` */
static __device__ __forceinline__ void mark(int* stamps, int* list, int* count, int t, int stamp)
{
    if (stamps[t] != stamp && atomicExch(stamps + t, stamp) != stamp)
        list[atomicAdd(count, 1)] = t;
}

/* One ensemble step over the work-list (list, *count): h -> hn.  With a
 * next list the following step's list is built; with a tape the processed
 * tiles' input values are saved (tile k of the list at tape + k * TW * TH)
 * and, with an elimination tape, each wet cell's elimination set (one byte
 * per cell at the same offsets). */
template <int TW, int TH>
__global__ void __launch_bounds__(sdt::THREADS) k_step(const Inst* __restrict__ inst, const int* __restrict__ tile_inst,
                                                       const double* __restrict__ z, const double* __restrict__ h,
                                                       double* __restrict__ hn, const int* __restrict__ list,
                                                       const int* __restrict__ count, int* list_next, int* count_next,
                                                       int* stamps, int stamp, double* __restrict__ tape,
                                                       unsigned char* __restrict__ etape,
                                                       const long long* __restrict__ toff, long long* toff_next,
                                                       long long tape_cap)
{
    extern __shared__ __align__(16) double smem[];
    using TL = sdt::Tile<TW, TH>;
    const int n = *count;
    if (toff) {
        /* the step's tiles at the device-computed offset; steps that do not
         * fit are not taped (the host sees `need` and runs again with a
         * larger tape).  When the whole rollout is taped the step also
         * places the next one: toff[t + 1] = toff[t] + its tiles. */
        const long long off = *toff;
        const long long end = off + (long long)n * (TW * TH);
        if (toff_next && blockIdx.x == 0 && threadIdx.x == 0)
            *toff_next = end;
        if (!tape || end > tape_cap) {
            tape = nullptr;
            etape = nullptr;
        } else {
            tape += off;
            etape = etape ? etape + off : nullptr;
        }
    }
    for (int k = blockIdx.x; k < n; k += gridDim.x) {
        const int t = list[k];
        const Inst I = inst[tile_inst[t]];
        const int lt = t - I.tile0;
        const int ty = lt / I.tiles_x, tx = lt - ty * I.tiles_x;
        const sdt::Params p = params_of(I, z, h, hn);
        const int wet = sdt::fused_tile<TW, TH, true>(p, ty * TH, tx * TW, smem, false,
                                                      etape ? etape + (size_t)k * (TW * TH) : nullptr);
        if (tape) {
            /* the tile's input h is still in shared memory (load region, +2 ring) */
            const double* sh = smem + TL::R2W * TL::R2H;
            double* dst = tape + (size_t)k * (TW * TH);
            for (int c = threadIdx.x; c < TW * TH; c += sdt::THREADS) {
                const int a = c / TW, b = c - a * TW;
                dst[c] = sh[(a + 2) * TL::R2W + b + 2];
            }
        }
        if (list_next && wet && threadIdx.x < 9) {
            const int y = ty + (int)threadIdx.x / 3 - 1, x = tx + (int)threadIdx.x % 3 - 1;
            if ((unsigned)y < (unsigned)I.tiles_y && (unsigned)x < (unsigned)I.tiles_x)
                mark(stamps, list_next, count_next, I.tile0 + y * I.tiles_x + x, stamp);
        }
        __syncthreads(); /* shared memory is reused by the next tile */
    }
}

/* the taped tiles of one step back into the state: h_{t+1} -> h_t */
template <int TW, int TH>
__global__ void __launch_bounds__(sdt::THREADS) k_restore(const Inst* __restrict__ inst,
                                                          const int* __restrict__ tile_inst,
                                                          const int* __restrict__ list, const int* __restrict__ count,
                                                          const double* __restrict__ tape, double* __restrict__ h,
                                                          const long long* __restrict__ toff, long long tape_cap)
{
    const int n = *count;
    if (toff) {
        const long long off = *toff;
        if (off + (long long)n * (TW * TH) > tape_cap)
            return; /* not taped (see k_step): this evaluation is discarded */
        tape += off;
    }
    for (int k = blockIdx.x; k < n; k += gridDim.x) {
        const int t = list[k];
        const Inst I = inst[tile_inst[t]];
        const int lt = t - I.tile0;
        const int ty = lt / I.tiles_x, tx = lt - ty * I.tiles_x;
        const double* src = tape + (size_t)k * (TW * TH);
        for (int c = threadIdx.x; c < TW * TH; c += sdt::THREADS) {
            const int a = c / TW, b = c - a * TW;
            const int i = ty * TH + a, j = tx * TW + b;
            if (i < I.rows && j < I.cols)
                h[I.off + (long long)i * I.cols + j] = src[c];
        }
    }
}

/* z after the initialisation (z_dem - h0 where h0 > 0), both h buffers = h0
 * with -0 made +0 (the first reference step adds 0.0 to every cell), and
 * list L_0 = the 3 x 3 tiles around every tile holding a wet cell */
__global__ void k_init(const Inst* __restrict__ inst, const long long* __restrict__ offs, int B, long long N, int tw,
                       int th, const double* __restrict__ z_dem, const double* __restrict__ h0, double* __restrict__ z,
                       double* __restrict__ h_a, double* __restrict__ h_b, int* stamps, int* list0, int* count0)
{
    extern __shared__ long long s_offs[];
    for (int k = threadIdx.x; k <= B; k += blockDim.x)
        s_offs[k] = offs[k];
    __syncthreads();
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        int b;
        if (!locate(s_offs, inst, B, c, &b)) {
            z[c] = 0.0;
            h_a[c] = 0.0;
            h_b[c] = 0.0;
            continue;
        }
        const Inst I = inst[b];
        const double hv = h0[c];
        z[c] = hv > 0.0 ? z_dem[c] - hv : z_dem[c];
        const double hc = sdt::plus_zero(hv);
        h_a[c] = hc;
        h_b[c] = hc;
        if (sdt::is_wet(hc, I.eps_bits)) {
            const long long lc = c - I.off;
            const int i = (int)(lc / I.cols), j = (int)(lc - (long long)i * I.cols);
            const int ty = i / th, tx = j / tw;
            for (int q = 0; q < 9; q++) {
                const int y = ty + q / 3 - 1, x = tx + q % 3 - 1;
                if ((unsigned)y < (unsigned)I.tiles_y && (unsigned)x < (unsigned)I.tiles_x)
                    mark(stamps, list0, count0, I.tile0 + y * I.tiles_x + x, 1);
            }
        }
    }
}

/* dL/dh_T = 2 (h_T - target), lambda_z = 0, and the per-instance loss */
__global__ void k_loss(const Inst* __restrict__ inst, const long long* __restrict__ offs, int B, long long N,
                       const double* __restrict__ hT, const double* __restrict__ tgt, double* __restrict__ lam,
                       double* __restrict__ lamz, double* __restrict__ loss)
{
    extern __shared__ long long s_offs[];
    for (int k = threadIdx.x; k <= B; k += blockDim.x)
        s_offs[k] = offs[k];
    __syncthreads();
    for (long long c0 = blockIdx.x * (long long)blockDim.x; c0 < N; c0 += (long long)gridDim.x * blockDim.x) {
        const long long c = c0 + threadIdx.x;
        double d2 = 0.0;
        int b = 0;
        bool valid = false;
        if (c < N) {
            valid = locate(s_offs, inst, B, c, &b);
            const double d = valid ? hT[c] - tgt[c] : 0.0;
            lam[c] = 2.0 * d;
            lamz[c] = 0.0;
            d2 = d * d;
        }
        const int b0 = __shfl_sync(0xffffffffu, b, 0);
        if (__all_sync(0xffffffffu, b == b0 || !valid)) {
            for (int o = 16; o > 0; o >>= 1)
                d2 += __shfl_down_sync(0xffffffffu, d2, o);
            if ((threadIdx.x & 31) == 0)
                atomicAdd(loss + b0, d2);
        } else if (valid) {
            atomicAdd(loss + b, d2);
        }
    }
}

/* neighbour n = 1..4 (north, west, east, south) of (i, j) in instance I; false outside (flat) */
static __device__ __forceinline__ bool nbr(const Inst& I, int i, int j, int n, long long* c)
{
    const int a = i + (n == 1 ? -1 : (n == 4 ? 1 : 0));
    const int b = j + (n == 2 ? -1 : (n == 3 ? 1 : 0));
    if ((unsigned)a >= (unsigned)I.rows || (unsigned)b >= (unsigned)I.cols)
        return false;
    *c = I.off + (long long)a * I.cols + b;
    return true;
}

/* the block's sums of a and b, in thread 0 (warp shuffles, then thread 0
 * over the warps in order); one barrier: s_red is next written after the
 * barriers that open the block's next tile */
static __device__ __forceinline__ void block_sum2(double& a, double& b, double2* s_red)
{
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0)
        s_red[threadIdx.x >> 5] = make_double2(a, b);
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0.0, sb = 0.0;
        for (int q = 0; q < T / 32; q++) {
            sa += s_red[q].x;
            sb += s_red[q].y;
        }
        a = sa;
        b = sb;
    }
}

/* adjoint coefficients g, gz, w of the wet cells of the listed tiles (the
 * single-model k_coeffs; k_gather reads them at wet cells only), and the
 * tiles' contributions to dL/dr, dL/deps.  The wet cells of a tile are
 * compacted first.  The elimination sets are the forward's, read from the
 * elimination tape (etape, at the step's offset *toff when toff is given),
 * so the minimisation is not iterated again: the average is the one sum
 * over the kept cells and one division, the last pass of the forward's
 * iteration, bit for bit.  A step that was not taped (the evaluation is
 * discarded and run again with a larger tape) is skipped. */
template <int TW, int TH>
__global__ void __launch_bounds__(T) k_coeffs(const Inst* __restrict__ inst, const int* __restrict__ tile_inst,
                                              const int* __restrict__ list, const int* __restrict__ count, long long N,
                                              const double* __restrict__ z, const double* __restrict__ h,
                                              const double* __restrict__ lam, double* __restrict__ g,
                                              double* __restrict__ gz, double* __restrict__ w,
                                              double* __restrict__ grad, int B, const unsigned char* __restrict__ etape,
                                              const long long* __restrict__ toff, long long tape_cap)
{
    __shared__ double2 s_red2[T / 32];
    __shared__ unsigned short s_wet[TW * TH];
    __shared__ int s_n;
    const int n = *count;
    if (etape && toff) {
        const long long off = *toff;
        etape = off + (long long)n * (TW * TH) > tape_cap ? nullptr : etape + off;
    }
    if (!etape)
        return;
    for (int k = blockIdx.x; k < n; k += gridDim.x) {
        const int t = list[k];
        const int bi = tile_inst[t];
        const Inst I = inst[bi];
        const int lt = t - I.tile0;
        const int ty = lt / I.tiles_x, tx = lt - ty * I.tiles_x;
        if (threadIdx.x == 0)
            s_n = 0;
        __syncthreads();
        for (int q0 = 0; q0 < TW * TH; q0 += T) {
            const int q = q0 + threadIdx.x;
            const int i = ty * TH + q / TW, j = tx * TW + q % TW;
            const bool wet = q < TW * TH && i < I.rows && j < I.cols &&
                             sdt::is_wet(h[I.off + (long long)i * I.cols + j], I.eps_bits);
            sdt::warp_append_shared(wet, q, s_wet, &s_n);
        }
        __syncthreads();
        const int nw = s_n;
        double pr = 0.0, pe = 0.0;
        for (int e = threadIdx.x; e < nw; e += T) {
            const int q = s_wet[e];
            const int i = ty * TH + q / TW, j = tx * TW + q % TW;
            const long long c = I.off + (long long)i * I.cols + j;
            const double hc = h[c];
            double gc = 0.0, gzc = 0.0, wc[4] = {0.0, 0.0, 0.0, 0.0};
            double u[5], lnb[4];
            u[0] = z[c] + I.eps;
#pragma unroll
            for (int d = 0; d < 4; d++) {
                long long cn = 0;
                const bool in = nbr(I, i, j, d + 1, &cn);
                u[d + 1] = in ? z[cn] + h[cn] : 0.0 + 0.0;
                lnb[d] = in ? lam[cn] : 0.0;
            }
            const double m = hc - I.eps;
            const unsigned elim = etape[(size_t)k * (TW * TH) + q];
            double avg = m;
            int cnt = 0;
#pragma unroll
            for (int d = 0; d < 5; d++)
                if (!(elim & (1u << d))) {
                    avg += u[d];
                    cnt++;
                }
            if (cnt != 0)
                avg = cal_div_small(avg, cnt);
            const unsigned a_set = (~elim) & 31u;
            const int kk = __popc(a_set);
            if (kk > 0) {
                const double lc = lam[c];
                double S = 0.0, lf[4];
#pragma unroll
                for (int d = 0; d < 4; d++) {
                    lf[d] = 0.0;
                    if (a_set & (1u << (d + 1))) {
                        lf[d] = lnb[d] - lc;
                        S += lf[d];
                        pr += lf[d] * (avg - u[d + 1]);
                    }
                }
                gc = cal_div_small(I.r, kk) * S; /* = (I.r / kk) * S: exact division by 1..5 on the integer pipe */
                gzc = (a_set & 1u) ? gc : 0.0;
                pe += cal_div_small(S * I.r * ((a_set & 1u) ? 0.0 : -1.0), kk);
#pragma unroll
                for (int d = 0; d < 4; d++)
                    if (a_set & (1u << (d + 1)))
                        wc[d] = gc - I.r * lf[d];
            }
            g[c] = gc;
            gz[c] = gzc;
#pragma unroll
            for (int d = 0; d < 4; d++)
                w[d * N + c] = wc[d];
        }
        block_sum2(pr, pe, s_red2);
        const double sr = pr, se = pe;
        if (threadIdx.x == 0) {
            if (sr != 0.0)
                atomicAdd(grad + bi, sr);
            if (se != 0.0)
                atomicAdd(grad + B + bi, se);
        }
    }
}

/* lambda_t = lambda_{t+1} + g + the wet neighbours' w (in place), and
 * lambda_z; coefficients are read only at wet cells, where this step's
 * k_coeffs wrote them (a wet cell's tile is always in the list) */
template <int TW, int TH>
__global__ void __launch_bounds__(T) k_gather(const Inst* __restrict__ inst, const int* __restrict__ tile_inst,
                                              const int* __restrict__ list, const int* __restrict__ count, long long N,
                                              const double* __restrict__ h, const double* __restrict__ g,
                                              const double* __restrict__ gz, const double* __restrict__ w,
                                              double* __restrict__ lam, double* __restrict__ lamz)
{
    const int n = *count;
    for (int k = blockIdx.x; k < n; k += gridDim.x) {
        const int t = list[k];
        const Inst I = inst[tile_inst[t]];
        const int lt = t - I.tile0;
        const int ty = lt / I.tiles_x, tx = lt - ty * I.tiles_x;
        /* two cells a thread per pass, their loads issued together (the
         * pass is bound by the latency of these loads); each cell's sums
         * keep their order */
        for (int q0 = threadIdx.x; q0 < TW * TH; q0 += 2 * T) {
            /* first the wet flags of both cells and their neighbours (ten
             * loads in flight), then the coefficients of the wet ones */
            unsigned wet[2] = {0u, 0u}; /* bit d: neighbour d + 1; bit 4: the cell */
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int q = q0 + u * T;
                const int i = ty * TH + q / TW, j = tx * TW + q % TW;
                if (q < TW * TH && i < I.rows && j < I.cols) {
                    long long cn = 0;
#pragma unroll
                    for (int d = 0; d < 4; d++)
                        if (nbr(I, i, j, d + 1, &cn) && sdt::is_wet(h[cn], I.eps_bits))
                            wet[u] |= 1u << d;
                    if (sdt::is_wet(h[I.off + (long long)i * I.cols + j], I.eps_bits))
                        wet[u] |= 16u;
                }
            }
#pragma unroll
            for (int u = 0; u < 2; u++) {
                if (!wet[u])
                    continue; /* nothing is added: lambda stays (the arrays are far
                               * larger than L2, so the skipped read and write are
                               * DRAM bytes) */
                const int q = q0 + u * T;
                const int i = ty * TH + q / TW, j = tx * TW + q % TW;
                const long long c = I.off + (long long)i * I.cols + j;
                double from_nb = 0.0;
                long long cn = 0;
                /* x is neighbour opp(d) of its neighbour d: north<->south,
                 * west<->east, so neighbour d contributes w of plane 3 - d */
#pragma unroll
                for (int d = 0; d < 4; d++)
                    if ((wet[u] >> d) & 1u) {
                        nbr(I, i, j, d + 1, &cn);
                        from_nb += w[(3 - d) * N + cn];
                    }
                double gc = 0.0, gzc = 0.0;
                if (wet[u] & 16u) {
                    gc = g[c];
                    gzc = gz[c];
                }
                lam[c] = lam[c] + gc + from_nb;
                lamz[c] += gzc + from_nb;
            }
        }
    }
}

__global__ void k_final_grad(const double* __restrict__ h0, const double* __restrict__ lam,
                             const double* __restrict__ lamz, double* __restrict__ g_h0, long long n)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        g_h0[c] = lam[c] - (h0[c] > 0.0 ? lamz[c] : 0.0);
}

/* Tape layout on the device: one warp per segment of K <= 32 steps scans
 * the segment's work-list sizes (counts[t] tiles of tc cells each) into the
 * offsets toff[t]; toff[steps] = the largest segment's total (the tape
 * size this evaluation needs). */
__global__ void k_tape_offsets(const int* __restrict__ counts, int steps, int K, int tc, long long* toff)
{
    __shared__ long long s_need;
    if (threadIdx.x == 0)
        s_need = 0;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nseg = (steps + K - 1) / K;
    for (int sg = warp; sg < nseg; sg += blockDim.x >> 5) {
        const int t = sg * K + lane;
        const bool in = lane < K && t < steps;
        const long long v = in ? (long long)counts[t] * tc : 0;
        long long incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
                incl += y;
        }
        if (in)
            toff[t] = incl - v;
        const long long total = __shfl_sync(0xffffffffu, incl, 31);
        if (lane == 0)
            atomicMax((unsigned long long*)&s_need, (unsigned long long)total);
    }
    __syncthreads();
    if (threadIdx.x == 0)
        toff[steps] = s_need;
}

static int dense_grid(long long n)
{
    long long b = (n + T - 1) / T;
    return (int)(b > 152 * 16 ? 152 * 16 : (b < 1 ? 1 : b));
}

/* a resident grid for the step kernel: SMs x blocks per SM */
template <int TW, int TH>
static int step_grid()
{
    static int blocks = 0;
    if (!blocks) {
        const int smem = (int)sdt::Tile<TW, TH>::smem_bytes;
        cudaFuncSetAttribute(k_step<TW, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        int per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step<TW, TH>, sdt::THREADS, smem);
        int dev = 0, sms = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        blocks = sms * (per_sm > 0 ? per_sm : 1);
    }
    return blocks;
}

/* step t: list L_t -> (mark ? L_{t+1}) */
template <int TW, int TH>
/* taped: the step's tiles go to the tape (and their elimination sets to the
 * elimination tape) at the device offset *toff, or at host_off when toff is
 * NULL; toff_next: where the step chains the next step's offset */
static void launch_step(Batch& bt, int t, const double* h, double* hn, bool mark, bool taped = false,
                        const long long* toff = nullptr, long long* toff_next = nullptr, size_t host_off = 0)
{
    const size_t nt = (size_t)bt.ntiles;
    double* tape = taped && bt.tape ? bt.tape + host_off : nullptr;
    unsigned char* etape = taped && bt.etape ? bt.etape + host_off : nullptr;
    k_step<TW, TH><<<step_grid<TW, TH>(), sdt::THREADS, sdt::Tile<TW, TH>::smem_bytes, bt.st>>>(
        bt.d_inst, bt.d_tile_inst, bt.z, h, hn, bt.lists + nt * t, bt.counts + t,
        mark ? bt.lists + nt * (t + 1) : nullptr, bt.counts + t + 1, bt.stamps, t + 2, tape, etape, toff,
        toff_next, (long long)bt.tape_cap);
}

template <int TW, int TH>
static void launch_restore(Batch& bt, int t, const double* tape, double* h, const long long* toff = nullptr)
{
    k_restore<TW, TH><<<152 * 8, sdt::THREADS, 0, bt.st>>>(bt.d_inst, bt.d_tile_inst, bt.lists + (size_t)bt.ntiles * t,
                                                            bt.counts + t, tape, h, toff, (long long)bt.tape_cap);
}

template <int TW, int TH>
static void launch_adjoint(Batch& bt, int t, const double* h, const long long* toff = nullptr, size_t host_off = 0)
{
    const int* list = bt.lists + (size_t)bt.ntiles * t;
    k_coeffs<TW, TH><<<152 * 8, T, 0, bt.st>>>(bt.d_inst, bt.d_tile_inst, list, bt.counts + t, bt.N, bt.z, h, bt.lam,
                                                bt.g, bt.gz, bt.w, bt.grad, bt.B,
                                                bt.etape ? bt.etape + host_off : nullptr, toff,
                                                (long long)bt.tape_cap);
    k_gather<TW, TH><<<152 * 8, T, 0, bt.st>>>(bt.d_inst, bt.d_tile_inst, list, bt.counts + t, bt.N, h, bt.g, bt.gz,
                                                bt.w, bt.lam, bt.lamz);
}

#define SDTB_DISPATCH(batch, fn, ...)                          \
    switch ((batch).shape) {                                   \
    case 0: fn<32, 16>(__VA_ARGS__); break;                    \
    case 1: fn<64, 16>(__VA_ARGS__); break;                    \
    case 3: fn<16, 8>(__VA_ARGS__); break;                     \
    case 4: fn<32, 8>(__VA_ARGS__); break;                     \
    default: fn<64, 32>(__VA_ARGS__); break;                   \
    }

/* forward over `steps` steps from h0; checkpoints every K steps when keep;
 * with `taped`, every step's tiles go to the tape at device-chained offsets
 * (toff[0] = 0, toff[t + 1] = toff[t] + the tiles of step t) */
static void forward(Batch& bt, int steps, bool keep, bool taped = false)
{
    const size_t nb = (size_t)bt.N * sizeof(double);
    const int tw = kShapes[bt.shape].tw, th = kShapes[bt.shape].th;
    cudaMemsetAsync(bt.stamps, 0, sizeof(int) * bt.ntiles, bt.st);
    cudaMemsetAsync(bt.counts, 0, sizeof(int) * (bt.steps + 1), bt.st);
    k_init<<<dense_grid(bt.N), T, sizeof(long long) * (bt.B + 1), bt.st>>>(bt.d_inst, bt.d_offs, bt.B, bt.N, tw, th,
                                                                           bt.z_dem, bt.h0, bt.z, bt.hbuf[0],
                                                                           bt.hbuf[1], bt.stamps, bt.lists, bt.counts);
    if (taped)
        cudaMemsetAsync(bt.toff, 0, sizeof(long long), bt.st);
    for (int t = 0; t < steps; t++) {
        if (keep && t % bt.K == 0)
            cudaMemcpyAsync(bt.ckpt + (size_t)(t / bt.K) * bt.N, bt.hbuf[t & 1], nb, cudaMemcpyDeviceToDevice, bt.st);
        if (taped) {
            SDTB_DISPATCH(bt, launch_step, bt, t, bt.hbuf[t & 1], bt.hbuf[(t + 1) & 1], true, true, bt.toff + t,
                          bt.toff + t + 1);
        } else {
            SDTB_DISPATCH(bt, launch_step, bt, t, bt.hbuf[t & 1], bt.hbuf[(t + 1) & 1], true);
        }
    }
}

static void destroy(Batch* bt)
{
    if (bt->st)
        cudaStreamSynchronize(bt->st);
    drop_graph(*bt);
    cudaFree(bt->toff);
    if (bt->h_out)
        cudaFreeHost(bt->h_out);
    void* ptrs[] = {bt->d_inst, bt->d_offs, bt->d_tile_inst, bt->stamps, bt->lists, bt->counts, bt->z_dem,
                    bt->z,      bt->h0,     bt->hbuf[0],      bt->hbuf[1], bt->ckpt, bt->tape,   bt->etape, bt->lam,
                    bt->lamz,   bt->g,      bt->gz,           bt->w,      bt->grad,  bt->loss};
    for (void* p : ptrs)
        cudaFree(p);
    if (bt->st)
        cudaStreamDestroy(bt->st);
    delete bt;
}

} // namespace sdtb

using sdtb::Batch;

/* Create an ensemble of B instances.  dims[2b], dims[2b+1] = rows, cols;
 * params[2b], params[2b+1] = p_r, p_eps; z_dem, h0: host arrays holding the
 * instances' rows*cols values back to back (row-major, unpadded); `steps`
 * per rollout.  NULL on a bad argument or when device memory runs out. */
extern "C" void* cal_sdt_batch_create(int B, const int* dims, const double* params, const double* z_dem_host,
                                      const double* h0_host, int steps)
{
    if (B <= 0 || B > sdtb::MAX_INST || steps < 0 || !dims || !params || !z_dem_host || !h0_host)
        return nullptr;
    Batch* bt = new Batch();
    bt->B = B;
    bt->steps = steps;
    bt->K = (int)ceil(sqrt((double)(steps > 0 ? steps : 1)));
    bt->nseg = steps > 0 ? (steps + bt->K - 1) / bt->K : 1;
    bt->offs.assign(B + 1, 0);
    for (int b = 0; b < B; b++) {
        sdtb::Inst I;
        memset(&I, 0, sizeof(I));
        I.rows = dims[2 * b];
        I.cols = dims[2 * b + 1];
        if (I.rows <= 0 || I.cols <= 0) {
            delete bt;
            return nullptr;
        }
        I.off = bt->offs[b];
        I.r = params[2 * b];
        I.eps = params[2 * b + 1];
        memcpy(&I.eps_bits, &I.eps, sizeof(double));
        bt->inst.push_back(I);
        const long long n = (long long)I.rows * I.cols;
        bt->offs[b + 1] = bt->offs[b] + (n + sdtb::ALIGN - 1) / sdtb::ALIGN * sdtb::ALIGN;
    }
    bt->N = bt->offs[B];
    const size_t nb = (size_t)bt->N * sizeof(double);
    bool ok = cudaStreamCreateWithFlags(&bt->st, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&bt->d_inst, sizeof(sdtb::Inst) * B) == cudaSuccess &&
              cudaMalloc(&bt->d_offs, sizeof(long long) * (B + 1)) == cudaSuccess &&
              cudaMalloc(&bt->counts, sizeof(int) * (steps + 1)) == cudaSuccess &&
              cudaMalloc(&bt->z_dem, nb) == cudaSuccess && cudaMalloc(&bt->z, nb) == cudaSuccess &&
              cudaMalloc(&bt->h0, nb) == cudaSuccess && cudaMalloc(&bt->hbuf[0], nb) == cudaSuccess &&
              cudaMalloc(&bt->hbuf[1], nb) == cudaSuccess && cudaMalloc(&bt->ckpt, nb * bt->nseg) == cudaSuccess &&
              cudaMalloc(&bt->lam, nb) == cudaSuccess && cudaMalloc(&bt->lamz, nb) == cudaSuccess &&
              cudaMalloc(&bt->g, nb) == cudaSuccess && cudaMalloc(&bt->gz, nb) == cudaSuccess &&
              cudaMalloc(&bt->w, 4 * nb) == cudaSuccess &&
              cudaMalloc(&bt->grad, 2 * B * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&bt->loss, B * sizeof(double)) == cudaSuccess;
    if (ok) {
        cudaMemcpy(bt->d_offs, bt->offs.data(), sizeof(long long) * (B + 1), cudaMemcpyHostToDevice);
        cudaMemset(bt->z_dem, 0, nb);
        cudaMemset(bt->h0, 0, nb);
        size_t src = 0;
        for (int b = 0; b < B; b++) {
            const size_t n = (size_t)bt->inst[b].rows * bt->inst[b].cols;
            cudaMemcpy(bt->z_dem + bt->offs[b], z_dem_host + src, n * sizeof(double), cudaMemcpyHostToDevice);
            cudaMemcpy(bt->h0 + bt->offs[b], h0_host + src, n * sizeof(double), cudaMemcpyHostToDevice);
            src += n;
        }
        ok = sdtb::tiles_for(*bt) && cudaGetLastError() == cudaSuccess;
    }
    if (!ok) {
        fprintf(stderr, "opencal-gb300: cal_sdt_batch_create: out of device memory\n");
        sdtb::destroy(bt);
        return nullptr;
    }
    return bt;
}

extern "C" void cal_sdt_batch_destroy(void* handle)
{
    if (handle)
        sdtb::destroy((Batch*)handle);
}

/* padded cell count and the B + 1 instance offsets of the device layout */
extern "C" long long cal_sdt_batch_cells(void* handle, long long* offsets)
{
    Batch* bt = (Batch*)handle;
    if (offsets)
        memcpy(offsets, bt->offs.data(), sizeof(long long) * (bt->B + 1));
    return bt->N;
}

extern "C" void* cal_sdt_batch_stream(void* handle) { return ((Batch*)handle)->st; }
extern "C" int cal_sdt_batch_shape(void* handle) { return ((Batch*)handle)->shape; }

/* replace the per-instance parameters (host array of 2B doubles: p_r, p_eps) */
extern "C" int cal_sdt_batch_set_params(void* handle, const double* params)
{
    Batch* bt = (Batch*)handle;
    for (int b = 0; b < bt->B; b++) {
        bt->inst[b].r = params[2 * b];
        bt->inst[b].eps = params[2 * b + 1];
        memcpy(&bt->inst[b].eps_bits, &bt->inst[b].eps, sizeof(double));
    }
    cudaStreamSynchronize(bt->st);
    return (int)cudaMemcpy(bt->d_inst, bt->inst.data(), sizeof(sdtb::Inst) * bt->B, cudaMemcpyHostToDevice);
}

/* Forward rollout of every instance (`steps` steps); h_T copied into hT (a
 * device array in the padded layout, or NULL).  Asynchronous on the
 * ensemble's stream. */
extern "C" int cal_sdt_batch_forward(void* handle, double* hT)
{
    Batch* bt = (Batch*)handle;
    sdtb::forward(*bt, bt->steps, false);
    if (hT)
        cudaMemcpyAsync(hT, bt->hbuf[bt->steps & 1], (size_t)bt->N * sizeof(double), cudaMemcpyDeviceToDevice, bt->st);
    return (int)cudaGetLastError();
}

/* Tiles processed by each step of the last rollout (steps + 1 counts: the
 * list built for step t, t in [0, steps]).  Synchronises. */
extern "C" int cal_sdt_batch_active_tiles(void* handle, int* out)
{
    Batch* bt = (Batch*)handle;
    cudaStreamSynchronize(bt->st);
    return (int)cudaMemcpy(out, bt->counts, sizeof(int) * (bt->steps + 1), cudaMemcpyDeviceToHost);
}

namespace sdtb {

/* The whole loss + gradient evaluation queued on the ensemble's stream with
 * the tape layout computed on the device (k_tape_offsets): forward with
 * checkpoints, loss, layout, the reverse sweep segment by segment, dL/dh0,
 * and the losses, gradients and the tape size needed copied into the
 * pinned h_out.  Nothing in it waits for the host, so it can be recorded. */
static void queue_loss_grad(Batch& bt, const double* target, double* g_h0)
{
    const size_t nb = (size_t)bt.N * sizeof(double);
    cudaStream_t st = bt.st;
    forward(bt, bt.steps, !bt.run_full, bt.run_full);
    cudaMemsetAsync(bt.loss, 0, bt.B * sizeof(double), st);
    cudaMemsetAsync(bt.grad, 0, 2 * bt.B * sizeof(double), st);
    k_loss<<<dense_grid(bt.N), T, sizeof(long long) * (bt.B + 1), st>>>(bt.d_inst, bt.d_offs, bt.B, bt.N,
                                                                         bt.hbuf[bt.steps & 1], target, bt.lam,
                                                                         bt.lamz, bt.loss);
    if (bt.run_full) {
        /* the whole rollout is on the tape: no recomputation, the state
         * buffer holding h_T is walked back one step at a time */
        double* X = bt.hbuf[bt.steps & 1];
        for (int t = bt.steps - 1; t >= 0; t--) {
            SDTB_DISPATCH(bt, launch_restore, bt, t, bt.tape, X, bt.toff + t);
            SDTB_DISPATCH(bt, launch_adjoint, bt, t, X, bt.toff + t);
        }
    } else {
        k_tape_offsets<<<1, 1024, 0, st>>>(bt.counts, bt.steps, bt.K, tile_cells(bt), bt.toff);
    }
    for (int s = bt.run_full ? -1 : bt.nseg - 1; s >= 0; s--) {
        const int t0 = s * bt.K, t1 = std::min(t0 + bt.K, bt.steps);
        if (t1 <= t0)
            continue;
        cudaMemcpyAsync(bt.hbuf[0], bt.ckpt + (size_t)s * bt.N, nb, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(bt.hbuf[1], bt.ckpt + (size_t)s * bt.N, nb, cudaMemcpyDeviceToDevice, st);
        for (int t = t0; t < t1; t++)
            SDTB_DISPATCH(bt, launch_step, bt, t, bt.hbuf[(t - t0) & 1], bt.hbuf[(t - t0 + 1) & 1], false, true,
                          bt.toff + t);
        double* X = bt.hbuf[(t1 - t0) & 1];
        for (int t = t1 - 1; t >= t0; t--) {
            SDTB_DISPATCH(bt, launch_restore, bt, t, bt.tape, X, bt.toff + t);
            SDTB_DISPATCH(bt, launch_adjoint, bt, t, X, bt.toff + t);
        }
    }
    if (g_h0)
        k_final_grad<<<dense_grid(bt.N), T, 0, st>>>(bt.h0, bt.lam, bt.lamz, g_h0, bt.N);
    cudaMemcpyAsync(bt.h_out, bt.loss, bt.B * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(bt.h_out + bt.B, bt.grad, 2 * bt.B * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(bt.h_out + 3 * bt.B, bt.toff + bt.steps, sizeof(long long), cudaMemcpyDeviceToHost, st);
}

/* One evaluation queued with the tape layout computed on the device: as one
 * launch of the recorded graph (recorded again when the target, the dL/dh0
 * buffer, the tile shape, the tape or what it holds changed), or launch by
 * launch.  When the tape was too small the evaluation is discarded, the tape
 * grown to the size the device reported (plus a quarter) and the evaluation
 * run again; in the memory-chosen mode a whole-rollout tape that would not
 * fit switches the ensemble to segments.  0 on success; SEGMENTS_ON_HOST
 * when segments of more than 32 steps are needed (the caller runs them with
 * the layout computed on the host). */
constexpr int SEGMENTS_ON_HOST = -2;

static int loss_grad_device(Batch& bt, const double* target, double* loss_out, double* grad_out, double* g_h0)
{
    cudaStream_t st = bt.st;
    if (!bt.toff && cudaMalloc(&bt.toff, sizeof(long long) * (bt.steps + 1)) != cudaSuccess)
        return (int)cudaErrorMemoryAllocation;
    if (!bt.h_out && cudaMallocHost(&bt.h_out, sizeof(double) * (3 * bt.B + 1)) != cudaSuccess)
        return (int)cudaErrorMemoryAllocation;
    for (int attempt = 0; attempt < 4; attempt++) {
        if (!bt.run_full && bt.K > 32)
            return SEGMENTS_ON_HOST;
        if (bt.use_graph) {
            if (!bt.gexec || bt.g_target != target || bt.g_gh0 != g_h0 || bt.g_shape != bt.shape ||
                bt.g_tape != bt.tape || bt.g_etape != bt.etape || bt.g_full != bt.run_full) {
                drop_graph(bt);
                cudaGraph_t graph = nullptr;
                if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                    return (int)cudaGetLastError();
                queue_loss_grad(bt, target, g_h0);
                cudaError_t e = cudaStreamEndCapture(st, &graph);
                if (e != cudaSuccess || !graph) {
                    (void)cudaGetLastError();
                    return (int)(e != cudaSuccess ? e : cudaErrorUnknown);
                }
                e = cudaGraphInstantiate(&bt.gexec, graph, 0);
                size_t nodes = 0;
                cudaGraphGetNodes(graph, nullptr, &nodes);
                bt.graph_nodes = (long long)nodes;
                cudaGraphDestroy(graph);
                if (e != cudaSuccess)
                    return (int)e;
                bt.g_target = target;
                bt.g_gh0 = g_h0;
                bt.g_shape = bt.shape;
                bt.g_tape = bt.tape;
                bt.g_etape = bt.etape;
                bt.g_full = bt.run_full;
            }
            if (cudaGraphLaunch(bt.gexec, st) != cudaSuccess)
                return (int)cudaGetLastError();
            bt.graph_launches++;
        } else
            queue_loss_grad(bt, target, g_h0);
        if (cudaStreamSynchronize(st) != cudaSuccess)
            return (int)cudaGetLastError();
        long long need = 0;
        memcpy(&need, bt.h_out + 3 * bt.B, sizeof(need));
        bt.last_need = need;
        if (need <= (long long)bt.tape_cap) {
            if (loss_out)
                memcpy(loss_out, bt.h_out, bt.B * sizeof(double));
            if (grad_out)
                for (int b = 0; b < bt.B; b++) {
                    grad_out[2 * b] = bt.h_out[bt.B + b];
                    grad_out[2 * b + 1] = bt.h_out[2 * bt.B + b];
                }
            return 0;
        }
        const size_t cap = (size_t)(need + need / 4);
        if (bt.run_full && bt.tape_mode < 0) {
            size_t free_b = 0, total_b = 0;
            cudaMemGetInfo(&free_b, &total_b);
            if (cap * (sizeof(double) + 1) > (free_b + bt.tape_cap * (sizeof(double) + 1)) / 2) {
                bt.run_full = false; /* the segments' tape is about sqrt(T) times smaller */
                continue;
            }
        }
        if (!grow_tape(bt, cap)) {
            if (bt.run_full && bt.tape_mode < 0) {
                bt.run_full = false;
                continue;
            }
            fprintf(stderr, "opencal-gb300: cal_sdt_batch_loss_grad: out of device memory for the tape\n");
            return (int)cudaErrorMemoryAllocation;
        }
    }
    return (int)cudaErrorUnknown;
}

} // namespace sdtb

/* Loss L_b = sum over instance b of (h_T - target)^2 and its gradients:
 * forward with checkpoints, then the adjoint.  target: device array in the
 * padded layout.  loss_out[B], grad_out[2B] (dL/dp_r, dL/dp_eps of each
 * instance, interleaved): host arrays; g_h0: device array for dL/dh0 (padded
 * layout), or NULL.  Synchronises. */
extern "C" int cal_sdt_batch_loss_grad(void* handle, const double* target, double* loss_out, double* grad_out,
                                       double* g_h0)
{
    Batch* bt = (Batch*)handle;
    /* the tape layout is computed on the device for the whole rollout and
     * for segments of at most 32 steps (one warp each in k_tape_offsets:
     * rollouts of up to 1024 steps); longer segments are laid out here */
    if (bt->steps > 0) {
        const int rc = sdtb::loss_grad_device(*bt, target, loss_out, grad_out, g_h0);
        if (rc != sdtb::SEGMENTS_ON_HOST)
            return rc;
    }
    const size_t nb = (size_t)bt->N * sizeof(double);
    const int tc = sdtb::tile_cells(*bt);
    cudaStream_t st = bt->st;
    sdtb::forward(*bt, bt->steps, true);
    bt->h_counts.resize(bt->steps + 1);
    cudaMemcpyAsync(bt->h_counts.data(), bt->counts, sizeof(int) * (bt->steps + 1), cudaMemcpyDeviceToHost, st);
    cudaMemsetAsync(bt->loss, 0, bt->B * sizeof(double), st);
    cudaMemsetAsync(bt->grad, 0, 2 * bt->B * sizeof(double), st);
    sdtb::k_loss<<<sdtb::dense_grid(bt->N), sdtb::T, sizeof(long long) * (bt->B + 1), st>>>(
        bt->d_inst, bt->d_offs, bt->B, bt->N, bt->hbuf[bt->steps & 1], target, bt->lam, bt->lamz, bt->loss);
    if (cudaStreamSynchronize(st) != cudaSuccess)
        return (int)cudaGetLastError();
    /* the tape holds one segment: its layout follows the work-list sizes */
    std::vector<size_t> tape_off(bt->steps + 1, 0);
    size_t need = 0;
    for (int s = 0; s < bt->nseg; s++) {
        const int t0 = s * bt->K, t1 = std::min(t0 + bt->K, bt->steps);
        size_t acc = 0;
        for (int t = t0; t < t1; t++) {
            tape_off[t] = acc;
            acc += (size_t)bt->h_counts[t] * tc;
        }
        need = std::max(need, acc);
    }
    bt->last_need = (long long)need;
    if (need > bt->tape_cap && !sdtb::grow_tape(*bt, need)) {
        fprintf(stderr, "opencal-gb300: cal_sdt_batch_loss_grad: out of device memory for the tape\n");
        return (int)cudaErrorMemoryAllocation;
    }
    for (int s = bt->nseg - 1; s >= 0; s--) {
        const int t0 = s * bt->K, t1 = std::min(t0 + bt->K, bt->steps);
        if (t1 <= t0)
            continue;
        cudaMemcpyAsync(bt->hbuf[0], bt->ckpt + (size_t)s * bt->N, nb, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(bt->hbuf[1], bt->ckpt + (size_t)s * bt->N, nb, cudaMemcpyDeviceToDevice, st);
        for (int t = t0; t < t1; t++)
            SDTB_DISPATCH(*bt, sdtb::launch_step, *bt, t, bt->hbuf[(t - t0) & 1], bt->hbuf[(t - t0 + 1) & 1], false,
                          true, nullptr, nullptr, tape_off[t]);
        double* X = bt->hbuf[(t1 - t0) & 1]; /* h_{t1} everywhere */
        for (int t = t1 - 1; t >= t0; t--) {
            SDTB_DISPATCH(*bt, sdtb::launch_restore, *bt, t, bt->tape + tape_off[t], X);
            SDTB_DISPATCH(*bt, sdtb::launch_adjoint, *bt, t, X, nullptr, tape_off[t]);
        }
    }
    if (g_h0)
        sdtb::k_final_grad<<<sdtb::dense_grid(bt->N), sdtb::T, 0, st>>>(bt->h0, bt->lam, bt->lamz, g_h0, bt->N);
    std::vector<double> tmp(2 * bt->B);
    cudaMemcpyAsync(tmp.data(), bt->grad, 2 * bt->B * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (loss_out)
        cudaMemcpyAsync(loss_out, bt->loss, bt->B * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    if (grad_out)
        for (int b = 0; b < bt->B; b++) {
            grad_out[2 * b] = tmp[b];
            grad_out[2 * b + 1] = tmp[bt->B + b];
        }
    return (int)cudaGetLastError();
}

/* Pick the fastest tile shape for this ensemble: a forward of `probe_steps`
 * steps per candidate (0: 32x16, 1: 64x16, 2: 64x32), timed with CUDA
 * events after one untimed probe.  Writes the milliseconds to ms[0..2]
 * (ms[3..4] = 0) and returns the chosen shape, or -1 on a CUDA error.  The
 * smaller shapes 3 (16x8) and 4 (32x8) are not candidates: on the 256
 * instance calibration ensemble 16x8 wins a 100-step forward probe (9.5
 * against 10.4 ms) but loses the forward + adjoint iteration (1.084 against
 * 0.963 s); cal_sdt_batch_set_shape selects them. */
extern "C" int cal_sdt_batch_autotune(void* handle, int probe_steps, float* ms)
{
    Batch* bt = (Batch*)handle;
    if (probe_steps > bt->steps)
        probe_steps = bt->steps;
    int best = bt->shape;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int s = 0; s < sdtb::NSHAPES; s++)
        if (ms)
            ms[s] = 0.f;
    for (int s = 0; s < 3; s++) {
        bt->shape = s;
        if (!sdtb::tiles_for(*bt)) {
            best = -1;
            break;
        }
        sdtb::forward(*bt, probe_steps, false);
        cudaEventRecord(e0, bt->st);
        sdtb::forward(*bt, probe_steps, false);
        cudaEventRecord(e1, bt->st);
        cudaEventSynchronize(e1);
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (ms)
            ms[s] = t;
        if (t < best_ms) {
            best_ms = t;
            best = s;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best < 0)
        return -1;
    bt->shape = best;
    if (!sdtb::tiles_for(*bt))
        return -1;
    return cudaGetLastError() == cudaSuccess ? best : -1;
}

/* set the tile shape (0: 32x16, 1: 64x16, 2: 64x32, 3: 16x8, 4: 32x8); 0 on
 * success */
extern "C" int cal_sdt_batch_set_shape(void* handle, int shape)
{
    Batch* bt = (Batch*)handle;
    if (shape < 0 || shape >= sdtb::NSHAPES)
        return 1;
    bt->shape = shape;
    return sdtb::tiles_for(*bt) ? 0 : 2;
}

/* 1 (default): cal_sdt_batch_loss_grad runs as one launch of a recorded
 * graph; 0: launch by launch */
extern "C" int cal_sdt_batch_set_graph(void* handle, int on)
{
    Batch* bt = (Batch*)handle;
    bt->use_graph = on != 0;
    return 0;
}

/* What the adjoint's tape holds: -1 (default) the whole rollout while it
 * fits in half of the free device memory, else sqrt(T) segments recomputed
 * from checkpoints; 0 always segments; 1 always the whole rollout.  1 on a
 * bad mode. */
extern "C" int cal_sdt_batch_set_tape(void* handle, int mode)
{
    Batch* bt = (Batch*)handle;
    if (mode < -1 || mode > 1)
        return 1;
    bt->tape_mode = mode;
    bt->run_full = mode != 0;
    return 0;
}

/* info[0] = 1 when the last evaluation taped the whole rollout (0:
 * segments), info[1] = the tape's capacity in bytes, info[2] = the bytes of
 * tape the last evaluation needed */
extern "C" int cal_sdt_batch_tape_info(void* handle, long long* info)
{
    Batch* bt = (Batch*)handle;
    info[0] = bt->run_full ? 1 : 0;
    info[1] = (long long)(bt->tape_cap * (sizeof(double) + 1));
    info[2] = bt->last_need * (long long)(sizeof(double) + 1);
    return 0;
}

/* graph launches made by cal_sdt_batch_loss_grad so far and the nodes of
 * the recorded evaluation (kernels and copies) */
extern "C" int cal_sdt_batch_graph_stats(void* handle, long long* launches, long long* nodes)
{
    Batch* bt = (Batch*)handle;
    if (launches)
        *launches = bt->graph_launches;
    if (nodes)
        *nodes = bt->graph_nodes;
    return 0;
}
