/*
 * life.cu -- Conway's Game of Life (B3/S23), Moore neighbourhood, on
 * opencal-gb300.  Rule: OpenCAL/examples/cal_life-glut/source/life.c:16-27.
 *
 * 1. The reference program: one device elementary process on a byte or an
 *    int substate, registered with calAddElementaryProcess2D.
 * 2. The fused step for byte substates: a block loads its tile plus a ring of
 *    K cells into shared memory once, advances K generations there
 *    (temporal blocking: the valid region shrinks by one cell per
 *    generation) and writes the tile to the other layer, which every launch
 *    overwrites completely, so the host exchanges the layers after each
 *    launch.  1 B read + 1 B write per cell per K generations.  Outside a
 *    flat grid cells are absent: they read as 0 and are never born.
 */
#include <stdint.h>
#include <string.h>

#include "opencal/cal2D.h"
#include "opencal/cal2DRun.h"

/* ======================= 1. the reference program ======================= */

__managed__ struct CALSubstate2Db* lifeQb;
__managed__ struct CALSubstate2Di* lifeQi;

CAL_ELEMENTARY_PROCESS_2D(lifeTransitionFunctionB)(struct CALModel2D* ca, int i, int j)
{
    int sum = 0, n;
    for (n = 1; n < ca->sizeof_X; n++)
        sum += calGetX2Db(ca, lifeQb, i, j, n);
    if ((sum == 3) || (sum == 2 && calGet2Db(ca, lifeQb, i, j) == 1))
        calSet2Db(ca, lifeQb, i, j, 1);
    else
        calSet2Db(ca, lifeQb, i, j, 0);
}

CAL_ELEMENTARY_PROCESS_2D(lifeTransitionFunctionI)(struct CALModel2D* ca, int i, int j)
{
    int sum = 0, n;
    for (n = 1; n < ca->sizeof_X; n++)
        sum += calGetX2Di(ca, lifeQi, i, j, n);
    if ((sum == 3) || (sum == 2 && calGet2Di(ca, lifeQi, i, j) == 1))
        calSet2Di(ca, lifeQi, i, j, 1);
    else
        calSet2Di(ca, lifeQi, i, j, 0);
}

/* ======================= 2. the fused, temporally blocked step ========== */

namespace life {

constexpr int TW = 64, TH = 32, THREADS = 256;

template <int K>
__global__ void __launch_bounds__(THREADS) fused_steps(const signed char* __restrict__ cur,
                                                       signed char* __restrict__ nxt, int rows, int cols,
                                                       int toroidal)
{
    constexpr int W = TW + 2 * K, H = TH + 2 * K;
    __shared__ signed char buf[2][H][W + 4];
    const int i0 = blockIdx.y * TH - K, j0 = blockIdx.x * TW - K;
    for (int t = threadIdx.x; t < H * W; t += THREADS) {
        const int a = t / W, b = t - a * W;
        int gi = i0 + a, gj = j0 + b;
        signed char v = 0;
        if (toroidal) {
            gi = ((gi % rows) + rows) % rows;
            gj = ((gj % cols) + cols) % cols;
            v = cur[(long long)gi * cols + gj];
        } else if ((unsigned)gi < (unsigned)rows && (unsigned)gj < (unsigned)cols) {
            v = cur[(long long)gi * cols + gj];
        }
        buf[0][a][b] = v;
    }
    __syncthreads();
#pragma unroll 1
    for (int g = 1; g <= K; g++) {
        const int src = (g - 1) & 1, dst = g & 1;
        /* generation g is valid on the region shrunk by g cells */
        const int lo = g, hw = W - 2 * g, hh = H - 2 * g;
        for (int t = threadIdx.x; t < hw * hh; t += THREADS) {
            const int a = lo + t / hw, b = lo + t % hw;
            const int s = buf[src][a - 1][b - 1] + buf[src][a - 1][b] + buf[src][a - 1][b + 1] + buf[src][a][b - 1] +
                          buf[src][a][b + 1] + buf[src][a + 1][b - 1] + buf[src][a + 1][b] + buf[src][a + 1][b + 1];
            signed char v = (s == 3 || (s == 2 && buf[src][a][b] == 1)) ? 1 : 0;
            if (!toroidal) {
                const int gi = i0 + a, gj = j0 + b;
                if ((unsigned)gi >= (unsigned)rows || (unsigned)gj >= (unsigned)cols)
                    v = 0; /* not a cell */
            }
            buf[dst][a][b] = v;
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < TH * TW; t += THREADS) {
        const int a = t / TW, b = t - a * TW;
        const int gi = i0 + K + a, gj = j0 + K + b;
        if (gi < rows && gj < cols)
            nxt[(long long)gi * cols + gj] = buf[K & 1][K + a][K + b];
    }
}

template <int K>
static void launch(const signed char* cur, signed char* nxt, int rows, int cols, int toroidal, cudaStream_t s)
{
    dim3 grid((cols + TW - 1) / TW, (rows + TH - 1) / TH);
    fused_steps<K><<<grid, THREADS, 0, s>>>(cur, nxt, rows, cols, toroidal);
}

/* ---- bit-sliced form: 32 cells per 32-bit word -------------------------
 * A tile of BTH rows x BTWW words (32 cells each) plus a ring of K rows and
 * one word on each side is loaded into shared memory as bits, bit b of a
 * word = the cell (column of the word's first cell) + b.  When the width is
 * a multiple of 32 a thread reads a word's 32 cells with two 16-byte loads
 * and packs them by multiplication (pack4); other widths read cell by cell.
 * Each generation, a thread takes a word and its eight neighbour bit-planes
 * (the rows above and below, each shifted one cell left and right with the
 * bit carried over from the adjacent word) and adds them with a carry-save
 * adder tree; with s0, s1, s2 the count's 1s, 2s and 4s bits, a cell lives
 * next generation when the count is 3, or 2 and it is alive:
 * s1 & ~s2 & (s0 | alive) (a count of 8 has s1 = 0).  The valid region
 * shrinks by one cell per generation; one halo word on each side covers
 * K <= 32.  Cells outside a flat grid are masked to 0 every generation.
 * The rule is the byte rule only for states 0 and 1 (the sum counts byte
 * values), which is what Life's generations produce; a byte outside {0, 1}
 * in the input sets *bad and the caller reports an error. */
constexpr int BTH = 32, BTWW = 4, BTHREADS = 256;

static __device__ __forceinline__ void add3(uint32_t a, uint32_t b, uint32_t c, uint32_t& s, uint32_t& k)
{
    const uint32_t t = a ^ b;
    s = t ^ c;
    k = (a & b) | (c & t);
}

/* four 0/1 bytes (byte k = cell k) -> four bits (bit k = cell k): the
 * product's partial terms b_k * 2^(8k + 3 + 7m) land on distinct bits, and
 * bits 24..27 receive exactly b_0..b_3 (m = 3 - k), so no carry reaches them */
static __device__ __forceinline__ uint32_t pack4(uint32_t x)
{
    return (x * 0x01020408u) >> 24;
}

/* four bits -> four 0/1 bytes: bit k lands at k + 7m (m = 0..3, all sixteen
 * positions distinct), and the mask keeps m = k, i.e. bit 8k */
static __device__ __forceinline__ uint32_t unpack4(uint32_t n)
{
    return (n * 0x00204081u) & 0x01010101u;
}

template <int K>
__global__ void __launch_bounds__(BTHREADS) bits_steps(const signed char* __restrict__ cur,
                                                       signed char* __restrict__ nxt, int rows, int cols,
                                                       int toroidal, int* bad)
{
    static_assert(K >= 1 && K <= 32, "one halo word covers at most 32 generations");
    constexpr int H = BTH + 2 * K, WW = BTWW + 2;
    __shared__ uint32_t buf[2][H][WW];
    __shared__ uint32_t inmask[H][WW];
    const int i0 = blockIdx.y * BTH - K;
    const int w0 = blockIdx.x * BTWW - 1; /* global word column of tile word 0 */
    const bool vec = (cols & 31) == 0;   /* rows hold whole, 32-byte aligned words */
    const int cw = cols >> 5;
    for (int t = threadIdx.x; t < H * WW; t += BTHREADS) {
        const int a = t / WW, w = t - a * WW;
        int gi = i0 + a;
        const int gw = w0 + w;
        uint32_t word = 0, m = 0;
        if (toroidal)
            gi = ((gi % rows) + rows) % rows;
        if (vec) {
            int wc = gw;
            bool in = true;
            if (toroidal)
                wc = ((gw % cw) + cw) % cw;
            else
                in = gi >= 0 && gi < rows && gw >= 0 && gw < cw;
            if (in) {
                const uint4* p = reinterpret_cast<const uint4*>(cur + (size_t)gi * cols + (size_t)wc * 32);
                const uint4 q0 = __ldg(p), q1 = __ldg(p + 1);
                const uint32_t x[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
                uint32_t any = 0;
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    word |= pack4(x[q]) << (4 * q);
                    any |= x[q];
                }
                if (any & 0xFEFEFEFEu)
                    atomicExch(bad, 1);
                m = 0xffffffffu;
            }
        } else {
            const bool row_in = toroidal || (gi >= 0 && gi < rows);
            for (int b = 0; b < 32; b++) {
                int gj = gw * 32 + b;
                if (toroidal)
                    gj = ((gj % cols) + cols) % cols;
                else if (!row_in || gj < 0 || gj >= cols)
                    continue;
                const signed char v = cur[(size_t)gi * cols + gj];
                if (v != 0 && v != 1)
                    atomicExch(bad, 1);
                word |= (uint32_t)(v != 0) << b;
                m |= 1u << b;
            }
        }
        buf[0][a][w] = word;
        inmask[a][w] = m;
    }
    __syncthreads();
#pragma unroll 1
    for (int g = 1; g <= K; g++) {
        const int src = (g - 1) & 1, dst = g & 1;
        const int nrows = H - 2 * g; /* rows g .. H-1-g are valid after generation g */
        for (int t = threadIdx.x; t < nrows * WW; t += BTHREADS) {
            const int a = g + t / WW, w = t - (t / WW) * WW;
            uint32_t x[8];
            uint32_t mid = 0;
#pragma unroll
            for (int r = 0; r < 3; r++) {
                const uint32_t* row = buf[src][a - 1 + r];
                const uint32_t c = row[w];
                const uint32_t l = w > 0 ? row[w - 1] : 0u, rt = w < WW - 1 ? row[w + 1] : 0u;
                const uint32_t cl = (c << 1) | (l >> 31); /* the cell to the left */
                const uint32_t cr = (c >> 1) | (rt << 31); /* the cell to the right */
                if (r == 1) {
                    mid = c;
                    x[3] = cl;
                    x[4] = cr;
                } else {
                    x[r == 0 ? 0 : 5] = cl;
                    x[r == 0 ? 1 : 6] = c;
                    x[r == 0 ? 2 : 7] = cr;
                }
            }
            uint32_t sa, ka, sb, kb, s0, kd, ts, tk;
            add3(x[0], x[1], x[2], sa, ka);
            add3(x[3], x[4], x[5], sb, kb);
            const uint32_t sc = x[6] ^ x[7], kc = x[6] & x[7];
            add3(sa, sb, sc, s0, kd);             /* ones */
            add3(ka, kb, kc, ts, tk);             /* three of the four twos */
            const uint32_t s1 = ts ^ kd;          /* twos */
            const uint32_t s2 = tk ^ (ts & kd);   /* fours (eights dropped: a count of 8 has s1 = 0) */
            uint32_t next = s1 & ~s2 & (s0 | mid);
            if (!toroidal)
                next &= inmask[a][w];
            buf[dst][a][w] = next;
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < BTH * BTWW; t += BTHREADS) {
        const int a = K + t / BTWW, w = 1 + t % BTWW;
        const int gi = i0 + a, gw = w0 + w;
        const uint32_t word = buf[K & 1][a][w];
        if (gi >= rows)
            continue;
        if (vec) {
            if (gw >= cw)
                continue;
            uint32_t x[8];
#pragma unroll
            for (int q = 0; q < 8; q++)
                x[q] = unpack4((word >> (4 * q)) & 15u);
            uint4* p = reinterpret_cast<uint4*>(nxt + (size_t)gi * cols + (size_t)gw * 32);
            p[0] = make_uint4(x[0], x[1], x[2], x[3]);
            p[1] = make_uint4(x[4], x[5], x[6], x[7]);
        } else {
            for (int b = 0; b < 32; b++) {
                const int gj = gw * 32 + b;
                if (gj < cols)
                    nxt[(size_t)gi * cols + gj] = (signed char)((word >> b) & 1u);
            }
        }
    }
}

template <int K>
static void launch_bits(const signed char* cur, signed char* nxt, int rows, int cols, int toroidal, int* bad,
                        cudaStream_t s)
{
    dim3 grid((cols + BTWW * 32 - 1) / (BTWW * 32), (rows + BTH - 1) / BTH);
    bits_steps<K><<<grid, BTHREADS, 0, s>>>(cur, nxt, rows, cols, toroidal, bad);
}

} // namespace life

static int g_life_block = 8; /* generations per launch */

/* advances `gens` generations of the byte substate with bit-sliced fused
 * launches of up to `block` (<= 32) generations each */
static void life_bits_generations(struct CALModel2D* ca, int gens, int block, int* bad)
{
    cudaStream_t s = (cudaStream_t)calGetStream2D(ca);
    const int tor = ca->T == CAL_SPACE_TOROIDAL;
    while (gens > 0) {
        const signed char* cur = (const signed char*)calGetDeviceBuffer2Db(ca, lifeQb, 0);
        signed char* nxt = (signed char*)calGetDeviceBuffer2Db(ca, lifeQb, 2);
        const int want = gens < block ? gens : block;
        int k;
        if (want >= 32) {
            life::launch_bits<32>(cur, nxt, ca->rows, ca->columns, tor, bad, s);
            k = 32;
        } else if (want >= 16) {
            life::launch_bits<16>(cur, nxt, ca->rows, ca->columns, tor, bad, s);
            k = 16;
        } else if (want >= 8) {
            life::launch_bits<8>(cur, nxt, ca->rows, ca->columns, tor, bad, s);
            k = 8;
        } else if (want >= 4) {
            life::launch_bits<4>(cur, nxt, ca->rows, ca->columns, tor, bad, s);
            k = 4;
        } else if (want >= 2) {
            life::launch_bits<2>(cur, nxt, ca->rows, ca->columns, tor, bad, s);
            k = 2;
        } else {
            life::launch_bits<1>(cur, nxt, ca->rows, ca->columns, tor, bad, s);
            k = 1;
        }
        calSwapSubstate2Db(ca, lifeQb);
        gens -= k;
    }
}

/* advances `gens` generations of the byte substate with fused launches */
static void life_fused_generations(struct CALModel2D* ca, int gens)
{
    cudaStream_t s = (cudaStream_t)calGetStream2D(ca);
    const int tor = ca->T == CAL_SPACE_TOROIDAL;
    while (gens > 0) {
        const signed char* cur = (const signed char*)calGetDeviceBuffer2Db(ca, lifeQb, 0);
        signed char* nxt = (signed char*)calGetDeviceBuffer2Db(ca, lifeQb, 2);
        int k = gens >= g_life_block ? g_life_block : gens;
        if (k >= 8) {
            life::launch<8>(cur, nxt, ca->rows, ca->columns, tor, s);
            k = 8;
        } else if (k >= 4) {
            life::launch<4>(cur, nxt, ca->rows, ca->columns, tor, s);
            k = 4;
        } else if (k >= 2) {
            life::launch<2>(cur, nxt, ca->rows, ca->columns, tor, s);
            k = 2;
        } else {
            life::launch<1>(cur, nxt, ca->rows, ca->columns, tor, s);
            k = 1;
        }
        calSwapSubstate2Db(ca, lifeQb);
        gens -= k;
    }
}

static void life_fused_transition(struct CALModel2D* ca)
{
    life_fused_generations(ca, 1);
}

/* Declarations for the reference program's process (mode 0), for runs
 * started afterwards: bit 0 declares it pure (calSetElementaryProcessPure2D:
 * tiles whose neighbourhood did not change are skipped), bit 1 declares
 * that it reads the state substate (calSetElementaryProcessReads2D: staged
 * by TMA tile by tile).  0 (default): the program as it stands. */
static int g_life_decl = 0;

extern "C" int cal_life2d_set_declarations(int flags)
{
    g_life_decl = flags & 3;
    return 0;
}

/* Runs Life for `steps` generations; state in/out as 0/1 bytes.
 * mode 0: the reference program (device process, byte or int substate);
 * mode 1: fused launches of one generation each (byte substate);
 * mode 2: fused launches of `block` generations each (temporal blocking);
 * mode 3: bit-sliced fused launches of up to `block` (<= 32) generations
 *         each (states must be 0 / 1: CAL_ERROR_INVALID_ARGUMENT otherwise).
 * *ms = device time of the generation loop. */
extern "C" int cal_life2d_run(int rows, int cols, int toroidal, int as_int, int steps, const unsigned char* s0,
                              unsigned char* s_out, int mode, int block, int graph, double* ms)
{
    calClearError();
    if (mode < 0 || mode > 3 || (mode != 0 && as_int))
        return CAL_ERROR_INVALID_ARGUMENT;
    struct CALModel2D* ca = calCADef2D(rows, cols, CAL_MOORE_NEIGHBORHOOD_2D,
                                       toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    if (!ca)
        return calGetLastError();
    struct CALRun2D* run = calRunDef2D(ca, 1, steps, CAL_UPDATE_IMPLICIT);
    const long long n = (long long)rows * cols;
    if (as_int) {
        lifeQi = calAddSubstate2Di(ca);
        calAddElementaryProcess2D(ca, lifeTransitionFunctionI);
        if (g_life_decl & 1)
            calSetElementaryProcessPure2D(ca, lifeTransitionFunctionI, CAL_TRUE);
        if (g_life_decl & 2) {
            const void* reads[1] = {lifeQi};
            calSetElementaryProcessReads2D(ca, lifeTransitionFunctionI, reads, 1);
        }
        for (long long c = 0; c < n; c++)
            lifeQi->current[c] = lifeQi->next[c] = s0[c];
    } else {
        lifeQb = calAddSubstate2Db(ca);
        if (mode == 0) {
            calAddElementaryProcess2D(ca, lifeTransitionFunctionB);
            if (g_life_decl & 1)
                calSetElementaryProcessPure2D(ca, lifeTransitionFunctionB, CAL_TRUE);
            if (g_life_decl & 2) {
                const void* reads[1] = {lifeQb};
                calSetElementaryProcessReads2D(ca, lifeTransitionFunctionB, reads, 1);
            }
        }
        if (mode == 1)
            calRunAddGlobalTransitionFunc2D(run, life_fused_transition);
        for (long long c = 0; c < n; c++)
            lifeQb->current[c] = lifeQb->next[c] = (CALbyte)s0[c];
    }
    calMarkHostDirty2D(ca);
    calRunSetGraph2D(run, graph ? CAL_TRUE : CAL_FALSE);
    if (calGetLastError() != CAL_SUCCESS) {
        int e = calGetLastError();
        calRunFinalize2D(run);
        calFinalize2D(ca);
        return e;
    }
    cudaStream_t s = (cudaStream_t)calGetStream2D(ca);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    calRunInitSimulation2D(run);
    /* make sure uploads are done before timing */
    if (!as_int)
        calGetDeviceBuffer2Db(ca, lifeQb, 0);
    int* d_bad = nullptr;
    if (mode == 3 && (cudaMalloc(&d_bad, sizeof(int)) != cudaSuccess || cudaMemset(d_bad, 0, sizeof(int)) != cudaSuccess)) {
        calRunFinalize2D(run);
        calFinalize2D(ca);
        return CAL_ERROR_OUT_OF_MEMORY;
    }
    cudaEventRecord(e0, s);
    if (mode == 2) {
        g_life_block = block > 0 ? block : 8;
        life_fused_generations(ca, steps);
    } else if (mode == 3) {
        life_bits_generations(ca, steps, block > 0 && block <= 32 ? block : 32, d_bad);
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
    for (long long c = 0; c < n; c++)
        s_out[c] = as_int ? (unsigned char)lifeQi->current[c] : (unsigned char)lifeQb->current[c];
    int err = calGetLastError();
    if (d_bad) {
        int bad = 0;
        cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost);
        cudaFree(d_bad);
        if (bad && err == CAL_SUCCESS)
            err = CAL_ERROR_INVALID_ARGUMENT; /* a state other than 0 / 1 */
    }
    calRunFinalize2D(run);
    calFinalize2D(ca);
    lifeQb = nullptr;
    lifeQi = nullptr;
    return err;
}
