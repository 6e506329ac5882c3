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

} // namespace life

static int g_life_block = 8; /* generations per launch */

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

/* Runs Life for `steps` generations; state in/out as 0/1 bytes.
 * mode 0: the reference program (device process, byte or int substate);
 * mode 1: fused launches of one generation each (byte substate);
 * mode 2: fused launches of `block` generations each (temporal blocking).
 * *ms = device time of the generation loop. */
extern "C" int cal_life2d_run(int rows, int cols, int toroidal, int as_int, int steps, const unsigned char* s0,
                              unsigned char* s_out, int mode, int block, int graph, double* ms)
{
    calClearError();
    if (mode != 0 && as_int)
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
        for (long long c = 0; c < n; c++)
            lifeQi->current[c] = lifeQi->next[c] = s0[c];
    } else {
        lifeQb = calAddSubstate2Db(ca);
        if (mode == 0)
            calAddElementaryProcess2D(ca, lifeTransitionFunctionB);
        else if (mode == 1)
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
    cudaEventRecord(e0, s);
    if (mode == 2) {
        g_life_block = block > 0 ? block : 8;
        life_fused_generations(ca, steps);
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
    calRunFinalize2D(run);
    calFinalize2D(ca);
    lifeQb = nullptr;
    lifeQi = nullptr;
    return err;
}
