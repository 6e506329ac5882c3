/*
 * sciara_batch.cu -- SCIARA-fv2 scenarios (one grid or many, each with its
 * own morphology, vents and emission rates) advanced by a split step:
 *
 *   K0 (vents): updateVentsEmission (OpenCAL-OMP/examples/calomp_sciara-fv2/
 *      source/Sciara.cpp:3-16): thickness += rate / Pac * Pclock at each
 *      emitting vent (the last vent listed for a cell wins, as the EP's
 *      get-current-then-set does), temperature = PTvent; a vent cell that
 *      had no lava joins the lava list.
 *   K1 (flows): empiricalFlows + outflowsMin (Sciara.cpp:18-105) for every
 *      cell of the lava list (Slt > 0), one thread each, spread over the
 *      whole GPU -- the power laws, the shear test and the minimisation
 *      are the step's FP64 work.  The eight outflows of list entry k, and
 *      each outflow times the cell's temperature (the product width_update
 *      forms at the receiver, same operands), go to compact slot k; a
 *      per-cell (epoch, slot) map makes them addressable by cell.  A
 *      receiver without lava joins the receiver list once (epoch stamp).
 *   K2 (update): width_update, updateTemperature and the steering's border
 *      reset (Sciara.cpp:106-169, 185-193) at every lava cell and every
 *      receiver, one thread each over the whole GPU, in place: a cell reads
 *      only its own state and the compact outflows; it joins the next lava
 *      list if it still holds lava.  Any other cell has no lava and no
 *      inflow, so it is unchanged (border cells hold 0 from the start).
 *   For the adjoint, K1 also flags the 32 x 16 tiles of the lava cells and
 *   receivers, and a tape kernel between K1 and K2 copies those tiles'
 *   state before the update.
 *
 * Arithmetic is the reference's, operation by operation (--fmad=false),
 * except the transcendental forms of sciara_math.cuh (exp10, the shear test
 * without atan / cos, T^3 and cbrt), shared with the device-process program
 * (sciara.cu), which this step reproduces bit for bit.  All scenarios share
 * the physical parameters and the emission schedule's length, so they run
 * the same number of steps (the reference stops when the elapsed time
 * reaches the emission's end).
 *
 * Layout: scenarios packed back to back (offsets padded to 32 cells); per
 * cell Sz, Slt, St, Msl (FP64), Mb (byte), the (epoch, slot) map (8 B), the
 * receiver stamp (4 B) and a copy of the initial Sz, Slt, St (every run
 * starts from it): 69 B per cell; per list slot (capacity chosen at
 * creation) two lava-list entries, a receiver entry and the outflows
 * (140 B).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "exact_div.cuh"
#include "sciara_math.cuh"

namespace sci2 {

constexpr int T = 256;
constexpr int K1T = 64;
constexpr int TW = 32, TH = 16; /* K2 tile; 2 cells per thread */
constexpr int K2_BLOCKS = 152 * 4;
constexpr int MAX_INST = 1024;

struct Phys {
    double Pclock, Pc, Pac, PTsol, PTvent, a, b, c, d, Pcool, Prho, Pepsilon, Psigma, Pcv, rad2;
    double rrad2, w2; /* RN(1 / rad2), Pc * Pc */
    int rad2_recip;   /* x / rad2 by cal_div_recip (its precondition holds) */
};

struct Inst {
    int rows, cols;
    long long off;
    int tiles_x, tiles_y, tile0, pad;
};

/* counts[]: [0] lava list length, [5] K2 ticket, [6] epoch, [7] tiles
 * flagged in this step, [8] lava- or receiver-list overflow flag, [9] tape
 * slots used so far (counted on past the capacity), [10] tape overflow
 * flag, [11] receiver list length, [12] tiles flagged in the previous step,
 * [13] lava cells after the last update */
struct Dev {
    const Inst* inst;
    const long long* offs;
    int B;
    double* Sz;
    double* Slt;
    double* St;
    double* Msl;
    const unsigned char* Mb;
    double* fc;   /* 16 doubles per list slot: f[8], f * St[8] */
    int2* map;    /* per cell: (epoch, slot) */
    int* recv;    /* per cell: epoch in which it was listed as a receiver */
    int* rlist;   /* cells without lava that receive a flow this step */
    int* list;    /* lava cells, tile by tile, row-major within a tile */
    unsigned* mask; /* per tile 16 words: bit j of word r = cell (r, j) holds lava after K2 */
    int* counts;
    int* tflag;
    int* tlist;
    long long ncells;
    int capacity;
    int nvents;
    const int* vent_cell;  /* packed cell index of each vent */
    const int* vent_first; /* B + 1: vents of instance b are [vent_first[b], vent_first[b + 1]) */
    /* vent cells: the vents of one scenario at one cell form a group, led
     * by its first vent; per group and phase the vent whose emission takes
     * effect (the last with a positive one, -1: none) and its thickness */
    int ngroups;
    const int* g_cell;    /* packed cell */
    const int* g_member;  /* g_mfirst[g]..g_mfirst[g+1]: the group's vents, leader first */
    const int* g_mfirst;
    const int* g_eff;     /* ngroups x nphases */
    const double* g_emit; /* ngroups x nphases */
    int nphases;
    unsigned emission_time;
    Phys ph;
};

static __device__ __forceinline__ int locate(const long long* s_offs, int B, long long c)
{
    int lo = 0, hi = B - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_offs[mid] <= c)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

/* Moore neighbour k = 0..8 (OpenCAL order: centre, N, W, E, S, NW, SW, SE, NE) */
__device__ __constant__ int kMi[9] = {0, -1, 0, 0, 1, -1, 1, 1, -1};
__device__ __constant__ int kMj[9] = {0, 0, -1, 1, 0, -1, -1, 1, 1};

static __device__ __forceinline__ bool nbr(const Inst& I, int i, int j, int k, long long* c)
{
    const int a = i + kMi[k], b = j + kMj[k];
    if ((unsigned)a >= (unsigned)I.rows || (unsigned)b >= (unsigned)I.cols)
        return false; /* flat boundary */
    *c = I.off + (long long)a * I.cols + b;
    return true;
}

static __device__ __forceinline__ void append(int* list, int* count, int capacity, int* overflow, int value)
{
    const int pos = atomicAdd(count, 1);
    if (pos < capacity)
        list[pos] = value;
    else
        atomicExch(overflow, 1);
}

static __device__ __forceinline__ void flag_tile(const Dev& d, int t, int epoch)
{
    if (d.tflag[t] != epoch && atomicExch(d.tflag + t, epoch) != epoch)
        d.tlist[atomicAdd(d.counts + 7, 1)] = t;
}

/* K0: the lava list of this step, and the vent emission.
 * The list is collected from the lava masks K2 left in the tiles flagged by
 * the previous step (every cell that can hold lava after an update lies in
 * one), tile by tile and row-major within a tile, so that neighbouring list
 * entries are neighbouring cells; the masks are cleared on the way.  Half a
 * warp reads a tile's 16 mask words and reserves the tile's run of list
 * slots with one atomic.  (The first step uses the list the priming kernel
 * built.)  Block 0 also emits at the vents, one thread per scenario; a
 * vent cell that had no lava is appended.  With a vent tape (one record of
 * 3 doubles per vent and step) the first vent of each cell records the
 * cell's thickness and temperature before the emission and which vent's
 * emission took effect. */
__global__ void __launch_bounds__(T) k_collect(const __grid_constant__ Dev d, unsigned phase, double* vtape,
                                               int rebuild)
{
    if (blockIdx.x == 0) {
        if (threadIdx.x == 0)
            d.counts[13] = 0;
        for (int g = threadIdx.x; g < d.ngroups; g += blockDim.x) {
            const int c = d.g_cell[g];
            const int m0 = d.g_mfirst[g], m1 = d.g_mfirst[g + 1];
            const int eff = phase < (unsigned)d.nphases ? d.g_eff[(size_t)g * d.nphases + phase] : -1;
            /* the process reads the current thickness: the cell's vents add
             * to the value before this step's emission, the last positive
             * one wins */
            const double orig = d.Slt[c];
            if (vtape) {
                const int lead = d.g_member[m0];
                vtape[3 * lead] = orig;
                vtape[3 * lead + 1] = d.St[c];
                vtape[3 * lead + 2] = (double)eff;
                for (int m = m0 + 1; m < m1; m++)
                    vtape[3 * d.g_member[m] + 2] = -2.0; /* handled with the cell's first vent */
            }
            if (eff >= 0) {
                d.Slt[c] = orig + d.g_emit[(size_t)g * d.nphases + phase];
                d.St[c] = d.ph.PTvent;
                if (!(orig > 0))
                    append(d.list, d.counts + 0, d.capacity, d.counts + 8, c);
            }
        }
    }
    if (!rebuild)
        return;
    const int ntiles = d.counts[12];
    const int lane = threadIdx.x & 31, half = lane >> 4, l = lane & 15;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int item0 = 2 * warp; item0 < ntiles; item0 += 2 * nwarps) {
        const int item = item0 + half;
        unsigned w = 0;
        int t = 0;
        if (item < ntiles) {
            t = d.tlist[item];
            w = d.mask[(size_t)t * 16 + l];
            if (w)
                d.mask[(size_t)t * 16 + l] = 0;
        }
        const int cnt = __popc(w);
        int inc = cnt; /* inclusive scan over the half warp */
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, inc, o, 16);
            if (l >= o)
                inc += v;
        }
        int base = 0;
        if (l == 15 && inc > 0)
            base = atomicAdd(d.counts + 0, inc);
        base = __shfl_sync(0xffffffffu, base, 15, 16);
        if (w) {
            int lo = 0, hi = d.B - 1; /* the tile's instance: largest b with tile0 <= t */
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (d.inst[mid].tile0 <= t)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const Inst I = d.inst[lo];
            const int lt = t - I.tile0;
            const int ty = lt / I.tiles_x, tx = lt - ty * I.tiles_x;
            const long long row = I.off + (long long)(ty * TH + l) * I.cols + tx * TW;
            int pos = base + inc - cnt;
            while (w) {
                const int bit = __ffs(w) - 1;
                w &= w - 1;
                if (pos < d.capacity)
                    d.list[pos] = (int)(row + bit);
                else
                    atomicExch(d.counts + 8, 1);
                pos++;
            }
        }
    }
}

/* outflowsMin (Sciara.cpp:23-90) at lava cell c, with what its adjoint needs */
struct Flow {
    double h[9], z[9], H[9], f[9];
    double avg, Pr, t;
    long long cn[9];
    unsigned inside, S, F; /* in-grid neighbours, final set, positive outflows */
    int nS;
};

/* The arithmetic of outflowsMin with every FP64 operation that can leave
 * the narrow FP64 pipe moved to the integer pipe, each with identical
 * results (exact_div.cuh): comparisons of non-negative values on the bit
 * patterns; z0 + h0 > z_k + h_k as the sign of their difference (for finite
 * values, a - b > 0 exactly when a > b); the average's division by the set
 * size (1..9) by integer long division; the diagonal altitude's division by
 * rad2 through its reciprocal with Markstein's correction. */
static __device__ __forceinline__ void compute_flows(const Dev& d, const Inst& I, long long c, int i, int j, Flow& F)
{
    double dz[9];
    bool in_set[9];
    const double t = d.St[c];
    F.t = t;
    F.Pr = sci_power_law(d.ph.a, d.ph.b, t);
    const double hc = sci_power_law(d.ph.c, d.ph.d, t);
    const double sz0 = d.Sz[c];
    const bool recip = d.ph.rad2_recip != 0;
    F.inside = 0;
#pragma unroll
    for (int q = 0; q < 9; q++) {
        const bool in = nbr(I, i, j, q, &F.cn[q]);
        F.inside |= (in ? 1u : 0u) << q;
        F.h[q] = in ? d.Slt[F.cn[q]] : 0.0;
        const double sz = in ? d.Sz[F.cn[q]] : 0.0;
        F.H[q] = F.f[q] = dz[q] = 0;
        if (q < 5)
            F.z[q] = sz;
        else
            F.z[q] = sz0 - (recip ? cal_div_recip(sz0 - sz, d.ph.rad2, d.ph.rrad2) : (sz0 - sz) / d.ph.rad2);
    }
    F.H[0] = F.z[0];
    in_set[0] = true;
    const double zh0 = F.z[0] + F.h[0];
#pragma unroll
    for (int q = 1; q < 9; q++) {
        const double Hq = F.z[q] + F.h[q];
        const double dq = zh0 - Hq;
        in_set[q] = cal_pos(dq);
        if (in_set[q]) {
            F.H[q] = Hq;
            dz[q] = dq;
        }
    }
    bool loop;
    double avg;
    int counter;
    do {
        loop = false;
        avg = F.h[0];
        counter = 0;
#pragma unroll
        for (int q = 0; q < 9; q++)
            if (in_set[q]) {
                avg += F.H[q];
                counter++;
            }
        if (counter != 0)
            avg = cal_div_small(avg, counter);
#pragma unroll
        for (int q = 0; q < 9; q++)
            if (in_set[q] && cal_le(avg, F.H[q])) {
                in_set[q] = false;
                loop = true;
            }
    } while (loop);
    /* the last average was formed over the set before the final (empty)
     * round of eliminations: that set is the final one */
    F.avg = avg;
    F.nS = counter;
    F.S = 0;
    F.F = 0;
#pragma unroll
    for (int q = 0; q < 9; q++)
        F.S |= (in_set[q] ? 1u : 0u) << q;
    const double h0 = F.h[0];
    const double h0sq = h0 * h0, rhs = hc * hc * d.ph.w2;
#pragma unroll
    for (int q = 1; q < 9; q++) {
        double fq = 0.0;
        /* sci_shear_exceeded(h0, hc, dz, w): h0 > 0 and h0^2 (w^2 + dz^2) > hc^2 w^2 */
        if (in_set[q] && cal_pos(h0) && cal_gt(h0sq * (d.ph.w2 + dz[q] * dz[q]), rhs))
            fq = F.Pr * (avg - F.H[q]);
        /* empiricalFlows stores only positive outflows; the rest stay 0 */
        if (!cal_pos(fq))
            fq = 0.0;
        F.f[q] = fq;
        if (cal_pos(fq))
            F.F |= 1u << q;
    }
}

/* K1: outflows of every lava cell into compact slots.  A receiver without
 * lava joins the receiver list once (epoch stamp), so that K2 visits
 * exactly the lava cells and the cells they flow into.  The tiles of the
 * lava cells and receivers are flagged: they hold every cell that can hold
 * lava after K2 (K0 of the next step collects the list from them) and every
 * cell the step changes besides the vents (the tape copies them). */
__global__ void __launch_bounds__(K1T) k_flows(const __grid_constant__ Dev d)
{
    __shared__ long long s_offs[MAX_INST + 1];
    for (int k = threadIdx.x; k <= d.B; k += blockDim.x)
        s_offs[k] = d.offs[k];
    __syncthreads();
    const int epoch = d.counts[6];
    const int n = min(d.counts[0], d.capacity);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int c = d.list[k];
        const Inst I = d.inst[locate(s_offs, d.B, c)];
        const long long lc = c - I.off;
        const int i = (int)(lc / I.cols), j = (int)(lc - (long long)i * I.cols);
        Flow F;
        compute_flows(d, I, c, i, j, F);
        double* slot = d.fc + (size_t)k * 16;
#pragma unroll
        for (int q = 1; q < 9; q++) {
            slot[q - 1] = F.f[q];
            slot[8 + q - 1] = F.f[q] * F.t;
            if ((F.F >> q) & (F.inside >> q) & 1u) {
                const int cn = (int)F.cn[q];
                if (!cal_pos(F.h[q]) && d.recv[cn] != epoch && atomicExch(d.recv + cn, epoch) != epoch) {
                    append(d.rlist, d.counts + 11, d.capacity, d.counts + 8, cn);
                    const long long rc = F.cn[q] - I.off;
                    const int ri = (int)(rc / I.cols), rj = (int)(rc - (long long)ri * I.cols);
                    flag_tile(d, I.tile0 + (ri / TH) * I.tiles_x + rj / TW, epoch);
                }
            }
        }
        d.map[c] = make_int2(epoch, k);
        flag_tile(d, I.tile0 + (i / TH) * I.tiles_x + j / TW, epoch);
    }
}

/* width_update and updateTemperature at one cell (Sciara.cpp:106-169):
 * the forward quantities, with the outflows found through the (epoch, slot)
 * map */
struct CellFwd {
    double h, t, sz, in_sum, out_sum, ht, residual, D, hn, tn, aus, st;
    bool flowcond, border, lava, solid;
};

static __device__ __forceinline__ void compute_cell(const Dev& d, const Inst& I, int i, int j, long long x, int epoch,
                                                    CellFwd& Cf)
{
    const int opp[8] = {3, 2, 1, 0, 6, 7, 4, 5};
    Cf.h = d.Slt[x];
    Cf.t = d.St[x];
    Cf.sz = d.Sz[x];
    const int2 me = d.map[x];
    const double* mine = me.x == epoch ? d.fc + (size_t)me.y * 16 : nullptr;
    double ht = 0, in_sum = 0, out_sum = 0;
#pragma unroll
    for (int n = 1; n < 9; n++) {
        long long cn;
        double in_flow = 0.0, in_ft = 0.0;
        if (nbr(I, i, j, n, &cn)) {
            const int2 m = d.map[cn];
            if (m.x == epoch) {
                const double* s = d.fc + (size_t)m.y * 16;
                in_flow = s[opp[n - 1]];
                in_ft = s[8 + opp[n - 1]];
            }
        }
        const double out_flow = mine ? mine[n - 1] : 0.0;
        ht += in_ft; /* inFlow * neigh_t, formed at the source with the same operands */
        in_sum += in_flow;
        out_sum += out_flow;
    }
    Cf.ht = ht;
    Cf.in_sum = in_sum;
    Cf.out_sum = out_sum;
    double h_next = Cf.h;
    double t_next = Cf.t;
    h_next += in_sum - out_sum;
    Cf.flowcond = in_sum > 0 || out_sum > 0;
    Cf.residual = 0.0;
    Cf.D = 1.0;
    if (Cf.flowcond) {
        Cf.residual = Cf.h - out_sum;
        Cf.D = Cf.residual + in_sum;
        t_next = (Cf.residual * Cf.t + ht) / Cf.D;
    }
    Cf.hn = h_next;
    Cf.tn = t_next;
    Cf.border = d.Mb[x] != 0;
    Cf.lava = h_next > 0 && !Cf.border;
    Cf.solid = false;
    Cf.aus = 1.0;
    Cf.st = t_next;
    if (Cf.lava) {
        const double nT = t_next;
        Cf.st = sci_cool(nT, h_next, d.ph.Pepsilon, d.ph.Psigma, d.ph.Pclock, d.ph.Pcool, d.ph.Prho, d.ph.Pcv,
                         d.ph.Pac, &Cf.aus);
        Cf.solid = Cf.st <= d.ph.PTsol;
    }
}

/* the step at one cell, in place (the border reset of the steering last) */
static __device__ __forceinline__ bool update_cell(const Dev& d, const Inst& I, int i, int j, int epoch)
{
    const long long x = I.off + (long long)i * I.cols + j;
    CellFwd Cf;
    compute_cell(d, I, i, j, x, epoch, Cf);
    double sh = Cf.hn, st = Cf.tn;
    if (Cf.lava) {
        st = Cf.st;
        if (Cf.solid) {
            d.Sz[x] = Cf.sz + sh;
            d.Msl[x] = d.Msl[x] + sh;
            sh = 0;
            st = d.ph.PTsol;
        }
    }
    if (Cf.border) {
        sh = 0;
        st = 0;
    }
    d.Slt[x] = sh;
    d.St[x] = st;
    return sh > 0;
}

/* undo tape of a run whose gradient is wanted: per flagged tile and step,
 * the tile's (Slt, St, Sz) before the update; per step and vent cell, its
 * thickness and temperature before the emission and the vent that emitted */
struct Tape {
    int* tile;        /* per slot: tile */
    double* state;    /* per slot: 3 x TW*TH */
    int* step_base;   /* per step: first slot */
    int* step_count;  /* per step: slots */
    double* vent;     /* per step and vent: orig Slt, orig St, emitting vent (-1: none, -2: not the cell's first) */
    long long cap;    /* slots */
};

/* With a tape: every cell of the flagged tiles, (Slt, St, Sz) before the
 * update, into the tape slot of the tile.  The flagged tiles hold every
 * cell K0 and K2 change in this step besides the vent cells, which the
 * vent tape records. */
__global__ void __launch_bounds__(T) k_tape(const __grid_constant__ Dev d, const __grid_constant__ Tape tp)
{
    const int ntiles = d.counts[7];
    const int base = d.counts[9];
    for (int item = blockIdx.x; item < ntiles; item += gridDim.x) {
        const int t = d.tlist[item];
        int lo = 0, hi = d.B - 1; /* the tile's instance: largest b with tile0 <= t */
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (d.inst[mid].tile0 <= t)
                lo = mid;
            else
                hi = mid - 1;
        }
        const Inst I = d.inst[lo];
        const int lt = t - I.tile0;
        const int ty = lt / I.tiles_x, tx = lt - ty * I.tiles_x;
        const long long slot = (long long)base + item;
        if (slot >= tp.cap) {
            if (threadIdx.x == 0)
                atomicExch(d.counts + 10, 1);
            continue;
        }
        if (threadIdx.x == 0)
            tp.tile[slot] = t;
        double* s = tp.state + (size_t)slot * 3 * TW * TH;
        for (int q = threadIdx.x; q < TW * TH; q += T) {
            const int i = ty * TH + q / TW, j = tx * TW + q % TW;
            if (i < I.rows && j < I.cols) {
                const long long x = I.off + (long long)i * I.cols + j;
                s[q] = d.Slt[x];
                s[TW * TH + q] = d.St[x];
                s[2 * TW * TH + q] = d.Sz[x];
            }
        }
    }
}

/* K2: width_update, updateTemperature and the border reset at every lava
 * cell and every receiver (the only cells whose state can change: any
 * other cell has no lava and no inflow, so h + (0 - 0) = h and the
 * temperature stays; border cells hold 0 from the start); one thread per
 * cell over the whole GPU; a cell that still holds lava sets its bit in
 * its tile's mask.  The last block to finish advances the step's
 * counters. */
__global__ void __launch_bounds__(K1T) k_update(const __grid_constant__ Dev d, const __grid_constant__ Tape tp,
                                                int step)
{
    __shared__ long long s_offs[MAX_INST + 1];
    for (int k = threadIdx.x; k <= d.B; k += blockDim.x)
        s_offs[k] = d.offs[k];
    __syncthreads();
    const int epoch = d.counts[6];
    const int nl = min(d.counts[0], d.capacity);
    const int n = nl + min(d.counts[11], d.capacity);
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int k0 = blockIdx.x * blockDim.x; k0 < n; k0 += stride) {
        const int k = k0 + threadIdx.x;
        bool lava = false;
        if (k < n) {
            const int c = k < nl ? d.list[k] : d.rlist[k - nl];
            const Inst I = d.inst[locate(s_offs, d.B, c)];
            const long long lc = c - I.off;
            const int i = (int)(lc / I.cols), j = (int)(lc - (long long)i * I.cols);
            lava = update_cell(d, I, i, j, epoch);
            if (lava)
                atomicOr(d.mask + (size_t)(I.tile0 + (i / TH) * I.tiles_x + j / TW) * 16 + (i % TH), 1u << (j % TW));
        }
        const unsigned m = __ballot_sync(0xffffffffu, lava);
        if (m && lane == 0)
            atomicAdd(d.counts + 13, __popc(m));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(reinterpret_cast<unsigned*>(d.counts + 5), 1u) == gridDim.x - 1) {
            if (tp.state) {
                const int ntiles = d.counts[7], base = d.counts[9];
                tp.step_base[step] = base;
                tp.step_count[step] = ntiles;
                d.counts[9] = base + ntiles;
            }
            d.counts[0] = 0; /* K0 of the next step collects the list from the masks */
            d.counts[5] = 0;
            d.counts[6] = epoch + 1;
            d.counts[12] = d.counts[7];
            d.counts[7] = 0;
            d.counts[11] = 0;
        }
    }
}

/* ---- adjoint of the final-thickness misfit --------------------------------
 * L = sum over every scenario's cells of (Slt_T - target)^2; gradient with
 * respect to every vent's emission rate of every phase.  The forward's
 * discrete decisions are frozen: the minimisation's elimination sets and the
 * shear-resistance test, whether a cell has any flow, whether it holds lava,
 * whether it solidifies, the border mask.  Reverse mode, step by step from
 * the last: restore the step's taped tiles (the state after its emission),
 * recompute its outflows, then
 *   B2 (per cell of the step's tiles): mixing and cooling backward, in
 *      place on the cell's own adjoints; keeps, per cell, dL/dh' (A_h),
 *      dL/dt' / D (A_t) and t' for the outflow adjoints;
 *   B1 (per lava cell): the adjoint of each outflow gathered from the two
 *      cells it connects, then the minimisation backward, scattered (FP64
 *      atomics) to the thickness, altitude and temperature adjoints of the
 *      nine cells it read;
 *   B0 (per scenario): the emission backward -- dL/drate += dL/dSlt(vent) *
 *      Pclock / Pac for the vent whose emission took effect, the temperature
 *      adjoint of the vent cell reset (the emission overwrote it) -- and the
 *      vent cells restored to their state before the emission. */
struct Adj {
    double* lh;   /* dense: dL/dSlt */
    double* lt;   /* dense: dL/dSt */
    double* lz;   /* dense: dL/dSz */
    double* fcb;  /* per compact cell: recomputed outflows (16 doubles) */
    double* Ah;   /* per compact cell */
    double* At;
    double* tp;
    double* grad; /* nvents x nphases, internal vent order */
};

static __device__ __forceinline__ int tile_instance(const Dev& d, int t)
{
    int lo = 0, hi = d.B - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (d.inst[mid].tile0 <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(T) k_brestore(const __grid_constant__ Dev d, const __grid_constant__ Tape tp, int base,
                                                int count)
{
    for (int item = blockIdx.x; item < count; item += gridDim.x) {
        const long long slot = (long long)base + item;
        const int t = tp.tile[slot];
        const Inst I = d.inst[tile_instance(d, t)];
        const int lt = t - I.tile0;
        const int ty = lt / I.tiles_x, tx = lt - ty * I.tiles_x;
        const double* s = tp.state + (size_t)slot * 3 * TW * TH;
        for (int q = threadIdx.x; q < TW * TH; q += T) {
            const int i = ty * TH + q / TW, j = tx * TW + q % TW;
            if (i < I.rows && j < I.cols) {
                const long long x = I.off + (long long)i * I.cols + j;
                d.Slt[x] = s[q];
                d.St[x] = s[TW * TH + q];
                d.Sz[x] = s[2 * TW * TH + q];
            }
        }
    }
}

/* the step's outflows again, from the restored state, into compact cells */
__global__ void __launch_bounds__(T) k_bflows(const __grid_constant__ Dev db, const __grid_constant__ Tape tp,
                                              int base, int count, int epoch_b)
{
    for (int item = blockIdx.x; item < count; item += gridDim.x) {
        const int t = tp.tile[(long long)base + item];
        const Inst I = db.inst[tile_instance(db, t)];
        const int lt = t - I.tile0;
        const int ty = lt / I.tiles_x, tx = lt - ty * I.tiles_x;
        for (int q = threadIdx.x; q < TW * TH; q += T) {
            const int i = ty * TH + q / TW, j = tx * TW + q % TW;
            if (i >= I.rows || j >= I.cols)
                continue;
            const long long x = I.off + (long long)i * I.cols + j;
            const int idx = item * TW * TH + q;
            double* slot = db.fc + (size_t)idx * 16;
            db.map[x] = make_int2(epoch_b, idx);
            if (db.Slt[x] > 0) {
                Flow F;
                compute_flows(db, I, x, i, j, F);
#pragma unroll
                for (int k = 1; k < 9; k++) {
                    slot[k - 1] = F.f[k];
                    slot[8 + k - 1] = F.f[k] * F.t;
                }
            } else {
#pragma unroll
                for (int k = 0; k < 16; k++)
                    slot[k] = 0.0;
            }
        }
    }
}

__global__ void __launch_bounds__(T) k_bcells(const __grid_constant__ Dev db, const __grid_constant__ Tape tp,
                                              const __grid_constant__ Adj a, int base, int count, int epoch_b)
{
    for (int item = blockIdx.x; item < count; item += gridDim.x) {
        const int t = tp.tile[(long long)base + item];
        const Inst I = db.inst[tile_instance(db, t)];
        const int lt = t - I.tile0;
        const int ty = lt / I.tiles_x, tx = lt - ty * I.tiles_x;
        for (int q = threadIdx.x; q < TW * TH; q += T) {
            const int i = ty * TH + q / TW, j = tx * TW + q % TW;
            if (i >= I.rows || j >= I.cols)
                continue;
            const long long x = I.off + (long long)i * I.cols + j;
            const int idx = item * TW * TH + q;
            CellFwd Cf;
            compute_cell(db, I, i, j, x, epoch_b, Cf);
            const double lh = a.lh[x], lt_ = a.lt[x];
            double Lh = lh, Lt = lt_; /* adjoints of h', t' */
            if (Cf.border) {
                Lh = 0.0;
                Lt = 0.0;
            } else if (Cf.lava) {
                if (Cf.solid) {
                    Lh = a.lz[x]; /* Sz += h' */
                    Lt = 0.0;
                } else {
                    /* st = nT / aus^(1/3), aus = 1 + 3 K nT^3 / (C h') */
                    const double K = db.ph.Pepsilon * db.ph.Psigma * db.ph.Pclock * db.ph.Pcool;
                    const double Cc = db.ph.Prho * db.ph.Pcv * db.ph.Pac;
                    const double nT = Cf.tn, hn = Cf.hn;
                    const double dst_daus = -Cf.st / (3.0 * Cf.aus);
                    const double daus_dT = 9.0 * K * nT * nT / (Cc * hn);
                    const double daus_dh = -3.0 * K * nT * nT * nT / (Cc * hn * hn);
                    const double dst_dT = Cf.st / nT + dst_daus * daus_dT;
                    Lh = lh + lt_ * (dst_daus * daus_dh);
                    Lt = lt_ * dst_dT;
                }
            }
            double new_lh = Lh, new_lt = Lt, At = 0.0;
            if (Cf.flowcond) {
                new_lh = Lh + Lt * (Cf.t - Cf.tn) / Cf.D;
                new_lt = Lt * Cf.residual / Cf.D;
                At = Lt / Cf.D;
            }
            a.lh[x] = new_lh;
            a.lt[x] = new_lt;
            a.Ah[idx] = Lh;
            a.At[idx] = At;
            a.tp[idx] = Cf.tn;
        }
    }
}

__global__ void __launch_bounds__(T) k_bflowadj(const __grid_constant__ Dev db, const __grid_constant__ Tape tp,
                                                const __grid_constant__ Adj a, int base, int count, int epoch_b)
{
    for (int item = blockIdx.x; item < count; item += gridDim.x) {
        const int t = tp.tile[(long long)base + item];
        const Inst I = db.inst[tile_instance(db, t)];
        const int lt = t - I.tile0;
        const int ty = lt / I.tiles_x, tx = lt - ty * I.tiles_x;
        for (int q0 = threadIdx.x; q0 < TW * TH; q0 += T) {
            const int i = ty * TH + q0 / TW, j = tx * TW + q0 % TW;
            if (i >= I.rows || j >= I.cols)
                continue;
            const long long x = I.off + (long long)i * I.cols + j;
            if (!(db.Slt[x] > 0))
                continue;
            Flow F;
            compute_flows(db, I, x, i, j, F);
            if (!F.F)
                continue;
            const int idx = item * TW * TH + q0;
            const double Ahc = a.Ah[idx], Atc = a.At[idx], tpc = a.tp[idx];
            double lf[9];
            double lt_add = 0.0;
#pragma unroll
            for (int k = 0; k < 9; k++)
                lf[k] = 0.0;
#pragma unroll
            for (int k = 1; k < 9; k++) {
                if (!((F.F >> k) & 1u))
                    continue;
                double v = -Ahc + Atc * (tpc - F.t); /* this cell's outflow */
                if ((F.inside >> k) & 1u) {
                    const int2 m = db.map[F.cn[k]];
                    if (m.x == epoch_b) { /* the receiver's inflow (its tile is in the list) */
                        const double Ahr = a.Ah[m.y], Atr = a.At[m.y], tpr = a.tp[m.y];
                        v += Ahr + Atr * (F.t - tpr);
                        lt_add += Atr * F.f[k]; /* the receiver's heat term f * t */
                    }
                }
                lf[k] = v;
            }
            /* f[k] = Pr(t) (avg - H[k]), avg = (h0 + sum_S H) / |S| */
            const double dPr = F.Pr * db.ph.b * 2.302585092994045684;
            double G = 0.0, lH[9];
#pragma unroll
            for (int k = 0; k < 9; k++)
                lH[k] = 0.0;
#pragma unroll
            for (int k = 1; k < 9; k++)
                if ((F.F >> k) & 1u) {
                    G += lf[k] * F.Pr;
                    lH[k] -= lf[k] * F.Pr;
                    lt_add += lf[k] * dPr * (F.avg - F.H[k]);
                }
            const double g = G / (double)F.nS;
#pragma unroll
            for (int k = 0; k < 9; k++)
                if ((F.S >> k) & 1u)
                    lH[k] += g;
            atomicAdd(a.lh + x, g); /* avg's h[0] */
            atomicAdd(a.lt + x, lt_add);
            const double inv = 1.0 / db.ph.rad2;
#pragma unroll
            for (int k = 0; k < 9; k++) {
                if (lH[k] == 0.0)
                    continue;
                const bool in = (F.inside >> k) & 1u;
                /* H[k] = z[k] + h[k] for k >= 1, H[0] = z[0] */
                if (k >= 1 && in)
                    atomicAdd(a.lh + F.cn[k], lH[k]);
                if (k < 5) {
                    if (in)
                        atomicAdd(a.lz + F.cn[k], lH[k]);
                } else {
                    /* z[k] = sz0 - (sz0 - sz_k) / rad2 */
                    if (in)
                        atomicAdd(a.lz + F.cn[k], lH[k] * inv);
                    atomicAdd(a.lz + x, lH[k] * (1.0 - inv));
                }
            }
        }
    }
}

__global__ void k_bvents(const __grid_constant__ Dev d, const __grid_constant__ Adj a, const double* vtape, int phase)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= d.B)
        return;
    for (int v = d.vent_first[b]; v < d.vent_first[b + 1]; v++) {
        const double* rec = vtape + 3 * v;
        const int eff = (int)rec[2];
        if (eff < 0)
            continue; /* not the cell's first vent, or no emission */
        const int c = d.vent_cell[v];
        if (phase < d.nphases)
            a.grad[(size_t)eff * d.nphases + phase] += a.lh[c] * d.ph.Pclock / d.ph.Pac;
        a.lt[c] = 0.0;
        d.Slt[c] = rec[0];
        d.St[c] = rec[1];
    }
}

/* dL/dSlt_T = 2 (Slt_T - target), the other adjoints 0; per-scenario loss */
__global__ void k_bloss(const __grid_constant__ Dev d, const __grid_constant__ Adj a, const double* tgt, double* loss)
{
    __shared__ long long s_offs[MAX_INST + 1];
    for (int k = threadIdx.x; k <= d.B; k += blockDim.x)
        s_offs[k] = d.offs[k];
    __syncthreads();
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < d.ncells; c += (long long)gridDim.x * blockDim.x) {
        const int b = locate(s_offs, d.B, c);
        const Inst I = d.inst[b];
        const bool valid = c - I.off < (long long)I.rows * I.cols;
        const double diff = valid ? d.Slt[c] - tgt[c] : 0.0;
        a.lh[c] = 2.0 * diff;
        a.lt[c] = 0.0;
        a.lz[c] = 0.0;
        if (valid && diff != 0.0)
            atomicAdd(loss + b, diff * diff);
    }
}

/* MakeBorder (Sciara.cpp:206-250) on the device, the border reset of the
 * initial state, and the first lava list */
__global__ void k_prime(const __grid_constant__ Dev d)
{
    __shared__ long long s_offs[MAX_INST + 1];
    for (int k = threadIdx.x; k <= d.B; k += blockDim.x)
        s_offs[k] = d.offs[k];
    __syncthreads();
    unsigned char* Mb = const_cast<unsigned char*>(d.Mb);
    for (long long c0 = (long long)blockIdx.x * blockDim.x; c0 < d.ncells; c0 += (long long)gridDim.x * blockDim.x) {
        const long long c = c0 + threadIdx.x;
        bool lava = false;
        if (c < d.ncells) {
            const Inst I = d.inst[locate(s_offs, d.B, c)];
            const long long lc = c - I.off;
            if (lc < (long long)I.rows * I.cols) {
                const int i = (int)(lc / I.cols), j = (int)(lc - (long long)i * I.cols);
                bool border = false;
                if (d.Sz[c] >= 0) {
                    if (i == 0 || i == I.rows - 1 || j == 0 || j == I.cols - 1) {
                        border = true;
                    } else {
                        for (int k = 1; k < 9 && !border; k++) {
                            long long cn;
                            if (nbr(I, i, j, k, &cn) && d.Sz[cn] < 0)
                                border = true;
                        }
                    }
                }
                Mb[c] = border ? 1 : 0;
                if (border) {
                    d.Slt[c] = 0;
                    d.St[c] = 0;
                } else if (cal_d2i(d.Slt[c]) == (long long)0x8000000000000000LL) {
                    d.Slt[c] = 0; /* -0 thickness: the first update would make it +0 */
                }
                lava = !border && d.Slt[c] > 0;
            } else {
                Mb[c] = 0;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, lava);
        if (m) {
            const int lane = threadIdx.x & 31;
            int base = 0;
            if (lane == 0)
                base = atomicAdd(d.counts + 0, __popc(m));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (lava) {
                const int pos = base + __popc(m & ((1u << lane) - 1u));
                if (pos < d.capacity)
                    d.list[pos] = (int)c;
                else
                    atomicExch(d.counts + 8, 1);
            }
        }
    }
}

struct Batch {
    int B = 0, nvents = 0, nphases = 0;
    unsigned emission_time = 0;
    long long N = 0;
    int ntiles = 0, capacity = 0;
    std::vector<Inst> inst;
    std::vector<long long> offs;
    Dev d;
    double effusion_duration = 0;
    std::vector<int> vent_order; /* internal vent k -> the caller's vent index */
    double *Sz0 = nullptr, *Slt0 = nullptr, *St0 = nullptr; /* the initial state, for every run */
    cudaStream_t st = nullptr;
    void* allocs[32] = {};
    int nalloc = 0;
    bool primed = false;
};

template <typename T>
static bool dalloc(Batch& bt, T** p, size_t bytes)
{
    if (bt.nalloc >= (int)(sizeof(bt.allocs) / sizeof(bt.allocs[0])) || cudaMalloc(p, bytes) != cudaSuccess)
        return false;
    bt.allocs[bt.nalloc++] = *p;
    return true;
}

static void destroy(Batch* bt)
{
    if (bt->st)
        cudaStreamSynchronize(bt->st);
    for (int k = 0; k < bt->nalloc; k++)
        cudaFree(bt->allocs[k]);
    if (bt->st)
        cudaStreamDestroy(bt->st);
    delete bt;
}

} // namespace sci2

using sci2::Batch;

/* Create B SCIARA-fv2 scenarios.  dims: 2B ints (rows, cols); z0, slt0, st0:
 * the scenarios' morphology, initial thickness and temperature back to back
 * (unpadded, row-major; slt0 / st0 may be NULL for zero); params: the 13
 * physical parameters (Pclock, PTsol, PTvent, Pr(Tsol), Pr(Tvent),
 * Phc(Tsol), Phc(Tvent), Pcool, Prho, Pepsilon, Psigma, Pcv, Pc); vents:
 * vent_inst[v] = scenario, vent_xy[2v..2v+1] = (x, y), in each scenario's
 * vent order; rates: nvents x nphases m^3/s, each phase emission_time
 * seconds.  list_fraction: lava-list capacity as a fraction of all cells,
 * or <= 0 for the default (all cells up to 16M cells, an eighth beyond); a
 * run that needs more reports CAL_ERROR_OUT_OF_MEMORY. */
extern "C" void* cal_sciara_batch_create(int B, const int* dims, const double* z0, const double* slt0,
                                         const double* st0, const double* params, int nvents, const int* vent_inst,
                                         const int* vent_xy, unsigned emission_time, int nphases, const double* rates,
                                         double list_fraction)
{
    if (B <= 0 || B > sci2::MAX_INST || nvents < 0 || nphases < 0 || emission_time == 0)
        return nullptr;
    Batch* bt = new Batch();
    bt->B = B;
    bt->nvents = nvents;
    bt->nphases = nphases;
    bt->emission_time = emission_time;
    bt->offs.assign(B + 1, 0);
    int tiles = 0;
    for (int b = 0; b < B; b++) {
        sci2::Inst I;
        memset(&I, 0, sizeof(I));
        I.rows = dims[2 * b];
        I.cols = dims[2 * b + 1];
        if (I.rows < 3 || I.cols < 3) {
            delete bt;
            return nullptr;
        }
        I.off = bt->offs[b];
        I.tiles_x = (I.cols + sci2::TW - 1) / sci2::TW;
        I.tiles_y = (I.rows + sci2::TH - 1) / sci2::TH;
        I.tile0 = tiles;
        tiles += I.tiles_x * I.tiles_y;
        bt->inst.push_back(I);
        const long long n = (long long)I.rows * I.cols;
        bt->offs[b + 1] = bt->offs[b] + (n + 31) / 32 * 32;
    }
    bt->N = bt->offs[B];
    bt->ntiles = tiles;
    /* default (list_fraction <= 0): every cell up to 16M cells, an eighth
     * beyond (lava covers a small part of a large volcano) */
    if (list_fraction <= 0)
        list_fraction = bt->N <= (16LL << 20) ? 1.0 : 0.125;
    const double frac = list_fraction > 1.0 ? 1.0 : list_fraction;
    bt->capacity = (int)std::min<long long>(bt->N, std::max<long long>(1024, (long long)(frac * bt->N)));
    /* vents: packed cell indices, grouped by scenario in the given order */
    std::vector<int> vcell(nvents), vfirst(B + 1, 0);
    std::vector<double> vrates((size_t)nvents * nphases);
    {
        std::vector<int> order(nvents);
        for (int v = 0; v < nvents; v++)
            order[v] = v;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return vent_inst[a] < vent_inst[b]; });
        bt->vent_order = order;
        for (int k = 0; k < nvents; k++) {
            const int v = order[k];
            const int b = vent_inst[v];
            const int x = vent_xy[2 * v], y = vent_xy[2 * v + 1];
            if (b < 0 || b >= B || x < 0 || y < 0 || x >= bt->inst[b].cols || y >= bt->inst[b].rows) {
                delete bt;
                return nullptr;
            }
            vcell[k] = (int)(bt->inst[b].off + (long long)y * bt->inst[b].cols + x);
            vfirst[b + 1]++;
            for (int p = 0; p < nphases; p++)
                vrates[(size_t)k * nphases + p] = rates[(size_t)v * nphases + p];
        }
        for (int b = 0; b < B; b++)
            vfirst[b + 1] += vfirst[b];
    }
    /* vent cells (groups) with, per phase, the vent that takes effect */
    std::vector<int> g_cell, g_member, g_mfirst(1, 0), g_eff;
    std::vector<double> g_emit;
    {
        const double Pac = params[12] * params[12], Pclock = params[0];
        for (int b = 0; b < B; b++)
            for (int v = vfirst[b]; v < vfirst[b + 1]; v++) {
                bool lead = true;
                for (int w = vfirst[b]; w < v; w++)
                    if (vcell[w] == vcell[v])
                        lead = false;
                if (!lead)
                    continue;
                g_cell.push_back(vcell[v]);
                for (int w = v; w < vfirst[b + 1]; w++)
                    if (vcell[w] == vcell[v])
                        g_member.push_back(w);
                g_mfirst.push_back((int)g_member.size());
                for (int p = 0; p < nphases; p++) {
                    int eff = -1;
                    double e = 0.0;
                    for (int m = g_mfirst[g_mfirst.size() - 2]; m < g_mfirst.back(); m++) {
                        /* updateVentsEmission's thickness, rate / Pac * Pclock */
                        const double em = vrates[(size_t)g_member[m] * nphases + p] / Pac * Pclock;
                        if (em > 0) {
                            eff = g_member[m];
                            e = em;
                        }
                    }
                    g_eff.push_back(eff);
                    g_emit.push_back(e);
                }
            }
    }
    const int ngroups = (int)g_cell.size();
    sci2::Dev& d = bt->d;
    memset(&d, 0, sizeof(d));
    d.B = B;
    d.ncells = bt->N;
    d.capacity = bt->capacity;
    d.nvents = nvents;
    d.nphases = nphases;
    d.emission_time = emission_time;
    d.ph.Pclock = params[0];
    d.ph.PTsol = params[1];
    d.ph.PTvent = params[2];
    const double Pr_Tsol = params[3], Pr_Tvent = params[4], Phc_Tsol = params[5], Phc_Tvent = params[6];
    d.ph.Pcool = params[7];
    d.ph.Prho = params[8];
    d.ph.Pepsilon = params[9];
    d.ph.Psigma = params[10];
    d.ph.Pcv = params[11];
    d.ph.Pc = params[12];
    d.ph.Pac = d.ph.Pc * d.ph.Pc;
    d.ph.rad2 = sqrt(2.0);
    d.ph.rrad2 = 1.0 / d.ph.rad2;
    d.ph.rad2_recip = cal_recip_exact_ok(d.ph.rad2, d.ph.rrad2) ? 1 : 0;
    d.ph.w2 = d.ph.Pc * d.ph.Pc;
    /* evaluatePowerLawParams (Sciara.cpp:199-204), C library log10 */
    d.ph.b = (log10(Pr_Tvent) - log10(Pr_Tsol)) / (d.ph.PTvent - d.ph.PTsol);
    d.ph.a = log10(Pr_Tsol) - d.ph.b * (d.ph.PTsol);
    d.ph.d = (log10(Phc_Tvent) - log10(Phc_Tsol)) / (d.ph.PTvent - d.ph.PTsol);
    d.ph.c = log10(Phc_Tsol) - d.ph.d * (d.ph.PTsol);
    bt->effusion_duration = (double)emission_time * nphases;

    const size_t nb = (size_t)bt->N * sizeof(double);
    bool ok = cudaStreamCreateWithFlags(&bt->st, cudaStreamNonBlocking) == cudaSuccess &&
              sci2::dalloc(*bt, (sci2::Inst**)&d.inst, sizeof(sci2::Inst) * B) &&
              sci2::dalloc(*bt, (long long**)&d.offs, sizeof(long long) * (B + 1)) &&
              sci2::dalloc(*bt, &d.Sz, nb) && sci2::dalloc(*bt, &d.Slt, nb) && sci2::dalloc(*bt, &d.St, nb) &&
              sci2::dalloc(*bt, &d.Msl, nb) && sci2::dalloc(*bt, (unsigned char**)&d.Mb, (size_t)bt->N) &&
              sci2::dalloc(*bt, &d.map, sizeof(int2) * (size_t)bt->N) &&
              sci2::dalloc(*bt, &d.recv, sizeof(int) * (size_t)bt->N) &&
              sci2::dalloc(*bt, &d.rlist, sizeof(int) * (size_t)bt->capacity) &&
              sci2::dalloc(*bt, &d.list, sizeof(int) * (size_t)bt->capacity) &&
              sci2::dalloc(*bt, &d.mask, sizeof(unsigned) * 16 * (size_t)tiles) &&
              sci2::dalloc(*bt, &d.fc, sizeof(double) * 16 * (size_t)bt->capacity) &&
              sci2::dalloc(*bt, &d.counts, 16 * sizeof(int)) &&
              sci2::dalloc(*bt, &d.tflag, sizeof(int) * (size_t)tiles) &&
              sci2::dalloc(*bt, &d.tlist, sizeof(int) * (size_t)tiles) &&
              sci2::dalloc(*bt, (int**)&d.vent_cell, sizeof(int) * std::max(1, nvents)) &&
              sci2::dalloc(*bt, (int**)&d.vent_first, sizeof(int) * (B + 1)) &&
              sci2::dalloc(*bt, (int**)&d.g_cell, sizeof(int) * std::max(1, ngroups)) &&
              sci2::dalloc(*bt, (int**)&d.g_member, sizeof(int) * std::max(1, nvents)) &&
              sci2::dalloc(*bt, (int**)&d.g_mfirst, sizeof(int) * (ngroups + 1)) &&
              sci2::dalloc(*bt, (int**)&d.g_eff, sizeof(int) * std::max<size_t>(1, g_eff.size())) &&
              sci2::dalloc(*bt, (double**)&d.g_emit, sizeof(double) * std::max<size_t>(1, g_emit.size())) &&
              sci2::dalloc(*bt, &bt->Sz0, nb) && sci2::dalloc(*bt, &bt->Slt0, nb) && sci2::dalloc(*bt, &bt->St0, nb);
    if (!ok) {
        fprintf(stderr, "opencal-gb300: cal_sciara_batch_create: out of device memory\n");
        sci2::destroy(bt);
        return nullptr;
    }
    cudaMemcpy((void*)d.inst, bt->inst.data(), sizeof(sci2::Inst) * B, cudaMemcpyHostToDevice);
    cudaMemcpy((void*)d.offs, bt->offs.data(), sizeof(long long) * (B + 1), cudaMemcpyHostToDevice);
    d.ngroups = ngroups;
    cudaMemcpy((void*)d.g_mfirst, g_mfirst.data(), sizeof(int) * (ngroups + 1), cudaMemcpyHostToDevice);
    if (nvents) {
        cudaMemcpy((void*)d.vent_cell, vcell.data(), sizeof(int) * nvents, cudaMemcpyHostToDevice);
        cudaMemcpy((void*)d.g_cell, g_cell.data(), sizeof(int) * ngroups, cudaMemcpyHostToDevice);
        cudaMemcpy((void*)d.g_member, g_member.data(), sizeof(int) * g_member.size(), cudaMemcpyHostToDevice);
        if (!g_eff.empty()) {
            cudaMemcpy((void*)d.g_eff, g_eff.data(), sizeof(int) * g_eff.size(), cudaMemcpyHostToDevice);
            cudaMemcpy((void*)d.g_emit, g_emit.data(), sizeof(double) * g_emit.size(), cudaMemcpyHostToDevice);
        }
    }
    cudaMemcpy((void*)d.vent_first, vfirst.data(), sizeof(int) * (B + 1), cudaMemcpyHostToDevice);
    cudaMemset(d.Sz, 0, nb);
    cudaMemset(d.Slt, 0, nb);
    cudaMemset(d.St, 0, nb);
    cudaMemset(d.Msl, 0, nb);
    size_t src = 0;
    for (int b = 0; b < B; b++) {
        const size_t n = (size_t)bt->inst[b].rows * bt->inst[b].cols;
        const long long o = bt->offs[b];
        cudaMemcpy(d.Sz + o, z0 + src, n * sizeof(double), cudaMemcpyHostToDevice);
        if (slt0)
            cudaMemcpy(d.Slt + o, slt0 + src, n * sizeof(double), cudaMemcpyHostToDevice);
        if (st0)
            cudaMemcpy(d.St + o, st0 + src, n * sizeof(double), cudaMemcpyHostToDevice);
        src += n;
    }
    cudaMemcpy(bt->Sz0, d.Sz, nb, cudaMemcpyDeviceToDevice);
    cudaMemcpy(bt->Slt0, d.Slt, nb, cudaMemcpyDeviceToDevice);
    cudaMemcpy(bt->St0, d.St, nb, cudaMemcpyDeviceToDevice);
    if (cudaGetLastError() != cudaSuccess) {
        sci2::destroy(bt);
        return nullptr;
    }
    return bt;
}

extern "C" void cal_sciara_batch_destroy(void* handle)
{
    if (handle)
        sci2::destroy((Batch*)handle);
}

namespace sci2 {

/* the run from the initial state: calRun2D's loop with the stop condition
 * of Sciara.cpp:177-183 (elapsed time >= emission's end).  With a tape the
 * undo records of every step are kept (vtape: steps x nvents x 3). */
static int forward(Batch* bt, int max_steps, const Tape* tape, double* vtape, std::vector<double>* elapsed_of,
                   int* steps_done, float* ms)
{
    Dev& d = bt->d;
    cudaStream_t st = bt->st;
    const size_t nb = (size_t)bt->N * sizeof(double);
    cudaMemcpyAsync(d.Sz, bt->Sz0, nb, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(d.Slt, bt->Slt0, nb, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(d.St, bt->St0, nb, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(d.Msl, 0, nb, st);
    cudaMemsetAsync(d.counts, 0, 16 * sizeof(int), st);
    cudaMemsetAsync(d.map, 0, sizeof(int2) * (size_t)bt->N, st);
    cudaMemsetAsync(d.recv, 0, sizeof(int) * (size_t)bt->N, st);
    cudaMemsetAsync(d.mask, 0, sizeof(unsigned) * 16 * (size_t)bt->ntiles, st);
    cudaMemsetAsync(d.tflag, 0, sizeof(int) * (size_t)bt->ntiles, st);
    const int one = 1;
    cudaMemcpyAsync(d.counts + 6, &one, sizeof(int), cudaMemcpyHostToDevice, st);
    int blocks = (int)std::min<long long>((bt->N + T - 1) / T, 152 * 16);
    k_prime<<<blocks, T, 0, st>>>(d);
    Tape tp;
    memset(&tp, 0, sizeof(tp));
    if (tape)
        tp = *tape;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    double elapsed = 0.0;
    int done = 0;
    for (int step = 1; max_steps <= 0 || step <= max_steps; step++) {
        if (elapsed_of)
            elapsed_of->push_back(elapsed);
        /* the phase as the vent process forms it: (unsigned)(elapsed / emission_time) */
        const unsigned phase = (unsigned)(elapsed / (double)bt->emission_time);
        k_collect<<<K2_BLOCKS, T, 0, st>>>(d, phase, vtape ? vtape + (size_t)done * 3 * bt->nvents : nullptr,
                                           done > 0);
        k_flows<<<152 * 32, K1T, 0, st>>>(d);
        if (tp.state)
            k_tape<<<K2_BLOCKS, T, 0, st>>>(d, tp);
        k_update<<<152 * 32, K1T, 0, st>>>(d, tp, done);
        done++;
        elapsed += d.ph.Pclock;
        if (elapsed >= bt->effusion_duration)
            break;
    }
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms)
        *ms = t;
    if (steps_done)
        *steps_done = done;
    int flags[3] = {0, 0, 0};
    cudaMemcpy(flags, d.counts + 8, sizeof(flags), cudaMemcpyDeviceToHost);
    if (cudaGetLastError() != cudaSuccess)
        return 3; /* CAL_ERROR_CUDA */
    return (flags[0] || flags[2]) ? 2 /* CAL_ERROR_OUT_OF_MEMORY: lava list or tape too small */ : 0;
}

/* steps a run takes (the stop condition's accumulation of the clock) */
static int run_length(const Batch* bt, int max_steps)
{
    double elapsed = 0.0;
    int done = 0;
    for (int step = 1; max_steps <= 0 || step <= max_steps; step++) {
        done++;
        elapsed += bt->d.ph.Pclock;
        if (elapsed >= bt->effusion_duration)
            break;
    }
    return done;
}

} // namespace sci2

/* Run every scenario from its initial state (as created) until the emission ends (or
 * max_steps > 0 steps); the state stays on the device for
 * cal_sciara_batch_read.  steps_done: steps run; ms: device time of the step
 * loop.  0, or a CALError code (CAL_ERROR_OUT_OF_MEMORY = list overflow). */
extern "C" int cal_sciara_batch_run(void* handle, int max_steps, int* steps_done, float* ms)
{
    return sci2::forward((Batch*)handle, max_steps, nullptr, nullptr, nullptr, steps_done, ms);
}

/* Loss L_b = sum over scenario b of (Slt_T - target)^2 and its gradient
 * with respect to every emission rate, by the adjoint with the forward's
 * decisions frozen.  target: host array, the scenarios' grids back to back
 * (unpadded); loss_out[B]; grad_out[nvents x nphases] in the caller's vent
 * order.  tape_slots: undo-tape capacity in tiles summed over the steps
 * (0: twice the scenarios' tiles + 4096, and when that proves too small,
 * the forward runs once more with a tape of the size it asked for; a given
 * tape_slots that is too small is an error).  The state after the call is the
 * run's final one for Slt, St, Sz (Msl is not restored).  0 or a CALError
 * code; ms: device time of forward + adjoint. */
extern "C" int cal_sciara_batch_loss_grad(void* handle, const double* target, int max_steps, double* loss_out,
                                          double* grad_out, int* steps_done, long long tape_slots, float* ms)
{
    Batch* bt = (Batch*)handle;
    sci2::Dev& d = bt->d;
    cudaStream_t st = bt->st;
    const int steps = sci2::run_length(bt, max_steps);
    const long long cap = tape_slots > 0 ? tape_slots : 2LL * bt->ntiles + 4096;
    const size_t tile_cells = (size_t)sci2::TW * sci2::TH;
    sci2::Tape tp;
    memset(&tp, 0, sizeof(tp));
    tp.cap = cap;
    double* vtape = nullptr;
    double* tgt = nullptr;
    double* dloss = nullptr;
    sci2::Adj a;
    memset(&a, 0, sizeof(a));
    std::vector<void*> mem;
    auto alloc = [&](void** p, size_t bytes) {
        if (cudaMalloc(p, bytes) != cudaSuccess)
            return false;
        mem.push_back(*p);
        return true;
    };
    const size_t nb = (size_t)bt->N * sizeof(double);
    bool ok = alloc((void**)&tp.step_base, sizeof(int) * (steps + 1)) &&
              alloc((void**)&tp.step_count, sizeof(int) * (steps + 1)) &&
              alloc((void**)&vtape, sizeof(double) * 3 * std::max(1, bt->nvents) * (size_t)steps) &&
              alloc((void**)&tgt, nb) && alloc((void**)&dloss, sizeof(double) * bt->B) &&
              alloc((void**)&a.lh, nb) && alloc((void**)&a.lt, nb) && alloc((void**)&a.lz, nb) &&
              alloc((void**)&a.grad, sizeof(double) * std::max(1, bt->nvents * bt->nphases));
    auto free_tape = [&]() {
        cudaStreamSynchronize(st);
        cudaFree(tp.tile);
        cudaFree(tp.state);
        tp.tile = nullptr;
        tp.state = nullptr;
    };
    auto alloc_tape = [&](long long slots) {
        tp.cap = slots;
        if (cudaMalloc((void**)&tp.tile, sizeof(int) * slots) != cudaSuccess ||
            cudaMalloc((void**)&tp.state, sizeof(double) * 3 * tile_cells * slots) != cudaSuccess) {
            cudaGetLastError();
            free_tape();
            return false;
        }
        return true;
    };
    auto release = [&]() {
        free_tape();
        for (void* p : mem)
            cudaFree(p);
    };
    if (!ok || !alloc_tape(cap)) {
        release();
        return 2; /* CAL_ERROR_OUT_OF_MEMORY */
    }
    /* target in the padded layout: an input, copied before the timed region */
    cudaMemsetAsync(tgt, 0, nb, st);
    size_t src = 0;
    for (int b = 0; b < bt->B; b++) {
        const size_t n = (size_t)bt->inst[b].rows * bt->inst[b].cols;
        cudaMemcpyAsync(tgt + bt->offs[b], target + src, n * sizeof(double), cudaMemcpyHostToDevice, st);
        src += n;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    std::vector<double> elapsed_of;
    int done = 0;
    int rc = sci2::forward(bt, max_steps, &tp, vtape, &elapsed_of, &done, nullptr);
    if (rc == 2 && tape_slots <= 0) {
        /* the default tape was too small but the lava list was not: the
         * forward counted every slot it wanted, so run it again once with
         * a tape of exactly that size */
        int c[3] = {0, 0, 0};
        cudaMemcpy(c, d.counts + 8, sizeof(c), cudaMemcpyDeviceToHost);
        if (!c[0] && c[2] && c[1] > cap) {
            const long long need = c[1];
            free_tape();
            if (!alloc_tape(need)) {
                release();
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                return 2;
            }
            elapsed_of.clear();
            cudaEventRecord(e0, st);
            rc = sci2::forward(bt, max_steps, &tp, vtape, &elapsed_of, &done, nullptr);
        }
    }
    if (rc) {
        release();
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return rc;
    }
    cudaMemsetAsync(dloss, 0, sizeof(double) * bt->B, st);
    cudaMemsetAsync(a.grad, 0, sizeof(double) * std::max(1, bt->nvents * bt->nphases), st);
    const int blocks = (int)std::min<long long>((bt->N + sci2::T - 1) / sci2::T, 152 * 16);
    sci2::k_bloss<<<blocks, sci2::T, 0, st>>>(d, a, tgt, dloss);
    /* backward scratch: the largest step's tiles */
    std::vector<int> base(done), count(done);
    cudaMemcpyAsync(base.data(), tp.step_base, sizeof(int) * done, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(count.data(), tp.step_count, sizeof(int) * done, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    int maxc = 1;
    for (int t = 0; t < done; t++)
        maxc = std::max(maxc, count[t]);
    const size_t nc = (size_t)maxc * tile_cells;
    ok = alloc((void**)&a.fcb, sizeof(double) * 16 * nc) && alloc((void**)&a.Ah, sizeof(double) * nc) &&
         alloc((void**)&a.At, sizeof(double) * nc) && alloc((void**)&a.tp, sizeof(double) * nc);
    if (!ok) {
        release();
        return 2;
    }
    sci2::Dev db = d;
    db.fc = a.fcb;
    for (int t = done - 1; t >= 0; t--) {
        const int epoch_b = -(t + 1);
        const int g = std::max(1, std::min(count[t], sci2::K2_BLOCKS));
        if (count[t] > 0) {
            sci2::k_brestore<<<g, sci2::T, 0, st>>>(d, tp, base[t], count[t]);
            sci2::k_bflows<<<g, sci2::T, 0, st>>>(db, tp, base[t], count[t], epoch_b);
            sci2::k_bcells<<<g, sci2::T, 0, st>>>(db, tp, a, base[t], count[t], epoch_b);
            sci2::k_bflowadj<<<g, sci2::T, 0, st>>>(db, tp, a, base[t], count[t], epoch_b);
        }
        const int phase = (int)(unsigned)(elapsed_of[t] / bt->emission_time);
        sci2::k_bvents<<<(bt->B + 63) / 64, 64, 0, st>>>(d, a, vtape + (size_t)t * 3 * bt->nvents, phase);
    }
    cudaEventRecord(e1, st);
    std::vector<double> grad((size_t)std::max(1, bt->nvents * bt->nphases));
    cudaMemcpyAsync(grad.data(), a.grad, sizeof(double) * grad.size(), cudaMemcpyDeviceToHost, st);
    if (loss_out)
        cudaMemcpyAsync(loss_out, dloss, sizeof(double) * bt->B, cudaMemcpyDeviceToHost, st);
    cudaEventSynchronize(e1);
    float t_ms = 0.f;
    cudaEventElapsedTime(&t_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms)
        *ms = t_ms;
    if (steps_done)
        *steps_done = done;
    if (grad_out)
        for (int k = 0; k < bt->nvents; k++)
            for (int p = 0; p < bt->nphases; p++)
                grad_out[(size_t)bt->vent_order[k] * bt->nphases + p] = grad[(size_t)k * bt->nphases + p];
    rc = cudaGetLastError() == cudaSuccess ? 0 : 3;
    release();
    /* the tape undid the run: run again so that reads see the final state,
     * as after cal_sciara_batch_run */
    if (!rc)
        rc = sci2::forward(bt, max_steps, nullptr, nullptr, nullptr, nullptr, nullptr);
    return rc;
}

/* the scenarios' final Sz, Slt, St, Msl, back to back and unpadded (any may be NULL) */
extern "C" int cal_sciara_batch_read(void* handle, double* z, double* slt, double* st, double* msl)
{
    Batch* bt = (Batch*)handle;
    cudaStreamSynchronize(bt->st);
    double* outs[4] = {z, slt, st, msl};
    const double* src[4] = {bt->d.Sz, bt->d.Slt, bt->d.St, bt->d.Msl};
    for (int q = 0; q < 4; q++) {
        if (!outs[q])
            continue;
        size_t pos = 0;
        for (int b = 0; b < bt->B; b++) {
            const size_t n = (size_t)bt->inst[b].rows * bt->inst[b].cols;
            cudaMemcpy(outs[q] + pos, src[q] + bt->offs[b], n * sizeof(double), cudaMemcpyDeviceToHost);
            pos += n;
        }
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

/* lava cells of the last step (all scenarios) */
extern "C" int cal_sciara_batch_lava_cells(void* handle)
{
    Batch* bt = (Batch*)handle;
    int c = 0;
    cudaStreamSynchronize(bt->st);
    cudaMemcpy(&c, bt->d.counts + 13, sizeof(int), cudaMemcpyDeviceToHost);
    return c;
}
