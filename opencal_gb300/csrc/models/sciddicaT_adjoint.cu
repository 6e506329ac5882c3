/*
 * sciddicaT_adjoint.cu -- reverse-mode adjoint of a SCIDDICA-T rollout
 * (plain mode), for calibration.
 *
 * Forward model (one step, every wet cell c, h_c > epsilon):
 *   m = h_c - eps, u_0 = z_c + eps, u_n = z_nb(n) + h_nb(n) (n = 1..4),
 *   A_c = cells left by the minimisation, k_c = |A_c|,
 *   avg_c = (m + sum_{n in A_c} u_n) / k_c,
 *   f_{c,n} = r (avg_c - u_n) for n in A_c, n >= 1, else 0;
 *   h'_x = h_x + sum_n (f_{nb(n), opp(n)} - f_{x,n}).
 * The elimination sets A_c and the wet set are discrete: they are taken
 * from the forward state (recomputed bit-identically from h_t) and frozen,
 * so the derivative is that of the piecewise-linear map the forward
 * actually evaluated.
 *
 * Adjoint of one step, with lambda' = dL/dh_{t+1}:
 *   lf_{c,n} = lambda'_nb(n) - lambda'_c       (0 for absent neighbours'
 *                                               lambda' on a flat grid)
 *   S_c = sum_{n in A_c, n>=1} lf_{c,n},  g_c = (r / k_c) S_c
 *   w_{c,m} = g_c - r lf_{c,m} for m in A_c, m >= 1, else 0
 *   lambda_t(x) = lambda'_x + g_x + sum_d w_{nb(d), opp(d)}
 *   lambda_z(x) += [0 in A_x] g_x + sum_d w_{nb(d), opp(d)}
 *   dL/dr   += sum_c sum_{n in A_c, n>=1} lf_{c,n} (avg_c - u_n)
 *   dL/deps += sum_c S_c r ([0 in A_c] - 1) / k_c
 * and the initialisation z = z_dem - h0 where h0 > 0 adds
 *   dL/dh0 = lambda_0 - [h0 > 0] lambda_z.
 *
 * Memory: sqrt(T) checkpointing -- h is stored every K = ceil(sqrt(T))
 * steps during the forward; the backward recomputes one segment of K states
 * at a time from its checkpoint (bit-identical forward) and runs the
 * adjoint through it in reverse.
 *
 * Sparsity: the forward step (16 x 8 tiles) reports per tile whether a
 * cell of it is wet before and after the step; during the recompute those
 * flags are kept for every state of the segment.  The adjoint of a step
 * then visits only the tiles holding a wet cell (coefficients) and those
 * tiles and their edge neighbours (gather), updating lambda in place: in
 * every other cell g, gz and w are 0, so lambda and lambda_z are unchanged
 * there, bit for bit as the dense sweep leaves them.
 *
 * Reductions of the parameter gradients use per-block partials folded in a
 * fixed order (deterministic).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sciddicaT_kernels.cuh"

namespace sdtadj {

constexpr int T = 256;      /* threads per block */
constexpr int PBLOCKS = 1024; /* partials of the parameter gradients */
constexpr int TW = 16, TH = 8; /* forward tiles, also the adjoint's unit of work */

struct Work {
    int rows = 0, cols = 0, steps = 0, toroidal = 0, K = 0, nseg = 0;
    long long n = 0;
    double r = 0, eps = 0;
    double* z = nullptr;       /* z after the initialisation (z_dem - h0 where h0 > 0) */
    double* h0 = nullptr;      /* initial thickness as given */
    double* ckpt = nullptr;    /* (nseg) checkpoints: h at steps 0, K, 2K, ... */
    double* seg = nullptr;     /* (K + 1) states of the segment being reversed */
    double* lam[2] = {nullptr, nullptr};
    double* lamz = nullptr;
    double* g = nullptr;       /* g_c */
    double* gz = nullptr;      /* [0 in A_c] g_c */
    double* w = nullptr;       /* 4 * n: w_{c,m} */
    unsigned char* flags = nullptr; /* (K + 1) x tiles: the forward's tile_wet of each step of the segment */
    unsigned char* all_wet = nullptr; /* tiles: 3 (every tile visited) */
    int tiles_x = 0, tiles_y = 0;
    double* partial = nullptr; /* 2 * PBLOCKS */
    double* result = nullptr;  /* 2 */
};

/* z after init and the canonical h0 (the first step turns -0 into +0) */
__global__ void k_init(const double* __restrict__ z_dem, const double* __restrict__ h0, double* __restrict__ z,
                       double* __restrict__ h, long long n)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const double hv = h0[c];
        z[c] = hv > 0.0 ? z_dem[c] - hv : z_dem[c];
        h[c] = hv;
    }
}

struct Geo {
    int rows, cols, toroidal;
    long long n;
};

/* neighbour n = 1..4 (north, west, east, south) of (i, j); false outside a flat grid */
static __device__ __forceinline__ bool nb(const Geo& g, int i, int j, int n, long long* c)
{
    int a = i + (n == 1 ? -1 : (n == 4 ? 1 : 0));
    int b = j + (n == 2 ? -1 : (n == 3 ? 1 : 0));
    if (g.toroidal) {
        a = a < 0 ? a + g.rows : (a >= g.rows ? a - g.rows : a);
        b = b < 0 ? b + g.cols : (b >= g.cols ? b - g.cols : b);
    } else if ((unsigned)a >= (unsigned)g.rows || (unsigned)b >= (unsigned)g.cols) {
        return false;
    }
    *c = (long long)a * g.cols + b;
    return true;
}

/* the forward's elimination, returning the set, the count, the average and u */
static __device__ __forceinline__ void eliminate(double hc, double zc, const double u14[4], double eps,
                                                 unsigned* elim_out, int* k_out, double* avg_out, double u[5])
{
    const double m = hc - eps;
    u[0] = zc + eps;
#pragma unroll
    for (int q = 0; q < 4; q++)
        u[q + 1] = u14[q];
    unsigned elim = 0;
    double average;
    int cells_count;
    bool again;
    do {
        again = false;
        average = m;
        cells_count = 0;
#pragma unroll
        for (int q = 0; q < 5; q++)
            if (!(elim & (1u << q))) {
                average += u[q];
                cells_count++;
            }
        if (cells_count != 0)
            average = cal_div_small(average, cells_count);
#pragma unroll
        for (int q = 0; q < 5; q++)
            if (!(elim & (1u << q)) && cal_le(average, u[q])) {
                elim |= 1u << q;
                again = true;
            }
    } while (again);
    /* the set A (cells NOT eliminated) and its size when the last average was formed */
    unsigned a_set = 0;
    int k = 0;
#pragma unroll
    for (int q = 0; q < 5; q++)
        if (!(elim & (1u << q))) {
            a_set |= 1u << q;
            k++;
        }
    (void)cells_count;
    *elim_out = a_set;
    *k_out = k;
    *avg_out = average;
}

/* per cell of the visited tiles: coefficients g, gz, w and partials of
 * dL/dr, dL/deps; then lambda_t and lambda_z by a gather (no atomics) */
static __device__ __forceinline__ int tile_of(int i, int j, int tiles_x)
{
    return (i / TH) * tiles_x + (j / TW);
}

/* k_coeffs_tiles: the tiles whose flag has `mask` set (a wet cell in h_t):
 * block b takes tiles b, b + gridDim.x, ...; every cell of a visited tile
 * is written (0 at dry cells) */
__global__ void __launch_bounds__(T) k_coeffs_tiles(Geo geo, const double* __restrict__ z,
                                                    const double* __restrict__ h, const double* __restrict__ lam,
                                                    double r, double eps, long long eps_bits,
                                                    double* __restrict__ g, double* __restrict__ gz,
                                                    double* __restrict__ w, double* __restrict__ partial,
                                                    const unsigned char* __restrict__ flags, int mask,
                                                    int tiles_x, int ntiles)
{
    __shared__ double sr[T / 32], se[T / 32];
    double pr = 0.0, pe = 0.0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        if (!(flags[t] & mask))
            continue;
        const int ty = t / tiles_x, tx = t - ty * tiles_x;
        for (int k = threadIdx.x; k < TW * TH; k += T) {
            const int i = ty * TH + k / TW, j = tx * TW + k % TW;
            if (i >= geo.rows || j >= geo.cols)
                continue;
            const long long c = (long long)i * geo.cols + j;
            const double hc = h[c];
            double gc = 0.0, gzc = 0.0, wc[4] = {0.0, 0.0, 0.0, 0.0};
            if (sdt::is_wet(hc, eps_bits)) {
                double u14[4], lnb[4];
                bool in[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    long long cn;
                    in[q] = nb(geo, i, j, q + 1, &cn);
                    u14[q] = in[q] ? z[cn] + h[cn] : 0.0 + 0.0;
                    lnb[q] = in[q] ? lam[cn] : 0.0;
                }
                unsigned a_set;
                int kk;
                double avg, u[5];
                eliminate(hc, z[c], u14, eps, &a_set, &kk, &avg, u);
                if (kk > 0) {
                    const double lc = lam[c];
                    double S = 0.0, lf[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        lf[q] = 0.0;
                        if (a_set & (1u << (q + 1))) {
                            lf[q] = lnb[q] - lc;
                            S += lf[q];
                            pr += lf[q] * (avg - u[q + 1]);
                        }
                    }
                    gc = cal_div_small(r, kk) * S; /* = (r / kk) * S: exact division by 1..5 on the integer pipe */
                    gzc = (a_set & 1u) ? gc : 0.0;
                    pe += cal_div_small(S * r * ((a_set & 1u) ? 0.0 : -1.0), kk);
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (a_set & (1u << (q + 1)))
                            wc[q] = gc - r * lf[q];
                }
            }
            g[c] = gc;
            gz[c] = gzc;
#pragma unroll
            for (int q = 0; q < 4; q++)
                w[q * geo.n + c] = wc[q];
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        pr += __shfl_down_sync(0xffffffffu, pr, o);
        pe += __shfl_down_sync(0xffffffffu, pe, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sr[threadIdx.x >> 5] = pr;
        se[threadIdx.x >> 5] = pe;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < T / 32; q++) {
            a += sr[q];
            b += se[q];
        }
        partial[blockIdx.x] += a;
        partial[PBLOCKS + blockIdx.x] += b;
    }
}

/* is tile (ty, tx) flagged?  Outside a flat grid: no */
static __device__ __forceinline__ bool tile_flag(const Geo& geo, const unsigned char* flags, int mask, int ty,
                                                 int tx, int tiles_x, int tiles_y)
{
    if (geo.toroidal) {
        ty = ty < 0 ? ty + tiles_y : (ty >= tiles_y ? ty - tiles_y : ty);
        tx = tx < 0 ? tx + tiles_x : (tx >= tiles_x ? tx - tiles_x : tx);
    } else if ((unsigned)ty >= (unsigned)tiles_y || (unsigned)tx >= (unsigned)tiles_x) {
        return false;
    }
    return (flags[ty * tiles_x + tx] & mask) != 0;
}

/* k_gather_tiles: in place, on the tiles that are flagged or have a flagged edge
 * neighbour; coefficients of unflagged tiles read as 0 (the dense sweep
 * wrote 0 there) */
__global__ void __launch_bounds__(T) k_gather_tiles(Geo geo, double* __restrict__ lam,
                                                    const double* __restrict__ g, const double* __restrict__ gz,
                                                    const double* __restrict__ w, double* __restrict__ lamz,
                                                    const unsigned char* __restrict__ flags, int mask, int tiles_x,
                                                    int tiles_y)
{
    const int ntiles = tiles_x * tiles_y;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int ty = t / tiles_x, tx = t - ty * tiles_x;
        const bool own = (flags[t] & mask) != 0;
        if (!own && !tile_flag(geo, flags, mask, ty - 1, tx, tiles_x, tiles_y) &&
            !tile_flag(geo, flags, mask, ty + 1, tx, tiles_x, tiles_y) &&
            !tile_flag(geo, flags, mask, ty, tx - 1, tiles_x, tiles_y) &&
            !tile_flag(geo, flags, mask, ty, tx + 1, tiles_x, tiles_y))
            continue;
        for (int k = threadIdx.x; k < TW * TH; k += T) {
            const int i = ty * TH + k / TW, j = tx * TW + k % TW;
            if (i >= geo.rows || j >= geo.cols)
                continue;
            const long long c = (long long)i * geo.cols + j;
            double from_nb = 0.0;
            long long cn;
            /* x is neighbour opp(d) of its neighbour d: north<->south (1<->4), west<->east (2<->3) */
            if (nb(geo, i, j, 1, &cn))
                from_nb += (flags[tile_of((int)(cn / geo.cols), (int)(cn % geo.cols), tiles_x)] & mask)
                               ? w[3 * geo.n + cn] : 0.0;
            if (nb(geo, i, j, 2, &cn))
                from_nb += (flags[tile_of((int)(cn / geo.cols), (int)(cn % geo.cols), tiles_x)] & mask)
                               ? w[2 * geo.n + cn] : 0.0;
            if (nb(geo, i, j, 3, &cn))
                from_nb += (flags[tile_of((int)(cn / geo.cols), (int)(cn % geo.cols), tiles_x)] & mask)
                               ? w[1 * geo.n + cn] : 0.0;
            if (nb(geo, i, j, 4, &cn))
                from_nb += (flags[tile_of((int)(cn / geo.cols), (int)(cn % geo.cols), tiles_x)] & mask)
                               ? w[cn] : 0.0;
            const double gc = own ? g[c] : 0.0, gzc = own ? gz[c] : 0.0;
            lam[c] = lam[c] + gc + from_nb;
            lamz[c] += gzc + from_nb;
        }
    }
}

__global__ void k_final_grad(const double* __restrict__ h0, const double* __restrict__ lam,
                             const double* __restrict__ lamz, double* __restrict__ g_h0, long long n)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        g_h0[c] = lam[c] - (h0[c] > 0.0 ? lamz[c] : 0.0);
}

__global__ void k_fold_partials(const double* __restrict__ partial, double* __restrict__ out)
{
    if (threadIdx.x < 2) {
        double a = 0.0;
        for (int b = 0; b < PBLOCKS; b++)
            a += partial[threadIdx.x * PBLOCKS + b];
        out[threadIdx.x] = a;
    }
}

static int grid_for(long long n)
{
    long long b = (n + T - 1) / T;
    return (int)(b > 152 * 8 ? 152 * 8 : (b < 1 ? 1 : b));
}

/* one forward step from `h` into `h_next` (the fused kernel, bit-exact);
 * tile_wet: optional per-tile wet flags before / after the step */
static void fwd_step(const Work& W, const double* h, double* h_next, cudaStream_t st,
                     unsigned char* tile_wet = nullptr)
{
    sdt::Params p;
    p.z = W.z;
    p.h = h;
    p.h_next = h_next;
    p.rows = W.rows;
    p.cols = W.cols;
    p.toroidal = W.toroidal;
    p.eps = W.eps;
    p.r = W.r;
    memcpy(&p.eps_bits, &W.eps, sizeof(double));
    p.tile_wet = tile_wet;
    sdt::launch<TW, TH>(p, st);
}

} // namespace sdtadj

using sdtadj::Work;

/* Workspace for rollouts of `steps` steps on a rows x cols grid. */
extern "C" void* cal_sdt_adj_create(int rows, int cols, int steps, int toroidal)
{
    Work* W = new Work();
    W->rows = rows;
    W->cols = cols;
    W->steps = steps;
    W->toroidal = toroidal;
    W->n = (long long)rows * cols;
    W->K = (int)ceil(sqrt((double)(steps > 0 ? steps : 1)));
    W->nseg = (steps + W->K - 1) / W->K;
    if (W->nseg < 1)
        W->nseg = 1;
    const size_t b = W->n * sizeof(double);
    bool ok = cudaMalloc(&W->z, b) == cudaSuccess && cudaMalloc(&W->h0, b) == cudaSuccess &&
              cudaMalloc(&W->ckpt, b * (size_t)W->nseg) == cudaSuccess &&
              cudaMalloc(&W->seg, b * (size_t)(W->K + 1)) == cudaSuccess &&
              cudaMalloc(&W->lam[0], b) == cudaSuccess && cudaMalloc(&W->lam[1], b) == cudaSuccess &&
              cudaMalloc(&W->lamz, b) == cudaSuccess && cudaMalloc(&W->g, b) == cudaSuccess &&
              cudaMalloc(&W->gz, b) == cudaSuccess && cudaMalloc(&W->w, 4 * b) == cudaSuccess &&
              cudaMalloc(&W->partial, 2 * sdtadj::PBLOCKS * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&W->result, 2 * sizeof(double)) == cudaSuccess;
    W->tiles_x = (cols + sdtadj::TW - 1) / sdtadj::TW;
    W->tiles_y = (rows + sdtadj::TH - 1) / sdtadj::TH;
    const size_t nt = (size_t)W->tiles_x * W->tiles_y;
    ok = ok && cudaMalloc(&W->flags, nt * (size_t)(W->K + 1)) == cudaSuccess &&
         cudaMalloc(&W->all_wet, nt) == cudaSuccess && cudaMemset(W->all_wet, 3, nt) == cudaSuccess;
    if (!ok) {
        fprintf(stderr, "opencal-gb300: cal_sdt_adj_create: out of device memory\n");
        return nullptr;
    }
    return W;
}

extern "C" void cal_sdt_adj_destroy(void* handle)
{
    Work* W = (Work*)handle;
    if (!W)
        return;
    cudaFree(W->z);
    cudaFree(W->h0);
    cudaFree(W->ckpt);
    cudaFree(W->seg);
    cudaFree(W->lam[0]);
    cudaFree(W->lam[1]);
    cudaFree(W->lamz);
    cudaFree(W->g);
    cudaFree(W->gz);
    cudaFree(W->w);
    cudaFree(W->partial);
    cudaFree(W->result);
    cudaFree(W->flags);
    cudaFree(W->all_wet);
    delete W;
}

/* Forward rollout on device buffers: init (z = z_dem - h0 where h0 > 0),
 * `steps` steps, h_T into hT; checkpoints kept for the backward. */
extern "C" int cal_sdt_adj_forward(void* handle, const double* z_dem, const double* h0, double p_r, double p_eps,
                                   double* hT, void* stream)
{
    Work* W = (Work*)handle;
    cudaStream_t st = (cudaStream_t)stream;
    W->r = p_r;
    W->eps = p_eps;
    const size_t b = W->n * sizeof(double);
    cudaMemcpyAsync(W->h0, h0, b, cudaMemcpyDeviceToDevice, st);
    double* cur = W->seg;
    double* nxt = W->seg + W->n;
    sdtadj::k_init<<<sdtadj::grid_for(W->n), sdtadj::T, 0, st>>>(z_dem, h0, W->z, cur, W->n);
    for (int t = 0; t < W->steps; t++) {
        if (t % W->K == 0)
            cudaMemcpyAsync(W->ckpt + (t / W->K) * W->n, cur, b, cudaMemcpyDeviceToDevice, st);
        sdtadj::fwd_step(*W, cur, nxt, st);
        double* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    if (W->steps == 0)
        cudaMemcpyAsync(W->ckpt, cur, b, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(hT, cur, b, cudaMemcpyDeviceToDevice, st);
    return (int)cudaGetLastError();
}

/* Backward: from dL/dh_T (gT) to dL/dh0 (g_h0, device) and dL/dp_r, dL/dp_eps
 * (host doubles; the call synchronises the stream). */
extern "C" int cal_sdt_adj_backward(void* handle, const double* gT, double* g_h0, double* g_r, double* g_eps,
                                    void* stream)
{
    Work* W = (Work*)handle;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t b = W->n * sizeof(double);
    long long eps_bits;
    memcpy(&eps_bits, &W->eps, sizeof(double));
    sdtadj::Geo geo = {W->rows, W->cols, W->toroidal, W->n};
    cudaMemcpyAsync(W->lam[0], gT, b, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(W->lamz, 0, b, st);
    cudaMemsetAsync(W->partial, 0, 2 * sdtadj::PBLOCKS * sizeof(double), st);
    const int ntiles = W->tiles_x * W->tiles_y;
    /* one resident wave of each kernel (blocks stride over the tiles): the
     * dry tiles cost a flag test, not a block launch */
    static int wave_c = 0, wave_g = 0;
    if (!wave_c) {
        int dev = 0, sms = 0, pc = 0, pg = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pc, sdtadj::k_coeffs_tiles, sdtadj::T, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pg, sdtadj::k_gather_tiles, sdtadj::T, 0);
        wave_c = sms * (pc > 0 ? pc : 1);
        wave_g = sms * (pg > 0 ? pg : 1);
    }
    int cgrid = ntiles < wave_c ? ntiles : wave_c;
    if (cgrid > sdtadj::PBLOCKS)
        cgrid = sdtadj::PBLOCKS;
    const int ggrid = ntiles < wave_g ? ntiles : wave_g;
    for (int s = W->nseg - 1; s >= 0; s--) {
        const int t0 = s * W->K;
        const int t1 = (t0 + W->K < W->steps) ? t0 + W->K : W->steps; /* states t0..t1-1 feed steps */
        /* recompute the states of the segment from its checkpoint, keeping
         * each step's tile flags (bit 0: wet before, bit 1: wet after) */
        cudaMemcpyAsync(W->seg, W->ckpt + s * W->n, b, cudaMemcpyDeviceToDevice, st);
        for (int t = t0; t < t1 - 1; t++)
            sdtadj::fwd_step(*W, W->seg + (t - t0) * W->n, W->seg + (t - t0 + 1) * W->n, st,
                             W->flags + (size_t)(t - t0) * ntiles);
        /* reverse through the segment: state t's wet tiles are bit 0 of the
         * step from t, or bit 1 of the step into it for the last state */
        for (int t = t1 - 1; t >= t0; t--) {
            const double* ht = W->seg + (t - t0) * W->n;
            const unsigned char* fl;
            int mask;
            if (t < t1 - 1) {
                fl = W->flags + (size_t)(t - t0) * ntiles;
                mask = 1;
            } else if (t > t0) {
                fl = W->flags + (size_t)(t - 1 - t0) * ntiles;
                mask = 2;
            } else {
                fl = W->all_wet; /* a one-state segment: no step reported on it */
                mask = 1;
            }
            sdtadj::k_coeffs_tiles<<<cgrid, sdtadj::T, 0, st>>>(geo, W->z, ht, W->lam[0], W->r, W->eps, eps_bits, W->g,
                                                               W->gz, W->w, W->partial, fl, mask, W->tiles_x, ntiles);
            sdtadj::k_gather_tiles<<<ggrid, sdtadj::T, 0, st>>>(geo, W->lam[0], W->g, W->gz, W->w, W->lamz, fl, mask,
                                                               W->tiles_x, W->tiles_y);
        }
    }
    const int cur = 0;
    sdtadj::k_final_grad<<<sdtadj::grid_for(W->n), sdtadj::T, 0, st>>>(W->h0, W->lam[cur], W->lamz, g_h0, W->n);
    sdtadj::k_fold_partials<<<1, 32, 0, st>>>(W->partial, W->result);
    double res[2] = {0.0, 0.0};
    cudaMemcpyAsync(res, W->result, sizeof(res), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    if (g_r)
        *g_r = res[0];
    if (g_eps)
        *g_eps = res[1];
    return (int)cudaGetLastError();
}
