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

/* per cell: coefficients g, gz, w and partials of dL/dr, dL/deps */
__global__ void __launch_bounds__(T) k_coeffs(Geo geo, const double* __restrict__ z, const double* __restrict__ h,
                                              const double* __restrict__ lam, double r, double eps,
                                              long long eps_bits, double* __restrict__ g, double* __restrict__ gz,
                                              double* __restrict__ w, double* __restrict__ partial)
{
    __shared__ double sr[T / 32], se[T / 32];
    double pr = 0.0, pe = 0.0;
    for (long long c = blockIdx.x * (long long)T + threadIdx.x; c < geo.n; c += (long long)gridDim.x * T) {
        const int i = (int)(c / geo.cols), j = (int)(c - (long long)i * geo.cols);
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
            int k;
            double avg, u[5];
            eliminate(hc, z[c], u14, eps, &a_set, &k, &avg, u);
            if (k > 0) {
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
                gc = (r / k) * S;
                gzc = (a_set & 1u) ? gc : 0.0;
                pe += S * r * ((a_set & 1u) ? 0.0 : -1.0) / k;
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

/* lambda_t and lambda_z from the coefficients (gather: no atomics) */
__global__ void __launch_bounds__(T) k_gather(Geo geo, const double* __restrict__ lam_next,
                                              const double* __restrict__ g, const double* __restrict__ gz,
                                              const double* __restrict__ w, double* __restrict__ lam_out,
                                              double* __restrict__ lamz)
{
    for (long long c = blockIdx.x * (long long)T + threadIdx.x; c < geo.n; c += (long long)gridDim.x * T) {
        const int i = (int)(c / geo.cols), j = (int)(c - (long long)i * geo.cols);
        double from_nb = 0.0;
        long long cn;
        /* x is neighbour opp(d) of its neighbour d: north<->south (1<->4), west<->east (2<->3) */
        if (nb(geo, i, j, 1, &cn))
            from_nb += w[3 * geo.n + cn]; /* north cell's w towards its south (m = 4) */
        if (nb(geo, i, j, 2, &cn))
            from_nb += w[2 * geo.n + cn]; /* west cell's w towards its east (m = 3) */
        if (nb(geo, i, j, 3, &cn))
            from_nb += w[1 * geo.n + cn]; /* east cell's w towards its west (m = 2) */
        if (nb(geo, i, j, 4, &cn))
            from_nb += w[cn];             /* south cell's w towards its north (m = 1) */
        lam_out[c] = lam_next[c] + g[c] + from_nb;
        lamz[c] += gz[c] + from_nb;
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

/* one forward step from `h` into `h_next` (the fused kernel, bit-exact) */
static void fwd_step(const Work& W, const double* h, double* h_next, cudaStream_t st)
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
    sdt::launch<64, 32>(p, st);
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
    int cur = 0;
    const int grid = sdtadj::grid_for(W->n) > sdtadj::PBLOCKS ? sdtadj::PBLOCKS : sdtadj::grid_for(W->n);
    for (int s = W->nseg - 1; s >= 0; s--) {
        const int t0 = s * W->K;
        const int t1 = (t0 + W->K < W->steps) ? t0 + W->K : W->steps; /* states t0..t1-1 feed steps */
        /* recompute the states of the segment from its checkpoint */
        cudaMemcpyAsync(W->seg, W->ckpt + s * W->n, b, cudaMemcpyDeviceToDevice, st);
        for (int t = t0; t < t1 - 1; t++)
            sdtadj::fwd_step(*W, W->seg + (t - t0) * W->n, W->seg + (t - t0 + 1) * W->n, st);
        /* reverse through the segment */
        for (int t = t1 - 1; t >= t0; t--) {
            const double* ht = W->seg + (t - t0) * W->n;
            sdtadj::k_coeffs<<<grid, sdtadj::T, 0, st>>>(geo, W->z, ht, W->lam[cur], W->r, W->eps, eps_bits, W->g,
                                                         W->gz, W->w, W->partial);
            sdtadj::k_gather<<<sdtadj::grid_for(W->n), sdtadj::T, 0, st>>>(geo, W->lam[cur], W->g, W->gz, W->w,
                                                                            W->lam[1 - cur], W->lamz);
            cur = 1 - cur;
        }
    }
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
