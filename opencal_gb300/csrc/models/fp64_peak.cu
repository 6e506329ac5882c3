/*
 * fp64_peak.cu -- measured FP64 throughput of the GPU, the denominator of
 * the FP64 roofline the benchmark reports for the SCIDDICA-T step (its wet
 * cells are bound by GB300's narrow FP64 pipe, not by HBM).
 *
 * Every thread runs CHAINS independent dependency chains of ITERS
 * operations (enough independent work per warp to keep the pipe issuing);
 * the grid fills every SM with 8 resident blocks of 256 threads.  Timed
 * with CUDA events on the default stream after one warm-up launch.
 *   op 0: DFMA  (__fma_rn), 2 flops per instruction
 *   op 1: DADD  (__dadd_rn), 1 flop per instruction
 *   op 2: DMUL  (__dmul_rn), 1 flop per instruction
 * The results feed a store that no input can make false, so nothing is
 * optimised away.  No counterpart in the reference (a measurement aid).
 */
#include <cuda_runtime.h>

namespace fp64peak {

constexpr int THREADS = 256;
constexpr int CHAINS = 8;
constexpr int ITERS = 2048;

template <int OP>
__global__ void __launch_bounds__(THREADS) k_chains(double seed, double b, double c, double* sink)
{
    double a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; k++)
        a[k] = seed + (double)(threadIdx.x + k);
    for (int it = 0; it < ITERS; it++) {
#pragma unroll
        for (int k = 0; k < CHAINS; k++) {
            if (OP == 0)
                a[k] = __fma_rn(a[k], b, c);
            else if (OP == 1)
                a[k] = __dadd_rn(a[k], c);
            else
                a[k] = __dmul_rn(a[k], b);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < CHAINS; k++)
        s += a[k];
    if (s == -1.0) /* never true for these inputs */
        sink[blockIdx.x] = s;
}

template <int OP>
static int run(int blocks, double* sink, float* ms)
{
    /* b, c keep every chain finite and normal: |a| stays near 1 */
    const double b = 0.999999, c = 1e-6;
    k_chains<OP><<<blocks, THREADS>>>(1.0, b, c, sink);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0);
    k_chains<OP><<<blocks, THREADS>>>(1.0, b, c, sink);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

} // namespace fp64peak

/* FP64 operations per second of operation `op` (0 DFMA, 1 DADD, 2 DMUL),
 * counted as instructions (a DFMA is one instruction, two flops); *ms: the
 * timed launch's duration.  Returns 0, or 1 on a CUDA error. */
extern "C" int cal_fp64_peak(int op, double* instr_per_s, float* ms)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8;
    double* sink = nullptr;
    if (cudaMalloc(&sink, sizeof(double) * blocks) != cudaSuccess)
        return 1;
    float t = 0.f;
    int rc = op == 0 ? fp64peak::run<0>(blocks, sink, &t)
                     : (op == 1 ? fp64peak::run<1>(blocks, sink, &t) : fp64peak::run<2>(blocks, sink, &t));
    cudaFree(sink);
    if (rc || t <= 0.f)
        return 1;
    const double instr = (double)blocks * fp64peak::THREADS * fp64peak::CHAINS * fp64peak::ITERS;
    *instr_per_s = instr / (t * 1e-3);
    *ms = t;
    return 0;
}
