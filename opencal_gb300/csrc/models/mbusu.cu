/*
 * mbusu.cu -- the reference's mbusu example (OpenCAL/examples/cal_mbusu-glut/
 * source/mbusu.c: unsaturated subsurface flow, Richards' equation with van
 * Genuchten-Mualem pedofunctions, 160 x 30 x 130 cells of 5 m, von Neumann
 * 3D, toroidal, 8 real substates) written against this library's 3D C API:
 * the transition function is a device elementary process
 * (CAL_ELEMENTARY_PROCESS_3D, one thread per cell), the steering's minimum
 * of the time-step bounds is a device reduction
 * (calReductionOperationDevice3Dr) followed by a one-thread kernel that
 * forms the float time step and its float accumulation, and the stop
 * condition (10 days) is a device predicate, so a whole run can be one
 * device-driven loop (calRunDevice3D).
 *
 * Arithmetic is the reference's, operation by operation (--fmad=false), with
 * its types: lato, rain and delta_t are floats used directly (their products
 * are float), the soil constants are float values copied into doubles.  The
 * per-cell pow calls are CUDA's (the reference's are the C library's), so
 * results agree with the reference to rounding; the initial state and the
 * per-soil constants pow(alfa 734, n) are computed on the host with the C
 * library, exactly as the reference computes them.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "opencal/cal3D.h"
#include "opencal/cal3DDevice.cuh"
#include "opencal/cal3DReduction.h"
#include "opencal/cal3DRun.h"

#define MB_ROWS 160
#define MB_COLS 30
#define MB_SLICES 130
#define MB_XW 0
#define MB_XE 159
#define MB_YIN 0
#define MB_YOUT 29
#define MB_ZFONDO 0
#define MB_ZSUP 129

struct MbusuSubstates {
    struct CALSubstate3Dr *teta, *moist_cont, *psi, *k, *h, *dqdh, *convergence, *moist_diff;
};

/* one soil type: float constants held in doubles (the program copies its
 * float globals into double locals), plus teta at the initial head, which
 * every cell of the soil recomputes from the same inputs */
struct MbusuSoil {
    double tetas, tetar, alfa, n, ks;
    double teta_start;
};

__managed__ struct MbusuSubstates MQ;
__constant__ struct MbusuSoil mb_soil_dev[4];
__device__ float mb_delta_t;     /* the program's float delta_t */
__device__ float mb_cum;         /* delta_t_cum */
__device__ float mb_cum_prec;    /* delta_t_cum_prec */
__device__ double mb_min;        /* the steering's minimum time-step bound */

static const float mb_lato = (float)5.0;
#define MB_LATO_DEV ((float)5.0)
#define MB_RAIN_DEV ((float)0.000023148148)
static const int mb_output_time = 864000;

static struct MbusuSoil mb_soils_host[4];

/* soil of row i at inverted depth kinv (mbusu.c:53-86), 0-based type - 1 */
static __host__ __device__ __forceinline__ int mb_soil_index(int i, int kinv)
{
    if (i > 19 && i < 60 && kinv > 79 && kinv < 100)
        return 3;
    if (kinv > 111 && kinv < 124)
        return 1;
    if (kinv > 123)
        return 0;
    return 2;
}

/* the pedofunctions (mbusu.c:121-145) of head psi; pow is the caller's
 * (the C library's on the host, CUDA's on the device) */
struct MbusuPedo {
    double dqdh_inv, teta, moist, mdiff, k;
};

static __host__ __device__ __forceinline__ MbusuPedo mb_pedo(const MbusuSoil& s, double psi)
{
    MbusuPedo p;
    const double a1 = pow(s.alfa * (-psi), (1 - s.n));
    const double a2 = pow(s.alfa * (-psi), s.n);
    const double a3 = pow((1 / (1 + a2)), (1 / s.n - 2));
    p.dqdh_inv = (a1 / (s.alfa * (s.n - 1) * (s.tetas - s.tetar))) * a3;
    /* denom_pow = pow(alfa (-psi), n): the same call as a2 */
    p.teta = s.tetar + ((s.tetas - s.tetar) * pow((1 / (1 + a2)), (1 - 1 / s.n)));
    p.moist = p.teta / s.tetas;
    p.mdiff = p.moist - s.teta_start / s.tetas;
    const double satur = (p.teta - s.tetar) / (s.tetas - s.tetar);
    const double exp_c = s.n / (s.n - 1);
    const double sc = pow(satur, exp_c);
    const double exp_d = 1 - (1 / s.n);
    const double sd = pow((1 - sc), exp_d);
    p.k = s.ks * pow(satur, 0.5) * pow((1 - sd), 2.0);
    return p;
}

/* mbusuTransitionFunction (mbusu.c:34-169) */
CAL_ELEMENTARY_PROCESS_3D(mbusu_transition)(struct CALModel3D* ca, int i, int j, int k)
{
    const int kinv = (ca->slices - 1) - k;
    const float lato = MB_LATO_DEV;
    const double volume = lato * lato * lato;
    const double quota = lato * kinv;
    const MbusuSoil s = mb_soil_dev[mb_soil_index(i, kinv)];
    const float dt = mb_delta_t;
    double h = calGet3Dr(ca, MQ.h, i, j, k);
    const double kc = calGet3Dr(ca, MQ.k, i, j, k);
    const double dq = calGet3Dr(ca, MQ.dqdh, i, j, k);
    for (int n = 1; n < ca->sizeof_X; n++) {
        double dh = h - calGetX3Dr(ca, MQ.h, i, j, k, n);
        /* no flux across the domain's faces (neighbours 1..6: i-1, j-1,
         * j+1, i+1, k-1, k+1) */
        if ((kinv == MB_ZSUP && n == 5) || (kinv == MB_ZFONDO && n == 6) || (i == MB_XW && n == 1) ||
            (i == MB_XE && n == 4) || (j == MB_YOUT && n == 3) || (j == MB_YIN && n == 2))
            dh = 0;
        const double kmean_dq = ((kc + calGetX3Dr(ca, MQ.k, i, j, k, n)) / 2.0) * dq;
        h = h - ((dh / (lato * lato)) * dt * kmean_dq);
    }
    const int ymid = MB_YOUT / 2;
    if (kinv == MB_ZSUP && i < 45 && j > (ymid - 20) && j < (ymid + 20)) {
        const double rain = lato * MB_RAIN_DEV * dt / volume;
        h = h + rain * dq;
    }
    const double psi = h - quota;
    const MbusuPedo p = mb_pedo(s, psi);
    double bound;
    if ((p.k > 0) && (p.dqdh_inv > 0))
        bound = lato * lato / (6 * p.k * p.dqdh_inv);
    else
        bound = 1.0;
    calSet3Dr(ca, MQ.dqdh, i, j, k, p.dqdh_inv);
    calSet3Dr(ca, MQ.psi, i, j, k, psi);
    calSet3Dr(ca, MQ.k, i, j, k, p.k);
    calSet3Dr(ca, MQ.h, i, j, k, h);
    calSet3Dr(ca, MQ.teta, i, j, k, p.teta);
    calSet3Dr(ca, MQ.moist_cont, i, j, k, p.moist);
    calSet3Dr(ca, MQ.moist_diff, i, j, k, p.mdiff);
    calSet3Dr(ca, MQ.convergence, i, j, k, bound);
}

/* mbusuSimulationSteering (mbusu.c:278-301) after the reduction */
__global__ void mbusu_steer_kernel()
{
    double lo = mb_min;
    if (lo > 105.0)
        lo = 105.0;
    mb_delta_t = 0.95 * lo;
    mb_cum_prec = mb_cum;
    mb_cum += mb_delta_t;
}

__global__ void mbusu_reset_kernel()
{
    mb_delta_t = (float)10.0;
    mb_cum = 0.0f;
    mb_cum_prec = 0.0f;
}

static double* mb_min_ptr()
{
    void* p = nullptr;
    cudaGetSymbolAddress(&p, mb_min);
    return (double*)p;
}

static void mbusu_steering(struct CALModel3D* ca)
{
    calReductionOperationDevice3Dr(ca, MQ.convergence, REDUCTION_MIN, mb_min_ptr());
    mbusu_steer_kernel<<<1, 1, 0, (cudaStream_t)calGetStream3D(ca)>>>();
}

/* mbusuSimulationStopCondition (mbusu.c:303-348), the printing left to the
 * caller: on the device for the device-driven loop, on the host (reading
 * the device's accumulators) otherwise */
CAL_DEVICE_STOP_CONDITION_3D(mbusu_stop_device)(struct CALModel3D* ca)
{
    (void)ca;
    return (mb_cum >= 864000 && mb_cum_prec <= 864000) ? CAL_TRUE : CAL_FALSE;
}

static CALbyte mbusu_stop_host(struct CALModel3D* ca)
{
    float cum = 0.f, prec = 0.f;
    cudaStream_t st = (cudaStream_t)calGetStream3D(ca);
    cudaMemcpyFromSymbolAsync(&cum, mb_cum, sizeof(float), 0, cudaMemcpyDeviceToHost, st);
    cudaMemcpyFromSymbolAsync(&prec, mb_cum_prec, sizeof(float), 0, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    return (cum >= mb_output_time && prec <= mb_output_time) ? CAL_TRUE : CAL_FALSE;
}

/* mbusuSimulationInit (mbusu.c:176-276) on the host, C library pow */
static void mbusu_init_host(struct CALModel3D* ca)
{
    const double tetas[4] = {(float)0.368, (float)0.351, (float)0.325, (float)0.325};
    const double tetar[4] = {(float)0.102, (float)0.0985, (float)0.0859, (float)0.0859};
    const double alfa[4] = {(float)0.0334, (float)0.0363, (float)0.0345, (float)0.0345};
    const double nn[4] = {(float)1.982, (float)1.632, (float)1.573, (float)1.573};
    const double ks[4] = {(float)0.009154, (float)0.005439, (float)0.004803, (float)0.048032};
    for (int t = 0; t < 4; t++) {
        MbusuSoil& s = mb_soils_host[t];
        s.tetas = tetas[t];
        s.tetar = tetar[t];
        s.alfa = alfa[t];
        s.n = nn[t];
        s.ks = ks[t];
        const double dp0 = pow(s.alfa * (734), s.n);
        s.teta_start = s.tetar + ((s.tetas - s.tetar) * pow((1 / (1 + dp0)), (1 - 1 / s.n)));
    }
    cudaMemcpyToSymbol(mb_soil_dev, mb_soils_host, sizeof(mb_soils_host));
    const long long rc = (long long)ca->rows * ca->columns;
    const size_t n = (size_t)rc * ca->slices;
    double* buf = (double*)malloc(8 * n * sizeof(double)); /* teta, moist, psi, k, h, dqdh, mdiff, convergence */
    if (!buf)
        return;
    for (int k = 0; k < ca->slices; k++)
        for (int i = 0; i < ca->rows; i++)
            for (int j = 0; j < ca->columns; j++) {
                const int kinv = (ca->slices - 1) - k;
                const double quota = mb_lato * kinv;
                const double h = -734 + quota;
                const double psi = h - quota;
                const MbusuPedo p = mb_pedo(mb_soils_host[mb_soil_index(i, kinv)], psi);
                const size_t c = (size_t)(k * rc + (long long)i * ca->columns + j);
                const double v[8] = {p.teta, p.moist, psi, p.k, h, p.dqdh_inv, p.mdiff, 0.0};
                for (int s = 0; s < 8; s++)
                    buf[s * n + c] = v[s];
            }
    struct CALSubstate3Dr* q[8] = {MQ.teta, MQ.moist_cont, MQ.psi, MQ.k, MQ.h, MQ.dqdh, MQ.moist_diff, MQ.convergence};
    for (int s = 0; s < 8; s++)
        calCopySubstateFromHost3Dr(ca, q[s], buf + s * n); /* pageable: copied before the call returns */
    free(buf);
}

/* Run mbusu: steps 0 = until the stop condition (10 days), > 0 = at most
 * that many steps, < 0 = none (the initial state).  mode: 0 = one launch
 * sequence per step with the host stop condition, 1 = the step recorded as
 * a CUDA graph and replayed, 2 = one device-driven loop ended by the device
 * stop condition.  state: 8 x 624000 doubles (teta, moist_cont, psi, k, h,
 * dqdh, convergence, moist_diff) or NULL; tail: step reached, delta_t,
 * delta_t_cum; ms: device time of the steps. */
extern "C" int cal_mbusu_run(int steps, int mode, double* state, double* tail, double* ms)
{
    calClearError();
    struct CALModel3D* ca = calCADef3D(MB_ROWS, MB_COLS, MB_SLICES, CAL_VON_NEUMANN_NEIGHBORHOOD_3D,
                                       CAL_SPACE_TOROIDAL, CAL_NO_OPT);
    if (!ca)
        return calGetLastError();
    struct CALRun3D* run = calRunDef3D(ca, 1, steps > 0 ? steps : CAL_RUN_LOOP, CAL_UPDATE_IMPLICIT);
    calAddElementaryProcess3D(ca, mbusu_transition);
    MQ.teta = calAddSubstate3Dr(ca);
    MQ.moist_cont = calAddSubstate3Dr(ca);
    MQ.psi = calAddSubstate3Dr(ca);
    MQ.k = calAddSubstate3Dr(ca);
    MQ.h = calAddSubstate3Dr(ca);
    MQ.dqdh = calAddSubstate3Dr(ca);
    MQ.convergence = calAddSubstate3Dr(ca);
    MQ.moist_diff = calAddSubstate3Dr(ca);
    mbusu_init_host(ca);
    cudaStream_t st = (cudaStream_t)calGetStream3D(ca);
    mbusu_reset_kernel<<<1, 1, 0, st>>>();
    calRunAddSteeringFunc3D(run, mbusu_steering);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    int done = 0;
    if (steps >= 0) {
        if (mode == 2) {
            calRunAddDeviceStopConditionFunc3D(run, mbusu_stop_device);
            calRunDevice3D(run);
            done = run->step; /* the step the stop condition fired at, or final + 1 */
            if (steps > 0 && done > steps)
                done = steps;
        } else {
            calRunAddStopConditionFunc3D(run, mbusu_stop_host);
            calRunSetGraph3D(run, mode == 1 ? CAL_TRUE : CAL_FALSE);
            calRunInitSimulation3D(run);
            for (;;) {
                run->step++;
                done++;
                if (!calRunCAStep3D(run) || (steps > 0 && done >= steps))
                    break;
            }
        }
    }
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms)
        *ms = t;
    calSync3D(ca);
    int rc = calGetLastError();
    if (state) {
        const size_t n = (size_t)MB_ROWS * MB_COLS * MB_SLICES;
        struct CALSubstate3Dr* q[8] = {MQ.teta, MQ.moist_cont, MQ.psi, MQ.k, MQ.h, MQ.dqdh, MQ.convergence,
                                       MQ.moist_diff};
        for (int s = 0; s < 8; s++)
            memcpy(state + s * n, q[s]->current, n * sizeof(double));
    }
    if (tail) {
        float dt = 0.f, cum = 0.f;
        cudaMemcpyFromSymbol(&dt, mb_delta_t, sizeof(float));
        cudaMemcpyFromSymbol(&cum, mb_cum, sizeof(float));
        tail[0] = done;
        tail[1] = dt;
        tail[2] = cum;
    }
    if (!rc && cudaGetLastError() != cudaSuccess)
        rc = CAL_ERROR_CUDA;
    calRunFinalize3D(run);
    calFinalize3D(ca);
    return rc;
}
