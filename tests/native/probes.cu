/*
 * probes.cu -- TEST INFRASTRUCTURE: small rules that exercise the engine's
 * semantics through the public C API, built into a test-only library
 * (tests/native/build/libopencal_probes.so, linked against
 * libopencal_gb300.so) and never shipped with the product.  Each entry
 * point has the same contract as the oracle's function of the same suffix
 * (oracle/oracle_models.c), so the parity tests compare them directly.
 *
 *   nbprobe2d  v' = v/4 + sum_n v_n * n/64 on any 2D neighbourhood (exercises
 *              the neighbour tables, including the hexagonal odd-column /
 *              odd-row shift of OpenCAL-OMP/source/cal2D.c:859-870, and
 *              custom neighbourhoods built with calAddNeighbor2D,
 *              OpenCAL-OMP/source/cal2D.c:444-466)
 *   acprobe    three processes with SCIDDICA-T's active-cell structure,
 *              2D or 3D (add on outflow, update, remove, steering on next)
 *   unsafe2d   every unsafe operation (cal2DUnsafe.h): integer spreads with
 *              calAddNext / calAddNextX, and single-writer neighbour stores
 *              with calSetX / calGetNextX / calSetCurrentX / calInitX
 *   reduce2d   the device reductions of cal2DReduction.h on a given array
 *   exact_div  device check of models/exact_div.cuh against IEEE division
 */
#include <string.h>

#include "opencal/cal2D.h"
#include "opencal/cal2DRun.h"
#include "opencal/cal2DUnsafe.h"
#include "opencal/cal3D.h"
#include "opencal/cal3DRun.h"

static int finish2d(struct CALModel2D* ca, struct CALRun2D* run)
{
    int err = calGetLastError();
    calRunFinalize2D(run);
    calFinalize2D(ca);
    return err;
}

static int finish3d(struct CALModel3D* ca, struct CALRun3D* run)
{
    int err = calGetLastError();
    calRunFinalize3D(run);
    calFinalize3D(ca);
    return err;
}
/* ======================= neighbourhood probe ============================ */

__managed__ struct CALSubstate2Dr* nbQ;

CAL_ELEMENTARY_PROCESS_2D(nbprobe_rule)(struct CALModel2D* ca, int i, int j)
{
    double acc = calGet2Dr(ca, nbQ, i, j) * 0.25;
    for (int n = 1; n < ca->sizeof_X; n++)
        acc += calGetX2Dr(ca, nbQ, i, j, n) * ((double)n * 0.015625);
    calSet2Dr(ca, nbQ, i, j, acc);
}

extern "C" int cal_nbprobe2d_run(int rows, int cols, int nbhd, int toroidal, int steps, const double* v0,
                                 double* v_out, int graph)
{
    calClearError();
    struct CALModel2D* ca = calCADef2D(rows, cols, (enum CALNeighborhood2D)nbhd,
                                       toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    if (!ca)
        return calGetLastError();
    struct CALRun2D* run = calRunDef2D(ca, 1, steps, CAL_UPDATE_IMPLICIT);
    calAddElementaryProcess2D(ca, nbprobe_rule);
    nbQ = calAddSubstate2Dr(ca);
    const size_t bytes = sizeof(double) * (size_t)rows * cols;
    memcpy(nbQ->current, v0, bytes);
    memcpy(nbQ->next, v0, bytes);
    calMarkHostDirty2D(ca);
    calRunSetGraph2D(run, graph ? CAL_TRUE : CAL_FALSE);
    if (steps > 0)
        calRun2D(run);
    calSync2D(ca);
    memcpy(v_out, nbQ->current, bytes);
    return finish2d(ca, run);
}

/* the same rule on a custom neighbourhood: CAL_CUSTOM_NEIGHBORHOOD_2D, then
 * the offsets (di, dj) appended with calAddNeighbor2D */
extern "C" int cal_nbprobe2d_custom_run(int rows, int cols, int toroidal, int steps, int nx, const int* offs,
                                        const double* v0, double* v_out, int graph)
{
    calClearError();
    struct CALModel2D* ca = calCADef2D(rows, cols, CAL_CUSTOM_NEIGHBORHOOD_2D,
                                       toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    if (!ca)
        return calGetLastError();
    for (int n = 0; n < nx; n++)
        calAddNeighbor2D(ca, offs[2 * n], offs[2 * n + 1]);
    struct CALRun2D* run = calRunDef2D(ca, 1, steps, CAL_UPDATE_IMPLICIT);
    calAddElementaryProcess2D(ca, nbprobe_rule);
    nbQ = calAddSubstate2Dr(ca);
    const size_t bytes = sizeof(double) * (size_t)rows * cols;
    memcpy(nbQ->current, v0, bytes);
    memcpy(nbQ->next, v0, bytes);
    calMarkHostDirty2D(ca);
    calRunSetGraph2D(run, graph ? CAL_TRUE : CAL_FALSE);
    if (steps > 0)
        calRun2D(run);
    calSync2D(ca);
    memcpy(v_out, nbQ->current, bytes);
    return finish2d(ca, run);
}

/* ======================= active-cell probe ============================== */

struct acp2_t {
    struct CALSubstate2Dr *v, *w;
};
struct acp3_t {
    struct CALSubstate3Dr *v, *w;
};
__managed__ struct acp2_t A2;
__managed__ struct acp3_t A3;
__managed__ double acp_thr;

CAL_ELEMENTARY_PROCESS_2D(acp2_ep1)(struct CALModel2D* ca, int i, int j)
{
    double c = calGet2Dr(ca, A2.v, i, j);
    if (c <= acp_thr)
        return;
    for (int n = 1; n < ca->sizeof_X; n++)
        if (calGetX2Dr(ca, A2.v, i, j, n) < c)
            calAddActiveCellX2D(ca, i, j, n);
    calSet2Dr(ca, A2.w, i, j, c * 0.125);
}

CAL_ELEMENTARY_PROCESS_2D(acp2_ep2)(struct CALModel2D* ca, int i, int j)
{
    double acc = calGet2Dr(ca, A2.v, i, j);
    for (int n = 1; n < ca->sizeof_X; n++)
        acc += calGetX2Dr(ca, A2.w, i, j, n) - calGet2Dr(ca, A2.w, i, j);
    calSet2Dr(ca, A2.v, i, j, acc);
}

CAL_ELEMENTARY_PROCESS_2D(acp2_ep3)(struct CALModel2D* ca, int i, int j)
{
    if (calGet2Dr(ca, A2.v, i, j) <= acp_thr)
        calRemoveActiveCell2D(ca, i, j);
}

static void acp2_init(struct CALModel2D* ca)
{
    calInitSubstate2Dr(ca, A2.w, 0);
    for (int i = 0; i < ca->rows; i++)
        for (int j = 0; j < ca->columns; j++)
            if (calGet2Dr(ca, A2.v, i, j) > acp_thr)
                calAddActiveCell2D(ca, i, j);
}

static void acp2_steer(struct CALModel2D* ca) { calInitSubstateNext2Dr(ca, A2.w, 0); }

CAL_ELEMENTARY_PROCESS_3D(acp3_ep1)(struct CALModel3D* ca, int i, int j, int k)
{
    double c = calGet3Dr(ca, A3.v, i, j, k);
    if (c <= acp_thr)
        return;
    for (int n = 1; n < ca->sizeof_X; n++)
        if (calGetX3Dr(ca, A3.v, i, j, k, n) < c)
            calAddActiveCellX3D(ca, i, j, k, n);
    calSet3Dr(ca, A3.w, i, j, k, c * 0.125);
}

CAL_ELEMENTARY_PROCESS_3D(acp3_ep2)(struct CALModel3D* ca, int i, int j, int k)
{
    double acc = calGet3Dr(ca, A3.v, i, j, k);
    for (int n = 1; n < ca->sizeof_X; n++)
        acc += calGetX3Dr(ca, A3.w, i, j, k, n) - calGet3Dr(ca, A3.w, i, j, k);
    calSet3Dr(ca, A3.v, i, j, k, acc);
}

CAL_ELEMENTARY_PROCESS_3D(acp3_ep3)(struct CALModel3D* ca, int i, int j, int k)
{
    if (calGet3Dr(ca, A3.v, i, j, k) <= acp_thr)
        calRemoveActiveCell3D(ca, i, j, k);
}

static void acp3_init(struct CALModel3D* ca)
{
    calInitSubstate3Dr(ca, A3.w, 0);
    for (int i = 0; i < ca->rows; i++)
        for (int j = 0; j < ca->columns; j++)
            for (int k = 0; k < ca->slices; k++)
                if (calGet3Dr(ca, A3.v, i, j, k) > acp_thr)
                    calAddActiveCell3D(ca, i, j, k);
}

static void acp3_steer(struct CALModel3D* ca) { calInitSubstateNext3Dr(ca, A3.w, 0); }

extern "C" int cal_acprobe_run(int dim, int rows, int cols, int slices, int nbhd, int toroidal, int steps,
                               double thr, const double* v0, double* v_out, long* n_active, int* cells_out, int graph)
{
    calClearError();
    acp_thr = thr;
    if (dim == 2) {
        struct CALModel2D* ca = calCADef2D(rows, cols, (enum CALNeighborhood2D)nbhd,
                                           toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_OPT_ACTIVE_CELLS);
        if (!ca)
            return calGetLastError();
        struct CALRun2D* run = calRunDef2D(ca, 1, steps, CAL_UPDATE_IMPLICIT);
        calAddElementaryProcess2D(ca, acp2_ep1);
        calAddElementaryProcess2D(ca, acp2_ep2);
        calAddElementaryProcess2D(ca, acp2_ep3);
        A2.v = calAddSubstate2Dr(ca);
        A2.w = calAddSubstate2Dr(ca);
        const size_t bytes = sizeof(double) * (size_t)rows * cols;
        memcpy(A2.v->current, v0, bytes);
        memcpy(A2.v->next, v0, bytes);
        calMarkHostDirty2D(ca);
        calRunAddInitFunc2D(run, acp2_init);
        calRunAddSteeringFunc2D(run, acp2_steer);
        calRunSetGraph2D(run, graph ? CAL_TRUE : CAL_FALSE);
        if (steps > 0)
            calRun2D(run);
        else
            calRunInitSimulation2D(run);
        calSync2D(ca);
        memcpy(v_out, A2.v->current, bytes);
        if (n_active)
            *n_active = ca->A.size_current;
        if (cells_out && ca->A.size_current > 0)
            memcpy(cells_out, ca->A.cells, sizeof(int) * 2 * (size_t)ca->A.size_current);
        return finish2d(ca, run);
    }
    struct CALModel3D* ca = calCADef3D(rows, cols, slices, (enum CALNeighborhood3D)nbhd,
                                       toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_OPT_ACTIVE_CELLS);
    if (!ca)
        return calGetLastError();
    struct CALRun3D* run = calRunDef3D(ca, 1, steps, CAL_UPDATE_IMPLICIT);
    calAddElementaryProcess3D(ca, acp3_ep1);
    calAddElementaryProcess3D(ca, acp3_ep2);
    calAddElementaryProcess3D(ca, acp3_ep3);
    A3.v = calAddSubstate3Dr(ca);
    A3.w = calAddSubstate3Dr(ca);
    const size_t bytes = sizeof(double) * (size_t)rows * cols * slices;
    memcpy(A3.v->current, v0, bytes);
    memcpy(A3.v->next, v0, bytes);
    calMarkHostDirty3D(ca);
    calRunAddInitFunc3D(run, acp3_init);
    calRunAddSteeringFunc3D(run, acp3_steer);
    calRunSetGraph3D(run, graph ? CAL_TRUE : CAL_FALSE);
    if (steps > 0)
        calRun3D(run);
    else
        calRunInitSimulation3D(run);
    calSync3D(ca);
    memcpy(v_out, A3.v->current, bytes);
    if (n_active)
        *n_active = ca->A.size_current;
    if (cells_out && ca->A.size_current > 0)
        memcpy(cells_out, ca->A.cells, sizeof(int) * 3 * (size_t)ca->A.size_current);
    return finish3d(ca, run);
}

/* ======================= exact small-integer division check ============= */
#include "exact_div.cuh"

__global__ void exact_div_kernel(const double* x, const int* c, const double* y, double b, double rb, double* q_exact,
                                 double* q_ieee, double* r_exact, double* r_ieee, int* le_exact, int* le_ieee,
                                 long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        q_exact[t] = cal_div_small(x[t], c[t]);
        q_ieee[t] = x[t] / (double)c[t];
        r_exact[t] = cal_div_recip(x[t], b, rb);
        r_ieee[t] = x[t] / b;
        le_exact[t] = (int)cal_le(x[t], y[t]) | (int)cal_gt(x[t], y[t]) << 1 | (int)cal_pos(x[t]) << 2;
        le_ieee[t] = (int)(x[t] <= y[t]) | (int)(x[t] > y[t]) << 1 | (int)(x[t] > 0) << 2;
    }
}

static bool same_bits(double a, double b)
{
    return memcmp(&a, &b, sizeof(double)) == 0 || (a != a && b != b);
}

/* Device-side check of exact_div.cuh against the device's own IEEE
 * division and comparisons: x / c (c in 1..9), x / b by the reciprocal
 * method (b = sqrt(2), the SCIARA-fv2 diagonal divisor), <=, > and > 0;
 * returns the number of mismatches (-1: CUDA error, -2: the reciprocal
 * method's precondition does not hold for b). */
extern "C" long cal_test_exact_div(const double* x_host, const int* c_host, const double* y_host, long long n)
{
    const double b = sqrt(2.0), rb = 1.0 / b;
    if (!cal_recip_exact_ok(b, rb))
        return -2;
    double *x, *y, *buf;
    int *c, *le, *li;
    cudaMalloc(&x, n * sizeof(double));
    cudaMalloc(&y, n * sizeof(double));
    cudaMalloc(&buf, 4 * n * sizeof(double));
    cudaMalloc(&c, n * sizeof(int));
    cudaMalloc(&le, n * sizeof(int));
    cudaMalloc(&li, n * sizeof(int));
    cudaMemcpy(x, x_host, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(y, y_host, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(c, c_host, n * sizeof(int), cudaMemcpyHostToDevice);
    exact_div_kernel<<<1024, 256>>>(x, c, y, b, rb, buf, buf + n, buf + 2 * n, buf + 3 * n, le, li, n);
    double* hq = (double*)malloc(4 * n * sizeof(double));
    int* hle = (int*)malloc(n * sizeof(int));
    int* hli = (int*)malloc(n * sizeof(int));
    cudaMemcpy(hq, buf, 4 * n * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(hle, le, n * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(hli, li, n * sizeof(int), cudaMemcpyDeviceToHost);
    long bad = cudaGetLastError() == cudaSuccess ? 0 : -1;
    for (long long t = 0; bad >= 0 && t < n; t++)
        if (!same_bits(hq[t], hq[n + t]) || !same_bits(hq[2 * n + t], hq[3 * n + t]) || hle[t] != hli[t])
            bad++;
    free(hq);
    free(hle);
    free(hli);
    cudaFree(x);
    cudaFree(y);
    cudaFree(buf);
    cudaFree(c);
    cudaFree(le);
    cudaFree(li);
    return bad;
}

/* ======================= reductions ===================================== */
#include "opencal/cal2DReduction.h"

/* Reduce `data` (rows x cols of type 0 byte / 1 int / 2 real) with `op`
 * through the C API; *out receives the result as a double. */
extern "C" int cal_reduce2d_run(int type, int rows, int cols, const void* data, int op, double* out)
{
    calClearError();
    struct CALModel2D* ca = calCADef2D(rows, cols, CAL_MOORE_NEIGHBORHOOD_2D, CAL_SPACE_TOROIDAL, CAL_NO_OPT);
    if (!ca)
        return calGetLastError();
    const long long n = (long long)rows * cols;
    if (type == 0) {
        struct CALSubstate2Db* q = calAddSubstate2Db(ca);
        memcpy(q->current, data, n);
        calMarkHostDirty2D(ca);
        *out = (double)calReductionOperation2Db(ca, q, (enum REDUCTION_OPERATION)op);
    } else if (type == 1) {
        struct CALSubstate2Di* q = calAddSubstate2Di(ca);
        memcpy(q->current, data, n * sizeof(int));
        calMarkHostDirty2D(ca);
        *out = (double)calReductionOperation2Di(ca, q, (enum REDUCTION_OPERATION)op);
    } else {
        struct CALSubstate2Dr* q = calAddSubstate2Dr(ca);
        memcpy(q->current, data, n * sizeof(double));
        calMarkHostDirty2D(ca);
        *out = calReductionOperation2Dr(ca, q, (enum REDUCTION_OPERATION)op);
    }
    int err = calGetLastError();
    calFinalize2D(ca);
    return err;
}

/* ======================= unsafe-operation probe ========================= */

struct UnsafeQ {
    struct CALSubstate2Di* v;
    struct CALSubstate2Db* b;
    struct CALSubstate2Dr* w;
    struct CALSubstate2Dr* u;
    struct CALSubstate2Dr* x;
};
__managed__ struct UnsafeQ UQ;

CAL_ELEMENTARY_PROCESS_2D(unsafe_ep1)(struct CALModel2D* ca, int i, int j)
{
    if (calGet2Di(ca, UQ.v, i, j) > 0) {
        for (int n = 1; n < ca->sizeof_X; n++)
            calAddNextX2Di(ca, UQ.v, i, j, n, 1);
        calAddNext2Di(ca, UQ.v, i, j, -(ca->sizeof_X - 1));
    }
    if (calGet2Db(ca, UQ.b, i, j) > 0) {
        calAddNextX2Db(ca, UQ.b, i, j, 1 + (i + j) % (ca->sizeof_X - 1), 1);
        calAddNext2Db(ca, UQ.b, i, j, -1);
    }
}

CAL_ELEMENTARY_PROCESS_2D(unsafe_ep2)(struct CALModel2D* ca, int i, int j)
{
    const double w = calGet2Dr(ca, UQ.w, i, j);
    calSetX2Dr(ca, UQ.w, i, j, 1, w * 0.5 + calGetNextX2Dr(ca, UQ.w, i, j, 1) * 0.25);
    calSetCurrentX2Dr(ca, UQ.u, i, j, 2, w);
    calInitX2Dr(ca, UQ.x, i, j, 3, w + 1.0);
}

extern "C" int cal_unsafe2d_run(int rows, int cols, int nbhd, int toroidal, int steps, const int* v0,
                                const signed char* b0, const double* w0, int* v_out, signed char* b_out,
                                double* w_out, double* u_out, double* x_out, int graph)
{
    calClearError();
    struct CALModel2D* ca = calCADef2D(rows, cols, (enum CALNeighborhood2D)nbhd,
                                       toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    if (!ca)
        return calGetLastError();
    calSetUnsafe2D(ca);
    struct CALRun2D* run = calRunDef2D(ca, 1, steps, CAL_UPDATE_IMPLICIT);
    calAddElementaryProcess2D(ca, unsafe_ep1);
    if (nbhd == CAL_VON_NEUMANN_NEIGHBORHOOD_2D || nbhd == CAL_MOORE_NEIGHBORHOOD_2D)
        calAddElementaryProcess2D(ca, unsafe_ep2);
    UQ.v = calAddSubstate2Di(ca);
    UQ.b = calAddSubstate2Db(ca);
    UQ.w = calAddSubstate2Dr(ca);
    UQ.u = calAddSingleLayerSubstate2Dr(ca);
    UQ.x = calAddSubstate2Dr(ca);
    const size_t n = (size_t)rows * cols;
    memcpy(UQ.v->current, v0, n * sizeof(int));
    memcpy(UQ.v->next, v0, n * sizeof(int));
    memcpy(UQ.b->current, b0, n);
    memcpy(UQ.b->next, b0, n);
    memcpy(UQ.w->current, w0, n * sizeof(double));
    memcpy(UQ.w->next, w0, n * sizeof(double));
    memset(UQ.u->current, 0, n * sizeof(double));
    memset(UQ.x->current, 0, n * sizeof(double));
    memset(UQ.x->next, 0, n * sizeof(double));
    calMarkHostDirty2D(ca);
    calRunSetGraph2D(run, graph ? CAL_TRUE : CAL_FALSE);
    if (steps > 0)
        calRun2D(run);
    calSync2D(ca);
    memcpy(v_out, UQ.v->current, n * sizeof(int));
    memcpy(b_out, UQ.b->current, n);
    memcpy(w_out, UQ.w->current, n * sizeof(double));
    memcpy(u_out, UQ.u->current, n * sizeof(double));
    memcpy(x_out, UQ.x->current, n * sizeof(double));
    return finish2d(ca, run);
}

/* ======================= substate text files ============================ */
#include "opencal/cal2DIO.h"
#include "opencal/cal3DIO.h"

/* a model on the GPU loads a substate (kind: 0 byte, 1 int, 2 real) from
 * in_path with calLoadSubstate2D / 3D (b, i, r), pushes it through an update
 * on the device, saves it with calSaveSubstate2D / 3D to out_path and copies
 * the current layer into data_out */
extern "C" int cal_io_roundtrip(int dim, int kind, int rows, int cols, int slices, const char* in_path,
                                const char* out_path, void* data_out)
{
    calClearError();
    const size_t n = (size_t)rows * cols * (dim == 3 ? slices : 1);
    int ok = 1;
    if (dim == 2) {
        struct CALModel2D* ca = calCADef2D(rows, cols, CAL_MOORE_NEIGHBORHOOD_2D, CAL_SPACE_TOROIDAL, CAL_NO_OPT);
        if (!ca)
            return calGetLastError();
        if (kind == 0) {
            struct CALSubstate2Db* q = calAddSubstate2Db(ca);
            ok = calLoadSubstate2Db(ca, q, (char*)in_path);
            calUpdate2D(ca);
            ok = ok && calSaveSubstate2Db(ca, q, (char*)out_path);
            calSync2D(ca);
            memcpy(data_out, q->current, n);
        } else if (kind == 1) {
            struct CALSubstate2Di* q = calAddSubstate2Di(ca);
            ok = calLoadSubstate2Di(ca, q, (char*)in_path);
            calUpdate2D(ca);
            ok = ok && calSaveSubstate2Di(ca, q, (char*)out_path);
            calSync2D(ca);
            memcpy(data_out, q->current, n * sizeof(int));
        } else {
            struct CALSubstate2Dr* q = calAddSubstate2Dr(ca);
            ok = calLoadSubstate2Dr(ca, q, (char*)in_path);
            calUpdate2D(ca);
            ok = ok && calSaveSubstate2Dr(ca, q, (char*)out_path);
            calSync2D(ca);
            memcpy(data_out, q->current, n * sizeof(double));
        }
        const int err = calGetLastError();
        calFinalize2D(ca);
        return err ? err : (ok ? 0 : CAL_ERROR_IO);
    }
    struct CALModel3D* ca = calCADef3D(rows, cols, slices, CAL_MOORE_NEIGHBORHOOD_3D, CAL_SPACE_TOROIDAL, CAL_NO_OPT);
    if (!ca)
        return calGetLastError();
    if (kind == 0) {
        struct CALSubstate3Db* q = calAddSubstate3Db(ca);
        ok = calLoadSubstate3Db(ca, q, (char*)in_path);
        calUpdate3D(ca);
        ok = ok && calSaveSubstate3Db(ca, q, (char*)out_path);
        calSync3D(ca);
        memcpy(data_out, q->current, n);
    } else if (kind == 1) {
        struct CALSubstate3Di* q = calAddSubstate3Di(ca);
        ok = calLoadSubstate3Di(ca, q, (char*)in_path);
        calUpdate3D(ca);
        ok = ok && calSaveSubstate3Di(ca, q, (char*)out_path);
        calSync3D(ca);
        memcpy(data_out, q->current, n * sizeof(int));
    } else {
        struct CALSubstate3Dr* q = calAddSubstate3Dr(ca);
        ok = calLoadSubstate3Dr(ca, q, (char*)in_path);
        calUpdate3D(ca);
        ok = ok && calSaveSubstate3Dr(ca, q, (char*)out_path);
        calSync3D(ca);
        memcpy(data_out, q->current, n * sizeof(double));
    }
    const int err = calGetLastError();
    calFinalize3D(ca);
    return err ? err : (ok ? 0 : CAL_ERROR_IO);
}
