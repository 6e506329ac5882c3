/*
 * ref_drivers.c -- headless drivers that run the parity rules on the REAL
 * reference library (OpenCAL-OMP sources compiled serially by
 * oracle/ref/Makefile).  They expose the same entry points as
 * oracle/oracle_models.c with a ref_ prefix, so tests can check the oracle
 * restatement against the reference itself on identical inputs.
 * Test infrastructure only; built only where the reference sources exist.
 *
 * The rules are the same restatements as in oracle_models.c, written against
 * the reference's C API (cal2D.h / cal2DRun.h / cal3D.h / cal3DRun.h).
 */
#include <cal2D.h>
#include <cal2DBuffer.h>
#include <cal2DRun.h>
#include <cal2DUnsafe.h>
#include <cal3D.h>
#include <cal3DBuffer.h>
#include <cal3DRun.h>
#include <stdlib.h>
#include <string.h>

/* flags come from the guard allocator; release them through it before
 * calFinalize2D/3D, which would otherwise free() an interior pointer */
static void finalize2d(struct CALModel2D* m)
{
    if (m->A.flags) {
        calDeleteBuffer2Db(m->A.flags);
        m->A.flags = NULL;
    }
    calFinalize2D(m);
}

static void finalize3d(struct CALModel3D* m)
{
    if (m->A.flags) {
        calDeleteBuffer3Db(m->A.flags);
        m->A.flags = NULL;
    }
    calFinalize3D(m);
}

static void export2d(struct CALModel2D* m, long* n_active, int* cells)
{
    int n;
    if (n_active)
        *n_active = m->A.cells ? m->A.size_current : 0;
    if (cells && m->A.cells)
        for (n = 0; n < m->A.size_current; n++) {
            cells[2 * n] = m->A.cells[n].i;
            cells[2 * n + 1] = m->A.cells[n].j;
        }
}

/* ======================= SCIDDICA-T ================================== */

static struct {
    struct CALSubstate2Dr *z, *h, *f[4];
    double r, eps;
    int ac;
} S;

static void s_flows(struct CALModel2D* m, int i, int j)
{
    CALbyte out[5] = {0, 0, 0, 0, 0};
    double u[5], mass, avg;
    int n, again, count;
    if (calGet2Dr(m, S.h, i, j) <= S.eps)
        return;
    mass = calGet2Dr(m, S.h, i, j) - S.eps;
    u[0] = calGet2Dr(m, S.z, i, j) + S.eps;
    for (n = 1; n < m->sizeof_X; n++) {
        double zn = calGetX2Dr(m, S.z, i, j, n);
        double hn = calGetX2Dr(m, S.h, i, j, n);
        u[n] = zn + hn;
    }
    do {
        again = 0;
        avg = mass;
        count = 0;
        for (n = 0; n < m->sizeof_X; n++)
            if (!out[n]) {
                avg += u[n];
                count++;
            }
        if (count != 0)
            avg /= count;
        for (n = 0; n < m->sizeof_X; n++)
            if (avg <= u[n] && !out[n]) {
                out[n] = 1;
                again = 1;
            }
    } while (again);
    for (n = 1; n < m->sizeof_X; n++) {
        if (out[n]) {
            calSet2Dr(m, S.f[n - 1], i, j, 0.0);
        } else {
            calSet2Dr(m, S.f[n - 1], i, j, (avg - u[n]) * S.r);
            if (S.ac)
                calAddActiveCellX2D(m, i, j, n);
        }
    }
}

static void s_width(struct CALModel2D* m, int i, int j)
{
    double hn = calGet2Dr(m, S.h, i, j);
    int n;
    for (n = 1; n < m->sizeof_X; n++)
        hn += calGetX2Dr(m, S.f[4 - n], i, j, n) - calGet2Dr(m, S.f[n - 1], i, j);
    calSet2Dr(m, S.h, i, j, hn);
}

static void s_remove(struct CALModel2D* m, int i, int j)
{
    if (calGet2Dr(m, S.h, i, j) <= S.eps)
        calRemoveActiveCell2D(m, i, j);
}

static void s_init(struct CALModel2D* m)
{
    int i, j, q;
    for (q = 0; q < 4; q++)
        calInitSubstate2Dr(m, S.f[q], 0);
    for (i = 0; i < m->rows; i++)
        for (j = 0; j < m->columns; j++) {
            double hc = calGet2Dr(m, S.h, i, j);
            if (hc > 0.0) {
                double zc = calGet2Dr(m, S.z, i, j);
                calSet2Dr(m, S.z, i, j, zc - hc);
                if (S.ac)
                    calAddActiveCell2D(m, i, j);
            }
        }
}

static void s_steer_plain(struct CALModel2D* m)
{
    int q;
    for (q = 0; q < 4; q++)
        calInitSubstate2Dr(m, S.f[q], 0);
}

static void s_steer_ac(struct CALModel2D* m)
{
    int q;
    for (q = 0; q < 4; q++)
        calInitSubstateNext2Dr(m, S.f[q], 0);
}

int ref_sciddicaT(int rows, int cols, int toroidal, int ac, int steps, double p_r, double p_eps,
                  const double* z0, const double* h0, double* z_out, double* h_out,
                  long* n_active, int* cells_out)
{
    struct CALModel2D* m = calCADef2D(rows, cols, CAL_VON_NEUMANN_NEIGHBORHOOD_2D,
                                      toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT,
                                      ac ? CAL_OPT_ACTIVE_CELLS : CAL_NO_OPT);
    struct CALRun2D* run = calRunDef2D(m, 1, steps, CAL_UPDATE_IMPLICIT);
    size_t bytes = sizeof(double) * (size_t)rows * cols;
    int q;
    S.ac = ac;
    S.r = p_r;
    S.eps = p_eps;
    calAddElementaryProcess2D(m, s_flows);
    calAddElementaryProcess2D(m, s_width);
    if (ac)
        calAddElementaryProcess2D(m, s_remove);
    S.z = calAddSubstate2Dr(m);
    S.h = calAddSubstate2Dr(m);
    for (q = 0; q < 4; q++)
        S.f[q] = calAddSubstate2Dr(m);
    memcpy(S.z->current, z0, bytes);
    memcpy(S.z->next, z0, bytes);
    memcpy(S.h->current, h0, bytes);
    memcpy(S.h->next, h0, bytes);
    calRunAddInitFunc2D(run, s_init);
    calRunAddSteeringFunc2D(run, ac ? s_steer_ac : s_steer_plain);
    if (steps > 0)
        calRun2D(run);
    else
        calRunInitSimulation2D(run);
    if (z_out)
        memcpy(z_out, S.z->current, bytes);
    if (h_out)
        memcpy(h_out, S.h->current, bytes);
    export2d(m, n_active, cells_out);
    calRunFinalize2D(run);
    finalize2d(m);
    return 0;
}

/* ======================= Life 2D ====================================== */

static struct CALSubstate2Db* LB;
static struct CALSubstate2Di* LI;

static void life_b(struct CALModel2D* m, int i, int j)
{
    int n, sum = 0;
    for (n = 1; n < m->sizeof_X; n++)
        sum += calGetX2Db(m, LB, i, j, n);
    if (sum == 3 || (sum == 2 && calGet2Db(m, LB, i, j) == 1))
        calSet2Db(m, LB, i, j, 1);
    else
        calSet2Db(m, LB, i, j, 0);
}

static void life_i(struct CALModel2D* m, int i, int j)
{
    int n, sum = 0;
    for (n = 1; n < m->sizeof_X; n++)
        sum += calGetX2Di(m, LI, i, j, n);
    if (sum == 3 || (sum == 2 && calGet2Di(m, LI, i, j) == 1))
        calSet2Di(m, LI, i, j, 1);
    else
        calSet2Di(m, LI, i, j, 0);
}

int ref_life2d(int rows, int cols, int toroidal, int as_int, int steps,
               const unsigned char* s0, unsigned char* s_out)
{
    struct CALModel2D* m = calCADef2D(rows, cols, CAL_MOORE_NEIGHBORHOOD_2D,
                                      toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    struct CALRun2D* run = calRunDef2D(m, 1, steps, CAL_UPDATE_IMPLICIT);
    long c, total = (long)rows * cols;
    if (as_int) {
        LI = calAddSubstate2Di(m);
        calAddElementaryProcess2D(m, life_i);
        for (c = 0; c < total; c++)
            LI->current[c] = LI->next[c] = s0[c];
    } else {
        LB = calAddSubstate2Db(m);
        calAddElementaryProcess2D(m, life_b);
        for (c = 0; c < total; c++)
            LB->current[c] = LB->next[c] = (CALbyte)s0[c];
    }
    if (steps > 0)
        calRun2D(run);
    for (c = 0; c < total; c++)
        s_out[c] = as_int ? (unsigned char)LI->current[c] : (unsigned char)LB->current[c];
    calRunFinalize2D(run);
    finalize2d(m);
    return 0;
}

/* ======================= neighbourhood probe ========================== */

static struct CALSubstate2Dr* HQ;

static void hex_rule(struct CALModel2D* m, int i, int j)
{
    double acc = calGet2Dr(m, HQ, i, j) * 0.25;
    int n;
    for (n = 1; n < m->sizeof_X; n++)
        acc += calGetX2Dr(m, HQ, i, j, n) * ((double)n * 0.015625);
    calSet2Dr(m, HQ, i, j, acc);
}

int ref_nbprobe2d(int rows, int cols, int nbhd, int toroidal, int steps, const double* v0, double* v_out)
{
    struct CALModel2D* m = calCADef2D(rows, cols, (enum CALNeighborhood2D)nbhd,
                                      toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    struct CALRun2D* run = calRunDef2D(m, 1, steps, CAL_UPDATE_IMPLICIT);
    size_t bytes = sizeof(double) * (size_t)rows * cols;
    calAddElementaryProcess2D(m, hex_rule);
    HQ = calAddSubstate2Dr(m);
    memcpy(HQ->current, v0, bytes);
    memcpy(HQ->next, v0, bytes);
    if (steps > 0)
        calRun2D(run);
    memcpy(v_out, HQ->current, bytes);
    calRunFinalize2D(run);
    finalize2d(m);
    return 0;
}

/* the rule on a custom neighbourhood built with calAddNeighbor2D */
int ref_nbprobe2d_custom(int rows, int cols, int toroidal, int steps, int nx, const int* offs, const double* v0,
                         double* v_out)
{
    struct CALModel2D* m = calCADef2D(rows, cols, CAL_CUSTOM_NEIGHBORHOOD_2D,
                                      toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    struct CALRun2D* run = calRunDef2D(m, 1, steps, CAL_UPDATE_IMPLICIT);
    size_t bytes = sizeof(double) * (size_t)rows * cols;
    int n;
    for (n = 0; n < nx; n++)
        calAddNeighbor2D(m, offs[2 * n], offs[2 * n + 1]);
    calAddElementaryProcess2D(m, hex_rule);
    HQ = calAddSubstate2Dr(m);
    memcpy(HQ->current, v0, bytes);
    memcpy(HQ->next, v0, bytes);
    if (steps > 0)
        calRun2D(run);
    memcpy(v_out, HQ->current, bytes);
    calRunFinalize2D(run);
    finalize2d(m);
    return 0;
}

/* ======================= active-cell spread probe ===================== */

static struct {
    struct CALSubstate2Dr *v, *w;
    struct CALSubstate3Dr *v3, *w3;
    double thr;
} A;

static void a_ep1(struct CALModel2D* m, int i, int j)
{
    double c = calGet2Dr(m, A.v, i, j);
    int n;
    if (c <= A.thr)
        return;
    for (n = 1; n < m->sizeof_X; n++)
        if (calGetX2Dr(m, A.v, i, j, n) < c)
            calAddActiveCellX2D(m, i, j, n);
    calSet2Dr(m, A.w, i, j, c * 0.125);
}

static void a_ep2(struct CALModel2D* m, int i, int j)
{
    double acc = calGet2Dr(m, A.v, i, j);
    int n;
    for (n = 1; n < m->sizeof_X; n++)
        acc += calGetX2Dr(m, A.w, i, j, n) - calGet2Dr(m, A.w, i, j);
    calSet2Dr(m, A.v, i, j, acc);
}

static void a_ep3(struct CALModel2D* m, int i, int j)
{
    if (calGet2Dr(m, A.v, i, j) <= A.thr)
        calRemoveActiveCell2D(m, i, j);
}

static void a_init(struct CALModel2D* m)
{
    int i, j;
    calInitSubstate2Dr(m, A.w, 0);
    for (i = 0; i < m->rows; i++)
        for (j = 0; j < m->columns; j++)
            if (calGet2Dr(m, A.v, i, j) > A.thr)
                calAddActiveCell2D(m, i, j);
}

static void a_steer(struct CALModel2D* m)
{
    calInitSubstateNext2Dr(m, A.w, 0);
}

static void a3_ep1(struct CALModel3D* m, int i, int j, int k)
{
    double c = calGet3Dr(m, A.v3, i, j, k);
    int n;
    if (c <= A.thr)
        return;
    for (n = 1; n < m->sizeof_X; n++)
        if (calGetX3Dr(m, A.v3, i, j, k, n) < c)
            calAddActiveCellX3D(m, i, j, k, n);
    calSet3Dr(m, A.w3, i, j, k, c * 0.125);
}

static void a3_ep2(struct CALModel3D* m, int i, int j, int k)
{
    double acc = calGet3Dr(m, A.v3, i, j, k);
    int n;
    for (n = 1; n < m->sizeof_X; n++)
        acc += calGetX3Dr(m, A.w3, i, j, k, n) - calGet3Dr(m, A.w3, i, j, k);
    calSet3Dr(m, A.v3, i, j, k, acc);
}

static void a3_ep3(struct CALModel3D* m, int i, int j, int k)
{
    if (calGet3Dr(m, A.v3, i, j, k) <= A.thr)
        calRemoveActiveCell3D(m, i, j, k);
}

static void a3_init(struct CALModel3D* m)
{
    int i, j, k;
    calInitSubstate3Dr(m, A.w3, 0);
    for (i = 0; i < m->rows; i++)
        for (j = 0; j < m->columns; j++)
            for (k = 0; k < m->slices; k++)
                if (calGet3Dr(m, A.v3, i, j, k) > A.thr)
                    calAddActiveCell3D(m, i, j, k);
}

static void a3_steer(struct CALModel3D* m)
{
    calInitSubstateNext3Dr(m, A.w3, 0);
}

int ref_acprobe(int dim, int rows, int cols, int slices, int nbhd, int toroidal, int steps,
                double thr, const double* v0, double* v_out, long* n_active, int* cells_out)
{
    A.thr = thr;
    if (dim == 2) {
        struct CALModel2D* m = calCADef2D(rows, cols, (enum CALNeighborhood2D)nbhd,
                                          toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT,
                                          CAL_OPT_ACTIVE_CELLS);
        struct CALRun2D* run = calRunDef2D(m, 1, steps, CAL_UPDATE_IMPLICIT);
        size_t bytes = sizeof(double) * (size_t)rows * cols;
        calAddElementaryProcess2D(m, a_ep1);
        calAddElementaryProcess2D(m, a_ep2);
        calAddElementaryProcess2D(m, a_ep3);
        A.v = calAddSubstate2Dr(m);
        A.w = calAddSubstate2Dr(m);
        memcpy(A.v->current, v0, bytes);
        memcpy(A.v->next, v0, bytes);
        calRunAddInitFunc2D(run, a_init);
        calRunAddSteeringFunc2D(run, a_steer);
        if (steps > 0)
            calRun2D(run);
        else
            calRunInitSimulation2D(run);
        memcpy(v_out, A.v->current, bytes);
        export2d(m, n_active, cells_out);
        calRunFinalize2D(run);
        finalize2d(m);
    } else {
        struct CALModel3D* m = calCADef3D(rows, cols, slices, (enum CALNeighborhood3D)nbhd,
                                          toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT,
                                          CAL_OPT_ACTIVE_CELLS);
        struct CALRun3D* run = calRunDef3D(m, 1, steps, CAL_UPDATE_IMPLICIT);
        size_t bytes = sizeof(double) * (size_t)rows * cols * slices;
        int n;
        calAddElementaryProcess3D(m, a3_ep1);
        calAddElementaryProcess3D(m, a3_ep2);
        calAddElementaryProcess3D(m, a3_ep3);
        A.v3 = calAddSubstate3Dr(m);
        A.w3 = calAddSubstate3Dr(m);
        memcpy(A.v3->current, v0, bytes);
        memcpy(A.v3->next, v0, bytes);
        calRunAddInitFunc3D(run, a3_init);
        calRunAddSteeringFunc3D(run, a3_steer);
        if (steps > 0)
            calRun3D(run);
        else
            calRunInitSimulation3D(run);
        memcpy(v_out, A.v3->current, bytes);
        if (n_active)
            *n_active = m->A.cells ? m->A.size_current : 0;
        if (cells_out && m->A.cells)
            for (n = 0; n < m->A.size_current; n++) {
                cells_out[3 * n] = m->A.cells[n].i;
                cells_out[3 * n + 1] = m->A.cells[n].j;
                cells_out[3 * n + 2] = m->A.cells[n].k;
            }
        calRunFinalize3D(run);
        finalize3d(m);
    }
    return 0;
}

/* ======================= Life 3D ====================================== */

static struct CALSubstate3Db* L3;
static int R1, R2, R3, R4;

static void life3d_rule(struct CALModel3D* m, int i, int j, int k)
{
    int n, sum = 0;
    CALbyte alive = calGet3Db(m, L3, i, j, k);
    CALbyte nxt = alive;
    for (n = 0; n < m->sizeof_X; n++)
        sum += calGetX3Db(m, L3, i, j, k, n);
    if (alive && (sum < R1 || sum > R2))
        nxt = 0;
    else if (!alive && (sum >= R3 && sum <= R4))
        nxt = 1;
    calSet3Db(m, L3, i, j, k, nxt);
}

int ref_life3d(int rows, int cols, int slices, int nbhd, int toroidal, int steps,
               int r1, int r2, int r3, int r4, const unsigned char* s0, unsigned char* s_out)
{
    struct CALModel3D* m = calCADef3D(rows, cols, slices, (enum CALNeighborhood3D)nbhd,
                                      toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    struct CALRun3D* run = calRunDef3D(m, 1, steps, CAL_UPDATE_IMPLICIT);
    long c, total = (long)rows * cols * slices;
    R1 = r1;
    R2 = r2;
    R3 = r3;
    R4 = r4;
    calAddElementaryProcess3D(m, life3d_rule);
    L3 = calAddSubstate3Db(m);
    for (c = 0; c < total; c++)
        L3->current[c] = L3->next[c] = (CALbyte)s0[c];
    if (steps > 0)
        calRun3D(run);
    for (c = 0; c < total; c++)
        s_out[c] = (unsigned char)L3->current[c];
    calRunFinalize3D(run);
    finalize3d(m);
    return 0;
}

/* ======================= unsafe-operation probe ======================= */

static struct {
    struct CALSubstate2Di* v;
    struct CALSubstate2Db* b;
    struct CALSubstate2Dr *w, *u, *x;
} UR;

static void ur_ep1(struct CALModel2D* m, int i, int j)
{
    int n;
    if (calGet2Di(m, UR.v, i, j) > 0) {
        for (n = 1; n < m->sizeof_X; n++)
            calAddNextX2Di(m, UR.v, i, j, n, 1);
        calAddNext2Di(m, UR.v, i, j, -(m->sizeof_X - 1));
    }
    if (calGet2Db(m, UR.b, i, j) > 0) {
        calAddNextX2Db(m, UR.b, i, j, 1 + (i + j) % (m->sizeof_X - 1), 1);
        calAddNext2Db(m, UR.b, i, j, -1);
    }
}

static void ur_ep2(struct CALModel2D* m, int i, int j)
{
    const double w = calGet2Dr(m, UR.w, i, j);
    calSetX2Dr(m, UR.w, i, j, 1, w * 0.5 + calGetNextX2Dr(m, UR.w, i, j, 1) * 0.25);
    calSetCurrentX2Dr(m, UR.u, i, j, 2, w);
    calInitX2Dr(m, UR.x, i, j, 3, w + 1.0);
}

int ref_unsafe2d(int rows, int cols, int nbhd, int toroidal, int steps, const int* v0, const signed char* b0,
                 const double* w0, int* v_out, signed char* b_out, double* w_out, double* u_out, double* x_out)
{
    struct CALModel2D* m = calCADef2D(rows, cols, (enum CALNeighborhood2D)nbhd,
                                      toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    struct CALRun2D* run = calRunDef2D(m, 1, steps, CAL_UPDATE_IMPLICIT);
    const size_t n = (size_t)rows * cols;
    calSetUnsafe2D(m);
    calAddElementaryProcess2D(m, ur_ep1);
    if (nbhd == CAL_VON_NEUMANN_NEIGHBORHOOD_2D || nbhd == CAL_MOORE_NEIGHBORHOOD_2D)
        calAddElementaryProcess2D(m, ur_ep2);
    UR.v = calAddSubstate2Di(m);
    UR.b = calAddSubstate2Db(m);
    UR.w = calAddSubstate2Dr(m);
    UR.u = calAddSingleLayerSubstate2Dr(m);
    UR.x = calAddSubstate2Dr(m);
    memcpy(UR.v->current, v0, n * sizeof(int));
    memcpy(UR.v->next, v0, n * sizeof(int));
    memcpy(UR.b->current, b0, n);
    memcpy(UR.b->next, b0, n);
    memcpy(UR.w->current, w0, n * sizeof(double));
    memcpy(UR.w->next, w0, n * sizeof(double));
    memset(UR.u->current, 0, n * sizeof(double));
    memset(UR.x->current, 0, n * sizeof(double));
    memset(UR.x->next, 0, n * sizeof(double));
    if (steps > 0)
        calRun2D(run);
    memcpy(v_out, UR.v->current, n * sizeof(int));
    memcpy(b_out, UR.b->current, n);
    memcpy(w_out, UR.w->current, n * sizeof(double));
    memcpy(u_out, UR.u->current, n * sizeof(double));
    memcpy(x_out, UR.x->current, n * sizeof(double));
    calRunFinalize2D(run);
    finalize2d(m);
    return 0;
}

/* ======================= SCIDDICA-T, unsafe form ====================== */
/* the transition of OpenCAL/examples/cal_sciddicaT-unsafe/source/sciddicaT.c,
 * written against the reference's API as there */

static struct {
    struct CALSubstate2Dr *z, *h;
    double r, eps;
} SUR;

static void sur_transition(struct CALModel2D* m, int i, int j)
{
    CALbyte out[5] = {CAL_FALSE, CAL_FALSE, CAL_FALSE, CAL_FALSE, CAL_FALSE};
    CALbyte again;
    CALint count, n;
    CALreal avg, mass, u[5], f;
    mass = calGet2Dr(m, SUR.h, i, j) - SUR.eps;
    u[0] = calGet2Dr(m, SUR.z, i, j) + SUR.eps;
    for (n = 1; n < m->sizeof_X; n++)
        u[n] = calGetX2Dr(m, SUR.z, i, j, n) + calGetX2Dr(m, SUR.h, i, j, n);
    do {
        again = CAL_FALSE;
        avg = mass;
        count = 0;
        for (n = 0; n < m->sizeof_X; n++)
            if (!out[n]) {
                avg += u[n];
                count++;
            }
        if (count != 0)
            avg /= count;
        for (n = 0; n < m->sizeof_X; n++)
            if ((avg <= u[n]) && (!out[n])) {
                out[n] = CAL_TRUE;
                again = CAL_TRUE;
            }
    } while (again);
    for (n = 1; n < m->sizeof_X; n++)
        if (!out[n]) {
            f = (avg - u[n]) * SUR.r;
            calSet2Dr(m, SUR.h, i, j, calGetNext2Dr(m, SUR.h, i, j) - f);
            calSetX2Dr(m, SUR.h, i, j, n, calGetNextX2Dr(m, SUR.h, i, j, n) + f);
        }
}

static void sur_init(struct CALModel2D* m)
{
    int i, j;
    for (i = 0; i < m->rows; i++)
        for (j = 0; j < m->columns; j++) {
            const CALreal h = calGet2Dr(m, SUR.h, i, j);
            if (h > 0.0)
                calSetCurrent2Dr(m, SUR.z, i, j, calGet2Dr(m, SUR.z, i, j) - h);
        }
}

int ref_sciddicaT_unsafe(int rows, int cols, int toroidal, int steps, double p_r, double p_eps, const double* z0,
                         const double* h0, double* z_out, double* h_out)
{
    struct CALModel2D* m = calCADef2D(rows, cols, CAL_VON_NEUMANN_NEIGHBORHOOD_2D,
                                      toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    struct CALRun2D* run = calRunDef2D(m, 1, steps, CAL_UPDATE_IMPLICIT);
    const size_t bytes = sizeof(double) * (size_t)rows * cols;
    calSetUnsafe2D(m);
    calAddElementaryProcess2D(m, sur_transition);
    SUR.z = calAddSubstate2Dr(m);
    SUR.h = calAddSubstate2Dr(m);
    SUR.r = p_r;
    SUR.eps = p_eps;
    memcpy(SUR.z->current, z0, bytes);
    memcpy(SUR.z->next, z0, bytes);
    memcpy(SUR.h->current, h0, bytes);
    memcpy(SUR.h->next, h0, bytes);
    calRunAddInitFunc2D(run, sur_init);
    if (steps > 0)
        calRun2D(run);
    else
        calRunInitSimulation2D(run);
    memcpy(z_out, SUR.z->current, bytes);
    memcpy(h_out, SUR.h->current, bytes);
    calRunFinalize2D(run);
    finalize2d(m);
    return 0;
}

/* ======================= reductions ===================================== */
/* the reference's own calReductionOperation2Db/i/r on a model holding
 * `data` (kind: 0 byte, 1 int, 2 real); its serial build folds elements
 * 0 .. rows-1 only (cal2DReduction.c:45-47), so callers compare it with the
 * oracle on grids of one column */
#include <cal2DReduction.h>

int ref_reduce2d(int kind, int rows, int cols, const void* data, int op, double* out)
{
    struct CALModel2D* m = calCADef2D(rows, cols, CAL_VON_NEUMANN_NEIGHBORHOOD_2D, CAL_SPACE_TOROIDAL, CAL_NO_OPT);
    size_t n = (size_t)rows * cols;
    if (kind == 0) {
        struct CALSubstate2Db* q = calAddSubstate2Db(m);
        memcpy(q->current, data, n);
        *out = (double)calReductionOperation2Db(m, q, (enum REDUCTION_OPERATION)op);
    } else if (kind == 1) {
        struct CALSubstate2Di* q = calAddSubstate2Di(m);
        memcpy(q->current, data, n * sizeof(int));
        *out = (double)calReductionOperation2Di(m, q, (enum REDUCTION_OPERATION)op);
    } else {
        struct CALSubstate2Dr* q = calAddSubstate2Dr(m);
        memcpy(q->current, data, n * sizeof(double));
        *out = calReductionOperation2Dr(m, q, (enum REDUCTION_OPERATION)op);
    }
    finalize2d(m);
    return 0;
}

/* ======================= substate text files ============================ */
/* the reference's own calSaveSubstate2D* / 3D* and calLoadSubstate2D* / 3D*
 * on a model holding `data` (kind: 0 byte, 1 int, 2 real; 3D slice-major) */
#include <cal2DIO.h>
#include <cal3DIO.h>

int ref_save_text(int dim, int kind, int rows, int cols, int slices, const void* data, const char* path)
{
    size_t n = (size_t)rows * cols * (dim == 3 ? slices : 1);
    CALbyte ok;
    if (dim == 2) {
        struct CALModel2D* m = calCADef2D(rows, cols, CAL_VON_NEUMANN_NEIGHBORHOOD_2D, CAL_SPACE_TOROIDAL, CAL_NO_OPT);
        if (kind == 0) {
            struct CALSubstate2Db* q = calAddSubstate2Db(m);
            memcpy(q->current, data, n);
            ok = calSaveSubstate2Db(m, q, (char*)path);
        } else if (kind == 1) {
            struct CALSubstate2Di* q = calAddSubstate2Di(m);
            memcpy(q->current, data, n * sizeof(int));
            ok = calSaveSubstate2Di(m, q, (char*)path);
        } else {
            struct CALSubstate2Dr* q = calAddSubstate2Dr(m);
            memcpy(q->current, data, n * sizeof(double));
            ok = calSaveSubstate2Dr(m, q, (char*)path);
        }
        finalize2d(m);
    } else {
        struct CALModel3D* m = calCADef3D(rows, cols, slices, CAL_VON_NEUMANN_NEIGHBORHOOD_3D, CAL_SPACE_TOROIDAL,
                                          CAL_NO_OPT);
        if (kind == 0) {
            struct CALSubstate3Db* q = calAddSubstate3Db(m);
            memcpy(q->current, data, n);
            ok = calSaveSubstate3Db(m, q, (char*)path);
        } else if (kind == 1) {
            struct CALSubstate3Di* q = calAddSubstate3Di(m);
            memcpy(q->current, data, n * sizeof(int));
            ok = calSaveSubstate3Di(m, q, (char*)path);
        } else {
            struct CALSubstate3Dr* q = calAddSubstate3Dr(m);
            memcpy(q->current, data, n * sizeof(double));
            ok = calSaveSubstate3Dr(m, q, (char*)path);
        }
        calFinalize3D(m);
    }
    return ok ? 0 : 1;
}

int ref_load_text(int dim, int kind, int rows, int cols, int slices, void* data, const char* path)
{
    size_t n = (size_t)rows * cols * (dim == 3 ? slices : 1);
    CALbyte ok;
    if (dim == 2) {
        struct CALModel2D* m = calCADef2D(rows, cols, CAL_VON_NEUMANN_NEIGHBORHOOD_2D, CAL_SPACE_TOROIDAL, CAL_NO_OPT);
        if (kind == 0) {
            struct CALSubstate2Db* q = calAddSubstate2Db(m);
            ok = calLoadSubstate2Db(m, q, (char*)path);
            memcpy(data, q->current, n);
        } else if (kind == 1) {
            struct CALSubstate2Di* q = calAddSubstate2Di(m);
            ok = calLoadSubstate2Di(m, q, (char*)path);
            memcpy(data, q->current, n * sizeof(int));
        } else {
            struct CALSubstate2Dr* q = calAddSubstate2Dr(m);
            ok = calLoadSubstate2Dr(m, q, (char*)path);
            memcpy(data, q->current, n * sizeof(double));
        }
        finalize2d(m);
    } else {
        struct CALModel3D* m = calCADef3D(rows, cols, slices, CAL_VON_NEUMANN_NEIGHBORHOOD_3D, CAL_SPACE_TOROIDAL,
                                          CAL_NO_OPT);
        if (kind == 0) {
            struct CALSubstate3Db* q = calAddSubstate3Db(m);
            ok = calLoadSubstate3Db(m, q, (char*)path);
            memcpy(data, q->current, n);
        } else if (kind == 1) {
            struct CALSubstate3Di* q = calAddSubstate3Di(m);
            ok = calLoadSubstate3Di(m, q, (char*)path);
            memcpy(data, q->current, n * sizeof(int));
        } else {
            struct CALSubstate3Dr* q = calAddSubstate3Dr(m);
            ok = calLoadSubstate3Dr(m, q, (char*)path);
            memcpy(data, q->current, n * sizeof(double));
        }
        calFinalize3D(m);
    }
    return ok ? 0 : 1;
}
