/*
 * oracle_models.c -- CPU restatements of the model rules that drive the
 * parity tests, run on the oracle engine (cal_oracle.c).  TEST INFRASTRUCTURE
 * ONLY: imported by tests/, smoke() and the bench's CPU-baseline leg.
 *
 * Rules restated (arithmetic and evaluation order kept identical, because the
 * GPU path must match bit for bit):
 *   SCIDDICA-T  OpenCAL-OMP/examples/calomp_sciddicaT/source/sciddicaT.c:36-136
 *               (plain), OpenCAL/examples/cal_sciddicaT-activecells-glut/
 *               source/sciddicaT.c:20-146 (active cells: add neighbour on
 *               outflow, remove when h <= epsilon, steering on next only)
 *   Life B3/S23 OpenCAL/examples/cal_life-glut/source/life.c:16-27
 *   Life 3D     OpenCAL/examples/cal_life3D-glut/source/life3D.cpp:70-83
 * plus two probe rules of this project (hexagonal weighted sum, active-cell
 * spread) that exercise neighbour indexing and active-list semantics.
 *
 * Every entry point returns 0 on success, non-zero on an engine error.
 */
#include "cal_oracle.h"

#include <stdlib.h>
#include <string.h>

/* ======================= SCIDDICA-T ================================== */

static struct {
    orc_sub *z, *h, *f[4];
    double r, eps;
    int ac;
    int steps;
} sdt;

static void sdt_flows(orc_ca* m, int i, int j)
{
    unsigned char out[5] = {0, 0, 0, 0, 0}; /* eliminated neighbours */
    double u[5], mass, avg;
    int n, again, count;
    double hc = orc_get(m, sdt.h, i, j, 0);

    if (hc <= sdt.eps)
        return;
    mass = hc - sdt.eps;
    u[0] = orc_get(m, sdt.z, i, j, 0) + sdt.eps;
    for (n = 1; n < m->nx; n++) {
        double zn = orc_getx(m, sdt.z, i, j, 0, n);
        double hn = orc_getx(m, sdt.h, i, j, 0, n);
        u[n] = zn + hn;
    }
    do {
        again = 0;
        avg = mass;
        count = 0;
        for (n = 0; n < m->nx; n++)
            if (!out[n]) {
                avg += u[n];
                count++;
            }
        if (count != 0)
            avg /= count;
        for (n = 0; n < m->nx; n++)
            if (avg <= u[n] && !out[n]) {
                out[n] = 1;
                again = 1;
            }
    } while (again);

    for (n = 1; n < m->nx; n++) {
        if (out[n]) {
            orc_set(m, sdt.f[n - 1], i, j, 0, 0.0);
        } else {
            orc_set(m, sdt.f[n - 1], i, j, 0, (avg - u[n]) * sdt.r);
            if (sdt.ac)
                orc_add_active_x(m, i, j, 0, n);
        }
    }
}

static void sdt_width(orc_ca* m, int i, int j)
{
    double hn = orc_get(m, sdt.h, i, j, 0);
    int n;
    for (n = 1; n < m->nx; n++)
        hn += orc_getx(m, sdt.f[4 - n], i, j, 0, n) - orc_get(m, sdt.f[n - 1], i, j, 0);
    orc_set(m, sdt.h, i, j, 0, hn);
}

static void sdt_remove(orc_ca* m, int i, int j)
{
    if (orc_get(m, sdt.h, i, j, 0) <= sdt.eps)
        orc_remove_active(m, i, j, 0);
}

static void sdt_init(orc_ca* m)
{
    int i, j, q;
    for (q = 0; q < 4; q++)
        orc_init_sub(m, sdt.f[q], 0.0);
    for (i = 0; i < m->rows; i++)
        for (j = 0; j < m->cols; j++) {
            double hc = orc_get(m, sdt.h, i, j, 0);
            if (hc > 0.0) {
                double zc = orc_get(m, sdt.z, i, j, 0);
                orc_set(m, sdt.z, i, j, 0, zc - hc);
                if (sdt.ac)
                    orc_add_active(m, i, j, 0);
            }
        }
}

static void sdt_steer_plain(orc_ca* m)
{
    int q;
    for (q = 0; q < 4; q++)
        orc_init_sub(m, sdt.f[q], 0.0);
}

static void sdt_steer_ac(orc_ca* m)
{
    int q;
    for (q = 0; q < 4; q++)
        orc_init_sub_next(m, sdt.f[q], 0.0);
}

/* Trace of a plain run on a flat grid, for the mass balance: after each
 * step (at the steering, when f holds the step's outflows) the outflows of
 * border cells towards absent neighbours -- the mass that leaves the grid --
 * are summed into outflux[step - 1], and the first step after which a cell
 * of the two-cell edge band holds h != 0 is recorded. */
static struct {
    double* outflux;
    int* edge_step;
    int step;
} trc;

static void sdt_steer_trace(orc_ca* m)
{
    const int R = m->rows, C = m->cols;
    double s = 0.0;
    int i, j;
    trc.step++;
    /* von Neumann: f[0] north, f[1] west, f[2] east, f[3] south */
    for (j = 0; j < C; j++)
        s += orc_get(m, sdt.f[0], 0, j, 0);
    for (j = 0; j < C; j++)
        s += orc_get(m, sdt.f[3], R - 1, j, 0);
    for (i = 0; i < R; i++)
        s += orc_get(m, sdt.f[1], i, 0, 0);
    for (i = 0; i < R; i++)
        s += orc_get(m, sdt.f[2], i, C - 1, 0);
    trc.outflux[trc.step - 1] = s;
    if (*trc.edge_step < 0) {
        for (i = 0; i < R && *trc.edge_step < 0; i++)
            for (j = 0; j < C; j++) {
                if (i >= 2 && i < R - 2 && j == 2) {
                    j = C - 3; /* skip the interior of the row */
                    continue;
                }
                if (orc_get(m, sdt.h, i, j, 0) != 0.0) {
                    *trc.edge_step = trc.step;
                    break;
                }
            }
    }
    sdt_steer_plain(m);
}

static void export_active(const orc_ca* m, long* n_active, int* cells_out)
{
    if (n_active)
        *n_active = m->cells ? m->ncells : 0;
    if (cells_out && m->cells)
        memcpy(cells_out, m->cells, sizeof(int) * (size_t)m->dim * (size_t)m->ncells);
}

int orc_sciddicaT(int rows, int cols, int toroidal, int ac, int steps, double p_r, double p_eps,
                  const double* z0, const double* h0, double* z_out, double* h_out,
                  long* n_active, int* cells_out)
{
    orc_run run;
    int q, err;
    orc_ca* m = orc_def2d(rows, cols, ORC_NB_VN, toroidal, ac);
    if (!m)
        return 1;
    memset(&sdt, 0, sizeof(sdt));
    sdt.ac = ac;
    sdt.r = p_r;
    sdt.eps = p_eps;
    orc_add_ep2(m, sdt_flows);
    orc_add_ep2(m, sdt_width);
    if (ac)
        orc_add_ep2(m, sdt_remove);
    sdt.z = orc_add_sub(m, ORC_R);
    sdt.h = orc_add_sub(m, ORC_R);
    for (q = 0; q < 4; q++)
        sdt.f[q] = orc_add_sub(m, ORC_R);
    orc_load(m, sdt.z, z0);
    orc_load(m, sdt.h, h0);

    memset(&run, 0, sizeof(run));
    run.m = m;
    run.initial = 1;
    run.final_ = steps;
    run.implicit = 1;
    run.init = sdt_init;
    run.steering = ac ? sdt_steer_ac : sdt_steer_plain;
    if (steps > 0)
        orc_run_all(&run);
    else
        orc_run_init(&run);

    if (z_out)
        orc_store(m, sdt.z, z_out);
    if (h_out)
        orc_store(m, sdt.h, h_out);
    export_active(m, n_active, cells_out);
    err = m->error;
    orc_free(m);
    return err;
}

/* plain SCIDDICA-T on a flat grid with the trace above: outflux[steps]
 * (mass leaving per step) and edge_step (-1 when the band stays dry) */
int orc_sciddicaT_trace(int rows, int cols, int steps, double p_r, double p_eps, const double* z0, const double* h0,
                        double* z_out, double* h_out, double* outflux, int* edge_step)
{
    orc_run run;
    int q, err;
    orc_ca* m = orc_def2d(rows, cols, ORC_NB_VN, 0, 0);
    if (!m || rows < 5 || cols < 5)
        return 1;
    memset(&sdt, 0, sizeof(sdt));
    sdt.r = p_r;
    sdt.eps = p_eps;
    orc_add_ep2(m, sdt_flows);
    orc_add_ep2(m, sdt_width);
    sdt.z = orc_add_sub(m, ORC_R);
    sdt.h = orc_add_sub(m, ORC_R);
    for (q = 0; q < 4; q++)
        sdt.f[q] = orc_add_sub(m, ORC_R);
    orc_load(m, sdt.z, z0);
    orc_load(m, sdt.h, h0);
    trc.outflux = outflux;
    trc.edge_step = edge_step;
    trc.step = 0;
    *edge_step = -1;

    memset(&run, 0, sizeof(run));
    run.m = m;
    run.initial = 1;
    run.final_ = steps;
    run.implicit = 1;
    run.init = sdt_init;
    run.steering = sdt_steer_trace;
    if (steps > 0)
        orc_run_all(&run);
    else
        orc_run_init(&run);
    if (z_out)
        orc_store(m, sdt.z, z_out);
    if (h_out)
        orc_store(m, sdt.h, h_out);
    err = m->error;
    orc_free(m);
    return err;
}


/* ======================= Life 2D (B3/S23) ============================= */

static orc_sub* life_q;

static void life_rule(orc_ca* m, int i, int j)
{
    int n, sum = 0;
    for (n = 1; n < m->nx; n++)
        sum += (int)orc_getx(m, life_q, i, j, 0, n);
    if (sum == 3 || (sum == 2 && (int)orc_get(m, life_q, i, j, 0) == 1))
        orc_set(m, life_q, i, j, 0, 1);
    else
        orc_set(m, life_q, i, j, 0, 0);
}

/* state in/out as bytes (0/1) whatever the substate type */
int orc_life2d(int rows, int cols, int toroidal, int as_int, int steps,
               const unsigned char* s0, unsigned char* s_out)
{
    long c, total = (long)rows * cols;
    orc_run run;
    orc_ca* m = orc_def2d(rows, cols, ORC_NB_MOORE, toroidal, 0);
    if (!m)
        return 1;
    orc_add_ep2(m, life_rule);
    life_q = orc_add_sub(m, as_int ? ORC_I : ORC_B);
    for (c = 0; c < total; c++) {
        if (as_int)
            ((int*)life_q->cur)[c] = s0[c];
        else
            ((signed char*)life_q->cur)[c] = (signed char)s0[c];
    }
    orc_load(m, life_q, life_q->cur);
    memset(&run, 0, sizeof(run));
    run.m = m;
    run.initial = 1;
    run.final_ = steps;
    run.implicit = 1;
    if (steps > 0)
        orc_run_all(&run);
    for (c = 0; c < total; c++)
        s_out[c] = as_int ? (unsigned char)((int*)life_q->cur)[c]
                          : (unsigned char)((signed char*)life_q->cur)[c];
    orc_free(m);
    return 0;
}

/* ======================= hexagonal probe ============================== */
/* v' = v/4 + sum_n v_n * n/64 over the 6 hexagonal neighbours; the distinct
 * weights make any mistake in the even/odd neighbour tables visible. */

static orc_sub* hex_q;

static void hex_rule(orc_ca* m, int i, int j)
{
    double acc = orc_get(m, hex_q, i, j, 0) * 0.25;
    int n;
    for (n = 1; n < m->nx; n++)
        acc += orc_getx(m, hex_q, i, j, 0, n) * ((double)n * 0.015625);
    orc_set(m, hex_q, i, j, 0, acc);
}

int orc_nbprobe2d(int rows, int cols, int nbhd, int toroidal, int steps, const double* v0, double* v_out)
{
    orc_run run;
    orc_ca* m = orc_def2d(rows, cols, nbhd, toroidal, 0);
    if (!m)
        return 1;
    orc_add_ep2(m, hex_rule);
    hex_q = orc_add_sub(m, ORC_R);
    orc_load(m, hex_q, v0);
    memset(&run, 0, sizeof(run));
    run.m = m;
    run.initial = 1;
    run.final_ = steps;
    run.implicit = 1;
    if (steps > 0)
        orc_run_all(&run);
    orc_store(m, hex_q, v_out);
    orc_free(m);
    return 0;
}

/* the same rule on a custom neighbourhood: the model is defined with
 * CAL_CUSTOM_NEIGHBORHOOD_2D (no entries) and the offsets (di, dj) are
 * appended in order, as calAddNeighbor2D does (OpenCAL-OMP/source/
 * cal2D.c:444-466); entry 0 is the caller's first offset */
int orc_nbprobe2d_custom(int rows, int cols, int toroidal, int steps, int nx, const int* offs, const double* v0,
                         double* v_out)
{
    orc_run run;
    int n;
    orc_ca* m = orc_def2d(rows, cols, ORC_NB_CUSTOM, toroidal, 0);
    if (!m || nx > ORC_MAX_X)
        return 1;
    for (n = 0; n < nx; n++)
        orc_add_neighbor(m, offs[2 * n], offs[2 * n + 1], 0);
    orc_add_ep2(m, hex_rule);
    hex_q = orc_add_sub(m, ORC_R);
    orc_load(m, hex_q, v0);
    memset(&run, 0, sizeof(run));
    run.m = m;
    run.initial = 1;
    run.final_ = steps;
    run.implicit = 1;
    if (steps > 0)
        orc_run_all(&run);
    orc_store(m, hex_q, v_out);
    orc_free(m);
    return 0;
}

/* ======================= active-cell spread probe ===================== */
/* Three EPs with SCIDDICA's structure (2D or 3D):
 *   EP1: if v > thr: add every neighbour whose v is lower, and set w = v/8
 *   EP2: v' = v + sum_n (w_n - w)
 *   EP3: remove the cell when v <= thr
 *   steering: w.next = 0 on the active cells (calInitSubstateNext)        */

static struct {
    orc_sub *v, *w;
    double thr;
} acp;

static void acp_ep1(orc_ca* m, int i, int j, int k)
{
    double c = orc_get(m, acp.v, i, j, k);
    int n;
    if (c <= acp.thr)
        return;
    for (n = 1; n < m->nx; n++)
        if (orc_getx(m, acp.v, i, j, k, n) < c)
            orc_add_active_x(m, i, j, k, n);
    orc_set(m, acp.w, i, j, k, c * 0.125);
}

static void acp_ep2(orc_ca* m, int i, int j, int k)
{
    double acc = orc_get(m, acp.v, i, j, k);
    int n;
    for (n = 1; n < m->nx; n++)
        acc += orc_getx(m, acp.w, i, j, k, n) - orc_get(m, acp.w, i, j, k);
    orc_set(m, acp.v, i, j, k, acc);
}

static void acp_ep3(orc_ca* m, int i, int j, int k)
{
    if (orc_get(m, acp.v, i, j, k) <= acp.thr)
        orc_remove_active(m, i, j, k);
}

static void acp_ep1_2d(orc_ca* m, int i, int j) { acp_ep1(m, i, j, 0); }
static void acp_ep2_2d(orc_ca* m, int i, int j) { acp_ep2(m, i, j, 0); }
static void acp_ep3_2d(orc_ca* m, int i, int j) { acp_ep3(m, i, j, 0); }

static void acp_init(orc_ca* m)
{
    int i, j, k;
    orc_init_sub(m, acp.w, 0.0);
    for (i = 0; i < m->rows; i++)
        for (j = 0; j < m->cols; j++)
            for (k = 0; k < m->slices; k++)
                if (orc_get(m, acp.v, i, j, k) > acp.thr)
                    orc_add_active(m, i, j, k);
}

static void acp_steer(orc_ca* m)
{
    orc_init_sub_next(m, acp.w, 0.0);
}

int orc_acprobe(int dim, int rows, int cols, int slices, int nbhd, int toroidal, int steps,
                double thr, const double* v0, double* v_out, long* n_active, int* cells_out)
{
    orc_run run;
    int err;
    orc_ca* m = dim == 3 ? orc_def3d(rows, cols, slices, nbhd, toroidal, 1)
                         : orc_def2d(rows, cols, nbhd, toroidal, 1);
    if (!m)
        return 1;
    acp.thr = thr;
    if (dim == 3) {
        orc_add_ep3(m, acp_ep1);
        orc_add_ep3(m, acp_ep2);
        orc_add_ep3(m, acp_ep3);
    } else {
        orc_add_ep2(m, acp_ep1_2d);
        orc_add_ep2(m, acp_ep2_2d);
        orc_add_ep2(m, acp_ep3_2d);
    }
    acp.v = orc_add_sub(m, ORC_R);
    acp.w = orc_add_sub(m, ORC_R);
    orc_load(m, acp.v, v0);
    memset(&run, 0, sizeof(run));
    run.m = m;
    run.initial = 1;
    run.final_ = steps;
    run.implicit = 1;
    run.init = acp_init;
    run.steering = acp_steer;
    if (steps > 0)
        orc_run_all(&run);
    else
        orc_run_init(&run);
    orc_store(m, acp.v, v_out);
    export_active(m, n_active, cells_out);
    err = m->error;
    orc_free(m);
    return err;
}

/* ======================= Life 3D ====================================== */

static struct {
    orc_sub* q;
    int r1, r2, r3, r4;
} l3;

static void life3d_rule(orc_ca* m, int i, int j, int k)
{
    int n, sum = 0;
    int alive = (int)orc_get(m, l3.q, i, j, k);
    int nxt = alive;
    for (n = 0; n < m->nx; n++)
        sum += (int)orc_getx(m, l3.q, i, j, k, n);
    if (alive && (sum < l3.r1 || sum > l3.r2))
        nxt = 0;
    else if (!alive && (sum >= l3.r3 && sum <= l3.r4))
        nxt = 1;
    orc_set(m, l3.q, i, j, k, nxt);
}

int orc_life3d(int rows, int cols, int slices, int nbhd, int toroidal, int steps,
               int r1, int r2, int r3, int r4, const unsigned char* s0, unsigned char* s_out)
{
    orc_run run;
    long c, total = (long)rows * cols * slices;
    orc_ca* m = orc_def3d(rows, cols, slices, nbhd, toroidal, 0);
    if (!m)
        return 1;
    l3.r1 = r1;
    l3.r2 = r2;
    l3.r3 = r3;
    l3.r4 = r4;
    orc_add_ep3(m, life3d_rule);
    l3.q = orc_add_sub(m, ORC_B);
    for (c = 0; c < total; c++)
        ((signed char*)l3.q->cur)[c] = (signed char)s0[c];
    orc_load(m, l3.q, l3.q->cur);
    memset(&run, 0, sizeof(run));
    run.m = m;
    run.initial = 1;
    run.final_ = steps;
    run.implicit = 1;
    if (steps > 0)
        orc_run_all(&run);
    for (c = 0; c < total; c++)
        s_out[c] = (unsigned char)((signed char*)l3.q->cur)[c];
    orc_free(m);
    return 0;
}

/* ======================= unsafe-operation probe ========================= */
/* A rule of this project exercising every unsafe operation:
 *   EP 1: a cell with v > 0 adds 1 to v at each neighbour and removes as
 *         much from itself (calAddNextX2Di / calAddNext2Di); a cell with
 *         b > 0 moves one unit of b to its neighbour 1 + (i + j) % (nx - 1)
 *         (calAddNextX2Db / calAddNext2Db).  Integer sums: order-free.
 *   EP 2 (von Neumann / Moore): each cell writes, as the only writer of the
 *         target: w.next of its neighbour 1 = 0.5 w + 0.25 w.next there
 *         (calSetX2Dr, calGetNextX2Dr); u.current (single layer) of its
 *         neighbour 2 = w (calSetCurrentX2Dr); both layers of x at its
 *         neighbour 3 = w + 1 (calInitX2Dr).
 * Implicit update after each process. */
static struct {
    orc_sub *v, *b, *w, *u, *x;
    int ep2;
} U;

static void unsafe_ep1(orc_ca* m, int i, int j)
{
    int n;
    if (orc_get(m, U.v, i, j, 0) > 0) {
        for (n = 1; n < m->nx; n++)
            orc_add_nextx(m, U.v, i, j, 0, n, 1);
        orc_add_next(m, U.v, i, j, 0, -(m->nx - 1));
    }
    if (orc_get(m, U.b, i, j, 0) > 0) {
        orc_add_nextx(m, U.b, i, j, 0, 1 + (i + j) % (m->nx - 1), 1);
        orc_add_next(m, U.b, i, j, 0, -1);
    }
}

static void unsafe_ep2(orc_ca* m, int i, int j)
{
    const double w = orc_get(m, U.w, i, j, 0);
    orc_setx(m, U.w, i, j, 0, 1, w * 0.5 + orc_getx_next(m, U.w, i, j, 0, 1) * 0.25);
    orc_setx_cur(m, U.u, i, j, 0, 2, w);
    orc_initx(m, U.x, i, j, 0, 3, w + 1.0);
}

int orc_unsafe2d(int rows, int cols, int nbhd, int toroidal, int steps, const int* v0, const signed char* b0,
                 const double* w0, int* v_out, signed char* b_out, double* w_out, double* u_out, double* x_out)
{
    orc_run run;
    int err;
    orc_ca* m = orc_def2d(rows, cols, nbhd, toroidal, 0);
    if (!m)
        return 1;
    memset(&U, 0, sizeof(U));
    U.ep2 = nbhd == ORC_NB_VN || nbhd == ORC_NB_MOORE;
    orc_add_ep2(m, unsafe_ep1);
    if (U.ep2)
        orc_add_ep2(m, unsafe_ep2);
    U.v = orc_add_sub(m, ORC_I);
    U.b = orc_add_sub(m, ORC_B);
    U.w = orc_add_sub(m, ORC_R);
    U.u = orc_add_single(m, ORC_R);
    U.x = orc_add_sub(m, ORC_R);
    orc_load(m, U.v, v0);
    orc_load(m, U.b, b0);
    orc_load(m, U.w, w0);
    orc_init_sub(m, U.u, 0.0);
    orc_init_sub(m, U.x, 0.0);
    memset(&run, 0, sizeof(run));
    run.m = m;
    run.initial = 1;
    run.final_ = steps;
    run.implicit = 1;
    if (steps > 0)
        orc_run_all(&run);
    orc_store(m, U.v, v_out);
    orc_store(m, U.b, b_out);
    orc_store(m, U.w, w_out);
    orc_store(m, U.u, u_out);
    orc_store(m, U.x, x_out);
    err = m->error;
    orc_free(m);
    return err;
}

/* ======================= SCIDDICA-T, unsafe form ======================== */
/* OpenCAL/examples/cal_sciddicaT-unsafe/source/sciddicaT.c:35-107 (plain):
 * one process computes the outflows and moves them at once,
 * next(h) -= f at the cell, next(h) += f at the receiver, through
 * calGetNext / calSet / calGetNextX / calSetX. */
static struct {
    orc_sub *z, *h;
    double r, eps;
} SU;

static void sdtu_transition(orc_ca* m, int i, int j)
{
    unsigned char out[5] = {0, 0, 0, 0, 0};
    double u[5], mass, avg, f;
    int n, again, count;
    mass = orc_get(m, SU.h, i, j, 0) - SU.eps;
    u[0] = orc_get(m, SU.z, i, j, 0) + SU.eps;
    for (n = 1; n < m->nx; n++)
        u[n] = orc_getx(m, SU.z, i, j, 0, n) + orc_getx(m, SU.h, i, j, 0, n);
    do {
        again = 0;
        avg = mass;
        count = 0;
        for (n = 0; n < m->nx; n++)
            if (!out[n]) {
                avg += u[n];
                count++;
            }
        if (count != 0)
            avg /= count;
        for (n = 0; n < m->nx; n++)
            if (avg <= u[n] && !out[n]) {
                out[n] = 1;
                again = 1;
            }
    } while (again);
    for (n = 1; n < m->nx; n++)
        if (!out[n]) {
            f = (avg - u[n]) * SU.r;
            orc_set(m, SU.h, i, j, 0, orc_get_next(m, SU.h, i, j, 0) - f);
            orc_setx(m, SU.h, i, j, 0, n, orc_getx_next(m, SU.h, i, j, 0, n) + f);
        }
}

static void sdtu_init(orc_ca* m)
{
    int i, j;
    for (i = 0; i < m->rows; i++)
        for (j = 0; j < m->cols; j++) {
            const double h = orc_get(m, SU.h, i, j, 0);
            if (h > 0.0)
                orc_set_cur(m, SU.z, i, j, 0, orc_get(m, SU.z, i, j, 0) - h);
        }
}

int orc_sciddicaT_unsafe(int rows, int cols, int toroidal, int steps, double p_r, double p_eps, const double* z0,
                         const double* h0, double* z_out, double* h_out)
{
    orc_run run;
    int err;
    orc_ca* m = orc_def2d(rows, cols, ORC_NB_VN, toroidal, 0);
    if (!m)
        return 1;
    memset(&SU, 0, sizeof(SU));
    SU.r = p_r;
    SU.eps = p_eps;
    orc_add_ep2(m, sdtu_transition);
    SU.z = orc_add_sub(m, ORC_R);
    SU.h = orc_add_sub(m, ORC_R);
    orc_load(m, SU.z, z0);
    orc_load(m, SU.h, h0);
    memset(&run, 0, sizeof(run));
    run.m = m;
    run.initial = 1;
    run.final_ = steps;
    run.implicit = 1;
    run.init = sdtu_init;
    if (steps > 0)
        orc_run_all(&run);
    else
        orc_run_init(&run);
    orc_store(m, SU.z, z_out);
    orc_store(m, SU.h, h_out);
    err = m->error;
    orc_free(m);
    return err;
}
