/*
 * oracle_sciara.c -- CPU restatement of the SCIARA-fv2 lava-flow program
 * (OpenCAL-OMP/examples/calomp_sciara-fv2, identical to
 * OpenCAL/examples/cal_sciara-fv2) on the oracle engine.  TEST
 * INFRASTRUCTURE ONLY: imported by tests/ and the bench's CPU-baseline leg.
 *
 * Restated, arithmetic and evaluation order kept:
 *   updateVentsEmission      source/Sciara.cpp:3-16, vent.h:74-82 (thickness)
 *   powerLaw, outflowsMin    source/Sciara.cpp:18-90 (Moore minimisation with
 *                            atan/cos shear-resistance test)
 *   empiricalFlows           source/Sciara.cpp:92-105
 *   width_update             source/Sciara.cpp:106-135 (mass and heat mixing)
 *   updateTemperature        source/Sciara.cpp:137-169 (radiative cooling,
 *                            solidification into Sz and Msl)
 *   removeActiveCells        source/Sciara.cpp:171-175
 *   stopCondition, steering  source/Sciara.cpp:177-197
 *   evaluatePowerLawParams, MakeBorder, simulationInitialize
 *                            source/Sciara.cpp:199-285
 *   initSciara (substates, EP order, run definition)
 *                            source/Sciara.cpp:287-356
 *   loadConfiguration's effect: Sz = DEM, vents in row-major order of the
 *   vent matrix, Pac = Pc * Pc  (source/io.cpp:226-240, vent.cpp:15-29)
 * The transcendental functions are the C library's (pow, atan, cos, log10),
 * as in the reference.
 *
 * params (13 doubles): Pclock, PTsol, PTvent, Pr(Tsol), Pr(Tvent), Phc(Tsol),
 * Phc(Tvent), Pcool, Prho, Pepsilon, Psigma, Pcv (the .cfg order), Pc (cell
 * size).  vents: nvents (x = column, y = row) pairs in the reference's vent
 * order; rates: nvents x nphases emission rates [m^3/s], each phase lasting
 * emission_time seconds.
 */
#include "cal_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define SCI_NF 8

static struct {
    orc_sub *Sz, *Slt, *St, *f[SCI_NF];
    orc_sub *Mb, *Msl, *Sz_t0, *Mv;
    double Pclock, PTsol, PTvent, Pr_Tsol, Pr_Tvent, Phc_Tsol, Phc_Tvent, Pcool, Prho, Pepsilon, Psigma, Pcv;
    double Pc, Pac, rad2, a, b, c, d;
    double elapsed_time, effusion_duration;
    unsigned emission_time;
    int nvents, nphases;
    const int* vent_xy;
    const double* rates;
    int ac;
} S;

static double vent_thickness(int v)
{
    unsigned i = (unsigned)(S.elapsed_time / S.emission_time);
    if (i >= (unsigned)S.nphases)
        return 0;
    return S.rates[v * S.nphases + i] / S.Pac * S.Pclock;
}

static void sci_vents(orc_ca* m, int i, int j)
{
    int k;
    for (k = 0; k < S.nvents; k++) {
        const int xv = S.vent_xy[2 * k], yv = S.vent_xy[2 * k + 1];
        if (i == yv && j == xv) {
            const double emitted = vent_thickness(k);
            if (emitted > 0) {
                orc_set(m, S.Slt, yv, xv, 0, orc_get(m, S.Slt, yv, xv, 0) + emitted);
                orc_set(m, S.St, yv, xv, 0, S.PTvent);
            }
        }
    }
}

static double power_law(double k1, double k2, double T) { return pow(10, k1 + k2 * T); }

static void outflows_min(orc_ca* m, int i, int j, double* f)
{
    int in_set[9];
    double z[9], h[9], H[9], theta[9], w[9], Pr[9];
    int loop, counter, k;
    double avg, _w, _Pr, hc;
    const double t = orc_get(m, S.St, i, j, 0);

    _w = S.Pc;
    _Pr = power_law(S.a, S.b, t);
    hc = power_law(S.c, S.d, t);
    for (k = 0; k < 9; k++) {
        double sz, sz0;
        h[k] = orc_getx(m, S.Slt, i, j, 0, k);
        H[k] = f[k] = theta[k] = 0;
        w[k] = _w;
        Pr[k] = _Pr;
        sz = orc_getx(m, S.Sz, i, j, 0, k);
        sz0 = orc_get(m, S.Sz, i, j, 0);
        if (k < 5)
            z[k] = orc_getx(m, S.Sz, i, j, 0, k);
        else
            z[k] = sz0 - (sz0 - sz) / S.rad2;
    }
    H[0] = z[0];
    in_set[0] = 1;
    for (k = 1; k < 9; k++)
        if (z[0] + h[0] > z[k] + h[k]) {
            H[k] = z[k] + h[k];
            theta[k] = atan(((z[0] + h[0]) - (z[k] + h[k])) / w[k]);
            in_set[k] = 1;
        } else {
            in_set[k] = 0;
        }
    do {
        loop = 0;
        avg = h[0];
        counter = 0;
        for (k = 0; k < 9; k++)
            if (in_set[k]) {
                avg += H[k];
                counter++;
            }
        if (counter != 0)
            avg = avg / (double)counter;
        for (k = 0; k < 9; k++)
            if (in_set[k] && avg <= H[k]) {
                in_set[k] = 0;
                loop = 1;
            }
    } while (loop);
    for (k = 1; k < 9; k++)
        if (in_set[k] && h[0] > hc * cos(theta[k]))
            f[k] = Pr[k] * (avg - H[k]);
}

static void sci_flows(orc_ca* m, int i, int j)
{
    if (orc_get(m, S.Slt, i, j, 0) > 0) {
        double f[9];
        int k;
        outflows_min(m, i, j, f);
        for (k = 1; k < 9; k++)
            if (f[k] > 0) {
                orc_set(m, S.f[k - 1], i, j, 0, f[k]);
                if (S.ac)
                    orc_add_active_x(m, i, j, 0, k);
            }
    }
}

static void sci_width(orc_ca* m, int i, int j)
{
    static const int opp[SCI_NF] = {3, 2, 1, 0, 6, 7, 4, 5};
    const double initial_h = orc_get(m, S.Slt, i, j, 0);
    const double initial_t = orc_get(m, S.St, i, j, 0);
    double residual_lava = initial_h;
    double h_next = initial_h, t_next;
    double ht = 0, in_sum = 0, out_sum = 0;
    int n;
    for (n = 1; n < m->nx; n++) {
        const double in_flow = orc_getx(m, S.f[opp[n - 1]], i, j, 0, n);
        const double out_flow = orc_get(m, S.f[n - 1], i, j, 0);
        const double neigh_t = orc_getx(m, S.St, i, j, 0, n);
        ht += in_flow * neigh_t;
        in_sum += in_flow;
        out_sum += out_flow;
    }
    h_next += in_sum - out_sum;
    orc_set(m, S.Slt, i, j, 0, h_next);
    if (in_sum > 0 || out_sum > 0) {
        residual_lava -= out_sum;
        t_next = (residual_lava * initial_t + ht) / (residual_lava + in_sum);
        orc_set(m, S.St, i, j, 0, t_next);
    }
}

static void sci_temperature(orc_ca* m, int i, int j)
{
    double nT, h, T, aus;
    const double sh = orc_get(m, S.Slt, i, j, 0);
    double st = orc_get(m, S.St, i, j, 0);
    const double sz = orc_get(m, S.Sz, i, j, 0);
    if (sh > 0 && !orc_get(m, S.Mb, i, j, 0)) {
        h = sh;
        T = st;
        if (h != 0) {
            nT = T;
            aus = 1.0 + (3 * pow(nT, 3.0) * S.Pepsilon * S.Psigma * S.Pclock * S.Pcool) /
                            (S.Prho * S.Pcv * h * S.Pac);
            st = nT / pow(aus, 1.0 / 3.0);
            orc_set(m, S.St, i, j, 0, st);
        }
        if (st <= S.PTsol && sh > 0) {
            orc_set(m, S.Sz, i, j, 0, sz + sh);
            orc_set_cur(m, S.Msl, i, j, 0, orc_get(m, S.Msl, i, j, 0) + sh);
            orc_set(m, S.Slt, i, j, 0, 0);
            orc_set(m, S.St, i, j, 0, S.PTsol);
        } else {
            orc_set(m, S.Sz, i, j, 0, sz);
        }
    }
}

static void sci_remove(orc_ca* m, int i, int j)
{
    const double st = orc_get(m, S.St, i, j, 0);
    if (st <= S.PTsol && !orc_get(m, S.Mb, i, j, 0))
        orc_remove_active(m, i, j, 0);
}

static int sci_stop(orc_ca* m)
{
    (void)m;
    return S.elapsed_time >= S.effusion_duration;
}

static void sci_steering(orc_ca* m)
{
    int q, i, j;
    for (q = 0; q < SCI_NF; q++)
        orc_init_sub(m, S.f[q], 0);
    for (i = 0; i < m->rows; i++)
        for (j = 0; j < m->cols; j++)
            if (orc_get(m, S.Mb, i, j, 0) == 1) {
                orc_set(m, S.Slt, i, j, 0, 0);
                orc_set(m, S.St, i, j, 0, 0);
            }
    S.elapsed_time += S.Pclock;
}

static void power_law_params(double value_sol, double value_vent, double* k1, double* k2)
{
    *k2 = (log10(value_vent) - log10(value_sol)) / (S.PTvent - S.PTsol);
    *k1 = log10(value_sol) - *k2 * (S.PTsol);
}

static void mark_border(orc_ca* m, int i, int j)
{
    orc_set_cur(m, S.Mb, i, j, 0, 1);
    if (S.ac)
        orc_add_active(m, i, j, 0);
}

static void make_border(orc_ca* m)
{
    int i, j, k;
    i = 0;
    for (j = 0; j < m->cols; j++)
        if (orc_get(m, S.Sz, i, j, 0) >= 0)
            mark_border(m, i, j);
    i = m->rows - 1;
    for (j = 0; j < m->cols; j++)
        if (orc_get(m, S.Sz, i, j, 0) >= 0)
            mark_border(m, i, j);
    j = 0;
    for (i = 0; i < m->rows; i++)
        if (orc_get(m, S.Sz, i, j, 0) >= 0)
            mark_border(m, i, j);
    j = m->cols - 1;
    for (i = 0; i < m->rows; i++)
        if (orc_get(m, S.Sz, i, j, 0) >= 0)
            mark_border(m, i, j);
    for (i = 1; i < m->rows - 1; i++)
        for (j = 1; j < m->cols - 1; j++)
            if (orc_get(m, S.Sz, i, j, 0) >= 0)
                for (k = 1; k < m->nx; k++)
                    if (orc_getx(m, S.Sz, i, j, 0, k) < 0) {
                        mark_border(m, i, j);
                        break;
                    }
}

static void sci_init(orc_ca* m)
{
    int k;
    S.elapsed_time = 0;
    S.effusion_duration = (double)S.emission_time * S.nphases;
    make_border(m);
    power_law_params(S.Pr_Tsol, S.Pr_Tvent, &S.a, &S.b);
    power_law_params(S.Phc_Tsol, S.Phc_Tvent, &S.c, &S.d);
    if (S.ac)
        for (k = 0; k < S.nvents; k++)
            orc_add_active(m, S.vent_xy[2 * k + 1], S.vent_xy[2 * k], 0);
    orc_update(m);
}

int orc_sciara(int rows, int cols, int ac, int max_steps, const double* params, int nvents, const int* vent_xy,
               unsigned emission_time, int nphases, const double* rates, const double* z0, const double* slt0,
               const double* st0, double* z_out, double* slt_out, double* st_out, double* msl_out, int* steps_done,
               long* n_active, int* cells_out)
{
    orc_run run;
    int q, err, done = 0;
    orc_ca* m = orc_def2d(rows, cols, ORC_NB_MOORE, 0, ac);
    if (!m)
        return 1;
    memset(&S, 0, sizeof(S));
    S.ac = ac;
    S.Pclock = params[0];
    S.PTsol = params[1];
    S.PTvent = params[2];
    S.Pr_Tsol = params[3];
    S.Pr_Tvent = params[4];
    S.Phc_Tsol = params[5];
    S.Phc_Tvent = params[6];
    S.Pcool = params[7];
    S.Prho = params[8];
    S.Pepsilon = params[9];
    S.Psigma = params[10];
    S.Pcv = params[11];
    S.Pc = params[12];
    S.Pac = S.Pc * S.Pc;
    S.rad2 = sqrt(2.0);
    S.nvents = nvents;
    S.vent_xy = vent_xy;
    S.emission_time = emission_time;
    S.nphases = nphases;
    S.rates = rates;

    S.Sz = orc_add_sub(m, ORC_R);
    S.Slt = orc_add_sub(m, ORC_R);
    S.St = orc_add_sub(m, ORC_R);
    S.Mb = orc_add_single(m, ORC_B);
    S.Mv = orc_add_single(m, ORC_I);
    S.Msl = orc_add_single(m, ORC_R);
    S.Sz_t0 = orc_add_single(m, ORC_R);
    for (q = 0; q < SCI_NF; q++)
        S.f[q] = orc_add_sub(m, ORC_R);
    orc_add_ep2(m, sci_vents);
    orc_add_ep2(m, sci_flows);
    orc_add_ep2(m, sci_width);
    orc_add_ep2(m, sci_temperature);
    if (ac)
        orc_add_ep2(m, sci_remove);
    orc_load(m, S.Sz, z0);
    orc_load(m, S.Sz_t0, z0);
    if (slt0)
        orc_load(m, S.Slt, slt0);
    if (st0)
        orc_load(m, S.St, st0);

    memset(&run, 0, sizeof(run));
    run.m = m;
    run.initial = 1;
    run.final_ = max_steps;
    run.implicit = 1;
    run.init = sci_init;
    run.steering = sci_steering;
    run.stop = sci_stop;
    orc_run_init(&run);
    for (run.step = run.initial; run.step <= run.final_ || run.final_ == 0; run.step++) {
        done++;
        if (!orc_run_step(&run))
            break;
    }
    if (steps_done)
        *steps_done = done;
    if (z_out)
        orc_store(m, S.Sz, z_out);
    if (slt_out)
        orc_store(m, S.Slt, slt_out);
    if (st_out)
        orc_store(m, S.St, st_out);
    if (msl_out)
        orc_store(m, S.Msl, msl_out);
    if (n_active)
        *n_active = m->cells ? m->ncells : 0;
    if (cells_out && m->cells)
        memcpy(cells_out, m->cells, sizeof(int) * 2 * (size_t)m->ncells);
    err = m->error;
    orc_free(m);
    return err;
}
