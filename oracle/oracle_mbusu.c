/*
 * oracle_mbusu.c -- CPU restatement of the mbusu unsaturated-subsurface-flow
 * program (OpenCAL/examples/cal_mbusu-glut/source/mbusu.c, identical to
 * OpenCAL-OMP/examples/calomp_mbusu-glut) on the oracle engine, 3D.  TEST
 * INFRASTRUCTURE ONLY: imported by tests/ as the checker.
 *
 * Restated, arithmetic, types and evaluation order kept:
 *   soil layers (four parameter sets)     mbusu.c:24-28, 53-86, 216-244
 *   transition function: per face of the
 *   von Neumann neighbourhood, in order,
 *   h -= dh / lato^2 * dt * mean(k) dqdh
 *   (h updated face by face), no flux
 *   across the domain's faces             mbusu.c:88-108
 *   rain on the top face                  mbusu.c:112-117
 *   pedofunctions (van Genuchten-Mualem):
 *   dq/dh, theta, moisture, k              mbusu.c:121-145, 246-266
 *   time-step bound                        mbusu.c:151-158
 *   initialisation h = -734 + quota        mbusu.c:176-276
 *   steering: dt = 0.95 min(bound, 105),
 *   accumulated in float                   mbusu.c:278-301
 *   stop at 10 days (864000 s)             mbusu.c:316-348
 *   model: 160 x 30 x 130, von Neumann 3D, toroidal, 8 real substates,
 *   implicit updates                       mbusu.c:354-376, mbusu.h:7-18
 *
 * The program's parameters are C `float`s.  lato, rain and delta_t enter
 * expressions directly, so products of them alone are evaluated in float
 * and promoted where they meet a double; the soil constants are copied into
 * double locals first, so their arithmetic is double -- both exactly as in
 * the reference.  The transcendental function is the C library's pow.
 *
 * orc_mbusu(steps, state, tail): steps 0 runs until the stop condition, a
 * negative count runs none (the initial state);
 * state (8 x 624000 doubles, or NULL) receives teta, moist_cont, psi, k, h,
 * dqdh, convergence, moist_diff; tail (3 doubles) the step reached, delta_t
 * and the accumulated time.
 */
#include "cal_oracle.h"

#include <math.h>
#include <stdlib.h>

enum { MB_ROWS = 160, MB_COLS = 30, MB_SLICES = 130 };
enum { MB_XW = 0, MB_XE = 159, MB_YIN = 0, MB_YOUT = 29, MB_ZFONDO = 0, MB_ZSUP = 129 };

/* The soil constants are float globals in the program, copied into double
 * locals before any arithmetic: here they are float-rounded values held in
 * doubles. */
typedef struct {
    double tetas, tetar, alfa, n, ks;
} mb_soil;

/* the four soil types, in the program's numbering 1..4; the values are
 * double constants converted to float, as the program's float globals are
 * initialised */
#define MB_F(x) ((float)(x))
static const mb_soil mb_soils[4] = {
    {MB_F(0.368), MB_F(0.102), MB_F(0.0334), MB_F(1.982), MB_F(0.009154)},
    {MB_F(0.351), MB_F(0.0985), MB_F(0.0363), MB_F(1.632), MB_F(0.005439)},
    {MB_F(0.325), MB_F(0.0859), MB_F(0.0345), MB_F(1.573), MB_F(0.004803)},
    {MB_F(0.325), MB_F(0.0859), MB_F(0.0345), MB_F(1.573), MB_F(0.048032)},
};

static const float mb_lato = MB_F(5.0);
static const float mb_rain = MB_F(0.000023148148);
static const int mb_output_time = 864000;

static struct {
    orc_sub *teta, *moist, *psi, *k, *h, *dqdh, *conv, *mdiff;
    float delta_t, delta_t_cum, delta_t_cum_prec;
} MB;

/* soil of cell row i at inverted depth index kinv */
static const mb_soil* mb_soil_of(int i, int kinv)
{
    if (i > 19 && i < 60 && kinv > 79 && kinv < 100)
        return &mb_soils[3];
    if (kinv > 111 && kinv < 124)
        return &mb_soils[1];
    if (kinv > 123)
        return &mb_soils[0];
    return &mb_soils[2];
}

typedef struct {
    double dqdh_inv, teta, moist, mdiff, k;
} mb_pedo;

/* the pedofunctions of pressure head psi for soil s */
static mb_pedo mb_pedofunctions(const mb_soil* s, double psi)
{
    mb_pedo p;
    const double a1 = pow(s->alfa * (-psi), (1 - s->n));
    const double a2 = pow(s->alfa * (-psi), s->n);
    const double a3 = pow((1 / (1 + a2)), (1 / s->n - 2));
    p.dqdh_inv = (a1 / (s->alfa * (s->n - 1) * (s->tetas - s->tetar))) * a3;
    const double dp = pow(s->alfa * (-psi), s->n);
    p.teta = s->tetar + ((s->tetas - s->tetar) * pow((1 / (1 + dp)), (1 - 1 / s->n)));
    const double dp0 = pow(s->alfa * (734), s->n);
    const double teta0 = s->tetar + ((s->tetas - s->tetar) * pow((1 / (1 + dp0)), (1 - 1 / s->n)));
    p.moist = p.teta / s->tetas;
    p.mdiff = p.moist - teta0 / s->tetas;
    const double satur = (p.teta - s->tetar) / (s->tetas - s->tetar);
    const double exp_c = s->n / (s->n - 1);
    const double sc = pow(satur, exp_c);
    const double exp_d = 1 - (1 / s->n);
    const double sd = pow((1 - sc), exp_d);
    p.k = s->ks * pow(satur, 0.5) * pow((1 - sd), 2);
    return p;
}

static void mb_transition(orc_ca* m, int i, int j, int k)
{
    const int kinv = (m->slices - 1) - k;
    const double volume = mb_lato * mb_lato * mb_lato;
    const double quota = mb_lato * kinv;
    const mb_soil* s = mb_soil_of(i, kinv);
    double h = orc_get(m, MB.h, i, j, k);
    const double kc = orc_get(m, MB.k, i, j, k);
    const double dq = orc_get(m, MB.dqdh, i, j, k);
    for (int n = 1; n < m->nx; n++) {
        double dh = h - orc_getx(m, MB.h, i, j, k, n);
        /* no flux across the domain's faces (neighbours 1..6: i-1, j-1,
         * j+1, i+1, k-1, k+1) */
        if ((kinv == MB_ZSUP && n == 5) || (kinv == MB_ZFONDO && n == 6) || (i == MB_XW && n == 1) ||
            (i == MB_XE && n == 4) || (j == MB_YOUT && n == 3) || (j == MB_YIN && n == 2))
            dh = 0;
        const double kmean_dq = ((kc + orc_getx(m, MB.k, i, j, k, n)) / 2.0) * dq;
        h = h - ((dh / (mb_lato * mb_lato)) * MB.delta_t * kmean_dq);
    }
    const int ymid = MB_YOUT / 2;
    if (kinv == MB_ZSUP && i < 45 && j > (ymid - 20) && j < (ymid + 20)) {
        const double rain = mb_lato * mb_rain * MB.delta_t / volume;
        h = h + rain * dq;
    }
    const double psi = h - quota;
    const mb_pedo p = mb_pedofunctions(s, psi);
    double bound;
    if ((p.k > 0) && (p.dqdh_inv > 0))
        bound = mb_lato * mb_lato / (6 * p.k * p.dqdh_inv);
    else
        bound = 1.0;
    orc_set(m, MB.dqdh, i, j, k, p.dqdh_inv);
    orc_set(m, MB.psi, i, j, k, psi);
    orc_set(m, MB.k, i, j, k, p.k);
    orc_set(m, MB.h, i, j, k, h);
    orc_set(m, MB.teta, i, j, k, p.teta);
    orc_set(m, MB.moist, i, j, k, p.moist);
    orc_set(m, MB.mdiff, i, j, k, p.mdiff);
    orc_set(m, MB.conv, i, j, k, bound);
}

static void mb_init(orc_ca* m)
{
    for (int k = 0; k < m->slices; k++)
        for (int i = 0; i < m->rows; i++)
            for (int j = 0; j < m->cols; j++) {
                const int kinv = (m->slices - 1) - k;
                const double quota = mb_lato * kinv;
                const double h = -734 + quota;
                const double psi = h - quota;
                const mb_pedo p = mb_pedofunctions(mb_soil_of(i, kinv), psi);
                orc_set(m, MB.dqdh, i, j, k, p.dqdh_inv);
                orc_set(m, MB.psi, i, j, k, psi);
                orc_set(m, MB.k, i, j, k, p.k);
                orc_set(m, MB.h, i, j, k, h);
                orc_set(m, MB.teta, i, j, k, p.teta);
                orc_set(m, MB.moist, i, j, k, p.moist);
                orc_set(m, MB.mdiff, i, j, k, p.mdiff);
            }
}

static void mb_steering(orc_ca* m)
{
    double lo = orc_get(m, MB.conv, 0, 0, 0);
    for (int k = 0; k < m->slices; k++)
        for (int i = 0; i < m->rows; i++)
            for (int j = 0; j < m->cols; j++) {
                const double v = orc_get(m, MB.conv, i, j, k);
                if (lo > v)
                    lo = v;
            }
    if (lo > 105.0)
        lo = 105.0;
    MB.delta_t = 0.95 * lo;
    MB.delta_t_cum_prec = MB.delta_t_cum;
    MB.delta_t_cum += MB.delta_t;
}

static int mb_stop(orc_ca* m)
{
    (void)m;
    return MB.delta_t_cum >= mb_output_time && MB.delta_t_cum_prec <= mb_output_time;
}

int orc_mbusu(int steps, double* state, double* tail)
{
    orc_ca* m = orc_def3d(MB_ROWS, MB_COLS, MB_SLICES, ORC_NB_VN, 1, 0);
    if (!m)
        return 1;
    MB.teta = orc_add_sub(m, ORC_R);
    MB.moist = orc_add_sub(m, ORC_R);
    MB.psi = orc_add_sub(m, ORC_R);
    MB.k = orc_add_sub(m, ORC_R);
    MB.h = orc_add_sub(m, ORC_R);
    MB.dqdh = orc_add_sub(m, ORC_R);
    MB.conv = orc_add_sub(m, ORC_R);
    MB.mdiff = orc_add_sub(m, ORC_R);
    orc_add_ep3(m, mb_transition);
    MB.delta_t = MB_F(10.0);
    MB.delta_t_cum = 0.0f;
    MB.delta_t_cum_prec = 0.0f;
    orc_run r = {0};
    r.m = m;
    r.step = 0;
    r.initial = 1;
    r.final_ = 0; /* CAL_RUN_LOOP */
    r.implicit = 1;
    r.init = mb_init;
    r.steering = mb_steering;
    r.stop = mb_stop;
    orc_run_init(&r);
    int done = 0;
    while (steps >= 0) {
        r.step++;
        const int again = orc_run_step(&r);
        done++;
        if (!again || (steps > 0 && done >= steps))
            break;
    }
    if (state) {
        orc_sub* q[8] = {MB.teta, MB.moist, MB.psi, MB.k, MB.h, MB.dqdh, MB.conv, MB.mdiff};
        const long n = (long)MB_ROWS * MB_COLS * MB_SLICES;
        for (int s = 0; s < 8; s++)
            orc_store(m, q[s], state + (size_t)s * n);
    }
    if (tail) {
        tail[0] = r.step;
        tail[1] = MB.delta_t;
        tail[2] = MB.delta_t_cum;
    }
    orc_free(m);
    return 0;
}
