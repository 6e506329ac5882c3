/*
 * sciara.cu -- the SCIARA-fv2 lava-flow program on opencal-gb300, written
 * against the C API as the reference writes it
 * (OpenCAL-OMP/examples/calomp_sciara-fv2/source/Sciara.cpp:3-356): five
 * elementary processes registered with calAddElementaryProcess2D (vent
 * emission, empirical flows by minimisation with the shear-resistance test,
 * mass and heat mixing, radiative cooling and solidification, removal of
 * solidified active cells), Moore neighbourhood, flat boundary with a
 * border mask, implicit update, steering and a stop condition at the end
 * of the emission.  Active cells on or off.
 *
 * GPU-side differences from the host program, none of which changes a
 * result:
 *   - the steering's border reset (Sciara.cpp:185-193, a host loop over all
 *     cells) is a device process applied with calApplyElementaryProcess2D:
 *     the border cells are exactly the cells it changes, and with active
 *     cells on they are always active (MakeBorder adds them, removal skips
 *     them), so both visit every border cell;
 *   - the elapsed time the vent process reads is a device variable advanced
 *     by a one-thread kernel in the steering (so that a recorded step
 *     replays correctly); the host stop condition keeps its own copy,
 *     advanced by the same additions, from the run's step counter.
 * The transcendental parts (power laws, shear test, cooling) use the
 * equivalent forms of sciara_math.cuh (exp10, no atan / cos, T^3, cbrt);
 * log10 of the power-law parameters is evaluated once on the host (C
 * library), as in the reference.  Results therefore agree with the
 * reference to rounding (not bit for bit) where those are involved.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "opencal/cal2D.h"
#include "opencal/cal2DRun.h"

#include "sciara_math.cuh"

#define SCI_NF 8
#define SCI_MAX_VENTS 64
#define SCI_MAX_PHASES 256

struct SciaraSubstates {
    struct CALSubstate2Dr* Sz;
    struct CALSubstate2Dr* Slt;
    struct CALSubstate2Dr* St;
    struct CALSubstate2Dr* Sz_t0;
    struct CALSubstate2Di* Mv;
    struct CALSubstate2Db* Mb;
    struct CALSubstate2Dr* Msl;
    struct CALSubstate2Dr* f[SCI_NF];
};

struct SciaraParams {
    double Pclock, Pc, Pac, PTsol, PTvent, Pr_Tsol, Pr_Tvent, a, b, Phc_Tsol, Phc_Tvent, c, d;
    double Pcool, Prho, Pepsilon, Psigma, Pcv, rad2;
    double effusion_duration;
    unsigned emission_time;
    int nvents, nphases, active;
    int libm; /* 1: pow / atan / cos as the reference calls them (sciara_math.cuh), 0: the identity forms */
    int vent_x[SCI_MAX_VENTS], vent_y[SCI_MAX_VENTS];
    double rates[SCI_MAX_VENTS * SCI_MAX_PHASES];
};

__managed__ struct SciaraSubstates SQ;
__managed__ struct SciaraParams SP;
__device__ double sci_elapsed_dev; /* the reference's sciara->elapsed_time, as the device sees it */

static struct CALRun2D* sci_run = nullptr;
static double sci_host_elapsed = 0.0;
static int sci_host_elapsed_step = 0;

/* TVent::thickness (include/vent.h:74-82) */
static __device__ __forceinline__ double sci_vent_thickness(int v, double elapsed)
{
    const unsigned i = (unsigned)(elapsed / SP.emission_time);
    if (i >= (unsigned)SP.nphases)
        return 0;
    return SP.rates[v * SP.nphases + i] / SP.Pac * SP.Pclock;
}

CAL_ELEMENTARY_PROCESS_2D(sciara_vents_emission)(struct CALModel2D* model, int i, int j)
{
    for (int k = 0; k < SP.nvents; k++) {
        const int xv = SP.vent_x[k], yv = SP.vent_y[k];
        if (i == yv && j == xv) {
            const double emitted = sci_vent_thickness(k, sci_elapsed_dev);
            if (emitted > 0) {
                calSet2Dr(model, SQ.Slt, yv, xv, calGet2Dr(model, SQ.Slt, yv, xv) + emitted);
                calSet2Dr(model, SQ.St, yv, xv, SP.PTvent);
            }
        }
    }
}

/* outflowsMin (Sciara.cpp:23-90); f[0..8], f[0] unused */
static __device__ void sci_outflows_min(struct CALModel2D* model, int i, int j, double* f)
{
    bool in_set[9];
    double z[9], h[9], H[9], dz[9];
    const double t = calGet2Dr(model, SQ.St, i, j);
    const double w = SP.Pc;
    const double Pr = SP.libm ? sci_power_law_libm(SP.a, SP.b, t) : sci_power_law(SP.a, SP.b, t);
    const double hc = SP.libm ? sci_power_law_libm(SP.c, SP.d, t) : sci_power_law(SP.c, SP.d, t);
    const double sz0 = calGet2Dr(model, SQ.Sz, i, j);
    for (int k = 0; k < 9; k++) {
        h[k] = calGetX2Dr(model, SQ.Slt, i, j, k);
        H[k] = f[k] = dz[k] = 0;
        const double sz = calGetX2Dr(model, SQ.Sz, i, j, k);
        if (k < 5)
            z[k] = sz;
        else
            z[k] = sz0 - (sz0 - sz) / SP.rad2;
    }
    H[0] = z[0];
    in_set[0] = true;
    for (int k = 1; k < 9; k++)
        if (z[0] + h[0] > z[k] + h[k]) {
            H[k] = z[k] + h[k];
            dz[k] = (z[0] + h[0]) - (z[k] + h[k]);
            in_set[k] = true;
        } else {
            in_set[k] = false;
        }
    bool loop;
    double avg;
    do {
        loop = false;
        avg = h[0];
        int counter = 0;
        for (int k = 0; k < 9; k++)
            if (in_set[k]) {
                avg += H[k];
                counter++;
            }
        if (counter != 0)
            avg = avg / (double)counter;
        for (int k = 0; k < 9; k++)
            if (in_set[k] && avg <= H[k]) {
                in_set[k] = false;
                loop = true;
            }
    } while (loop);
    for (int k = 1; k < 9; k++)
        if (in_set[k] && (SP.libm ? sci_shear_exceeded_libm(h[0], hc, dz[k], w)
                                  : sci_shear_exceeded(h[0], hc, dz[k], w)))
            f[k] = Pr * (avg - H[k]);
}

CAL_ELEMENTARY_PROCESS_2D(sciara_empirical_flows)(struct CALModel2D* model, int i, int j)
{
    if (calGet2Dr(model, SQ.Slt, i, j) > 0) {
        double f[9];
        sci_outflows_min(model, i, j, f);
        for (int k = 1; k < 9; k++)
            if (f[k] > 0) {
                calSet2Dr(model, SQ.f[k - 1], i, j, f[k]);
                if (SP.active)
                    calAddActiveCellX2D(model, i, j, k);
            }
    }
}

CAL_ELEMENTARY_PROCESS_2D(sciara_width_update)(struct CALModel2D* model, int i, int j)
{
    const int opp[SCI_NF] = {3, 2, 1, 0, 6, 7, 4, 5};
    const double initial_h = calGet2Dr(model, SQ.Slt, i, j);
    const double initial_t = calGet2Dr(model, SQ.St, i, j);
    double residual_lava = initial_h;
    double h_next = initial_h;
    double ht = 0, in_sum = 0, out_sum = 0;
    for (int n = 1; n < model->sizeof_X; n++) {
        const double in_flow = calGetX2Dr(model, SQ.f[opp[n - 1]], i, j, n);
        const double out_flow = calGet2Dr(model, SQ.f[n - 1], i, j);
        const double neigh_t = calGetX2Dr(model, SQ.St, i, j, n);
        ht += in_flow * neigh_t;
        in_sum += in_flow;
        out_sum += out_flow;
    }
    h_next += in_sum - out_sum;
    calSet2Dr(model, SQ.Slt, i, j, h_next);
    if (in_sum > 0 || out_sum > 0) {
        residual_lava -= out_sum;
        const double t_next = (residual_lava * initial_t + ht) / (residual_lava + in_sum);
        calSet2Dr(model, SQ.St, i, j, t_next);
    }
}

CAL_ELEMENTARY_PROCESS_2D(sciara_update_temperature)(struct CALModel2D* model, int i, int j)
{
    const double sh = calGet2Dr(model, SQ.Slt, i, j);
    double st = calGet2Dr(model, SQ.St, i, j);
    const double sz = calGet2Dr(model, SQ.Sz, i, j);
    if (sh > 0 && !calGet2Db(model, SQ.Mb, i, j)) {
        const double h = sh;
        const double T = st;
        if (h != 0) {
            const double nT = T;
            double aus;
            st = SP.libm ? sci_cool_libm(nT, h, SP.Pepsilon, SP.Psigma, SP.Pclock, SP.Pcool, SP.Prho, SP.Pcv,
                                         SP.Pac, &aus)
                         : sci_cool(nT, h, SP.Pepsilon, SP.Psigma, SP.Pclock, SP.Pcool, SP.Prho, SP.Pcv, SP.Pac,
                                    &aus);
            calSet2Dr(model, SQ.St, i, j, st);
        }
        if (st <= SP.PTsol && sh > 0) {
            calSet2Dr(model, SQ.Sz, i, j, sz + sh);
            calSetCurrent2Dr(model, SQ.Msl, i, j, calGet2Dr(model, SQ.Msl, i, j) + sh);
            calSet2Dr(model, SQ.Slt, i, j, 0);
            calSet2Dr(model, SQ.St, i, j, SP.PTsol);
        } else {
            calSet2Dr(model, SQ.Sz, i, j, sz);
        }
    }
}

CAL_ELEMENTARY_PROCESS_2D(sciara_remove_active_cells)(struct CALModel2D* model, int i, int j)
{
    const double st = calGet2Dr(model, SQ.St, i, j);
    if (st <= SP.PTsol && !calGet2Db(model, SQ.Mb, i, j))
        calRemoveActiveCell2D(model, i, j);
}

/* the steering's border reset (Sciara.cpp:187-192) */
CAL_ELEMENTARY_PROCESS_2D(sciara_border_reset)(struct CALModel2D* model, int i, int j)
{
    if (calGet2Db(model, SQ.Mb, i, j) == CAL_TRUE) {
        calSet2Dr(model, SQ.Slt, i, j, 0);
        calSet2Dr(model, SQ.St, i, j, 0);
    }
}

__global__ void sci_advance_elapsed(double dt)
{
    sci_elapsed_dev += dt;
}

__global__ void sci_reset_elapsed() { sci_elapsed_dev = 0.0; }

/* stopCondition (Sciara.cpp:177-183): elapsed time as the steering of the
 * steps run so far accumulated it */
static CALbyte sciara_stop(struct CALModel2D* model)
{
    (void)model;
    const int step = sci_run ? sci_run->step : 0;
    while (sci_host_elapsed_step < step) {
        sci_host_elapsed += SP.Pclock;
        sci_host_elapsed_step++;
    }
    return sci_host_elapsed >= SP.effusion_duration ? CAL_TRUE : CAL_FALSE;
}

static void sciara_steering(struct CALModel2D* model)
{
    for (int q = 0; q < SCI_NF; q++)
        calInitSubstate2Dr(model, SQ.f[q], 0);
    calApplyElementaryProcess2D(model, sciara_border_reset);
    sci_advance_elapsed<<<1, 1, 0, (cudaStream_t)calGetStream2D(model)>>>(SP.Pclock);
}

static void sci_power_law_params(double value_sol, double value_vent, double* k1, double* k2)
{
    *k2 = (log10(value_vent) - log10(value_sol)) / (SP.PTvent - SP.PTsol);
    *k1 = log10(value_sol) - *k2 * (SP.PTsol);
}

static void sci_mark_border(struct CALModel2D* model, int i, int j)
{
    calSetCurrent2Db(model, SQ.Mb, i, j, CAL_TRUE);
    if (SP.active)
        calAddActiveCell2D(model, i, j);
}

/* MakeBorder (Sciara.cpp:206-250), on the host mirrors */
static void sci_make_border(struct CALModel2D* model)
{
    const int rows = model->rows, cols = model->columns;
    int i, j;
    i = 0;
    for (j = 0; j < cols; j++)
        if (calGet2Dr(model, SQ.Sz, i, j) >= 0)
            sci_mark_border(model, i, j);
    i = rows - 1;
    for (j = 0; j < cols; j++)
        if (calGet2Dr(model, SQ.Sz, i, j) >= 0)
            sci_mark_border(model, i, j);
    j = 0;
    for (i = 0; i < rows; i++)
        if (calGet2Dr(model, SQ.Sz, i, j) >= 0)
            sci_mark_border(model, i, j);
    j = cols - 1;
    for (i = 0; i < rows; i++)
        if (calGet2Dr(model, SQ.Sz, i, j) >= 0)
            sci_mark_border(model, i, j);
    for (i = 1; i < rows - 1; i++)
        for (j = 1; j < cols - 1; j++)
            if (calGet2Dr(model, SQ.Sz, i, j) >= 0)
                for (int k = 1; k < model->sizeof_X; k++)
                    if (calGetX2Dr(model, SQ.Sz, i, j, k) < 0) {
                        sci_mark_border(model, i, j);
                        break;
                    }
}

/* simulationInitialize (Sciara.cpp:252-285) */
static void sciara_init(struct CALModel2D* model)
{
    sci_host_elapsed = 0.0;
    sci_host_elapsed_step = 0;
    sci_reset_elapsed<<<1, 1, 0, (cudaStream_t)calGetStream2D(model)>>>();
    SP.effusion_duration = (double)SP.emission_time * SP.nphases;
    sci_make_border(model);
    sci_power_law_params(SP.Pr_Tsol, SP.Pr_Tvent, &SP.a, &SP.b);
    sci_power_law_params(SP.Phc_Tsol, SP.Phc_Tvent, &SP.c, &SP.d);
    if (SP.active)
        for (int k = 0; k < SP.nvents; k++)
            calAddActiveCell2D(model, SP.vent_y[k], SP.vent_x[k]);
    calUpdate2D(model);
}

/* Runs SCIARA-fv2 on the given inputs and returns the final state -- the
 * contract of the oracle's orc_sciara.  params: Pclock, PTsol, PTvent,
 * Pr(Tsol), Pr(Tvent), Phc(Tsol), Phc(Tvent), Pcool, Prho, Pepsilon, Psigma,
 * Pcv, Pc.  vents: (x, y) pairs; rates: nvents x nphases m^3/s.  max_steps 0
 * runs until the emission ends.  graph != 0 replays a recorded step. */
/* 0: the identity forms of sciara_math.cuh (default); 1: pow / atan / cos
 * as the reference writes them (CUDA's functions); applies to the following
 * cal_sciara_run calls */
static int g_sci_libm = 0;
extern "C" int cal_sciara_set_math(int form)
{
    if (form != 0 && form != 1)
        return CAL_ERROR_INVALID_ARGUMENT;
    g_sci_libm = form;
    return CAL_SUCCESS;
}

extern "C" int cal_sciara_run(int rows, int cols, int ac, int max_steps, const double* params, int nvents,
                              const int* vent_xy, unsigned emission_time, int nphases, const double* rates,
                              const double* z0, const double* slt0, const double* st0, double* z_out,
                              double* slt_out, double* st_out, double* msl_out, int* steps_done, long* n_active,
                              int* cells_out, int graph, double* ms)
{
    calClearError();
    if (nvents < 0 || nvents > SCI_MAX_VENTS || nphases < 0 || nphases > SCI_MAX_PHASES)
        return CAL_ERROR_INVALID_ARGUMENT;
    memset(&SP, 0, sizeof(SP));
    SP.Pclock = params[0];
    SP.PTsol = params[1];
    SP.PTvent = params[2];
    SP.Pr_Tsol = params[3];
    SP.Pr_Tvent = params[4];
    SP.Phc_Tsol = params[5];
    SP.Phc_Tvent = params[6];
    SP.Pcool = params[7];
    SP.Prho = params[8];
    SP.Pepsilon = params[9];
    SP.Psigma = params[10];
    SP.Pcv = params[11];
    SP.Pc = params[12];
    SP.Pac = SP.Pc * SP.Pc;
    SP.rad2 = sqrt(2.0);
    SP.emission_time = emission_time;
    SP.nvents = nvents;
    SP.nphases = nphases;
    SP.active = ac;
    SP.libm = g_sci_libm;
    for (int k = 0; k < nvents; k++) {
        SP.vent_x[k] = vent_xy[2 * k];
        SP.vent_y[k] = vent_xy[2 * k + 1];
    }
    memcpy(SP.rates, rates, sizeof(double) * (size_t)nvents * nphases);

    struct CALModel2D* model = calCADef2D(rows, cols, CAL_MOORE_NEIGHBORHOOD_2D, CAL_SPACE_FLAT,
                                          ac ? CAL_OPT_ACTIVE_CELLS : CAL_NO_OPT);
    if (!model)
        return calGetLastError();
    SQ.Sz = calAddSubstate2Dr(model);
    SQ.Slt = calAddSubstate2Dr(model);
    SQ.St = calAddSubstate2Dr(model);
    SQ.Mb = calAddSingleLayerSubstate2Db(model);
    SQ.Mv = calAddSingleLayerSubstate2Di(model);
    SQ.Msl = calAddSingleLayerSubstate2Dr(model);
    SQ.Sz_t0 = calAddSingleLayerSubstate2Dr(model);
    calInitSubstate2Dr(model, SQ.Sz, 0);
    calInitSubstate2Dr(model, SQ.Slt, 0);
    calInitSubstate2Dr(model, SQ.St, 0);
    calInitSubstate2Db(model, SQ.Mb, CAL_FALSE);
    calInitSubstate2Di(model, SQ.Mv, 0);
    calInitSubstate2Dr(model, SQ.Msl, 0);
    calInitSubstate2Dr(model, SQ.Sz_t0, 0);
    for (int q = 0; q < SCI_NF; q++) {
        SQ.f[q] = calAddSubstate2Dr(model);
        calInitSubstate2Dr(model, SQ.f[q], 0);
    }
    calAddElementaryProcess2D(model, sciara_vents_emission);
    calAddElementaryProcess2D(model, sciara_empirical_flows);
    calAddElementaryProcess2D(model, sciara_width_update);
    calAddElementaryProcess2D(model, sciara_update_temperature);
    if (ac)
        calAddElementaryProcess2D(model, sciara_remove_active_cells);

    /* loadConfiguration's effect: Sz (both layers) and Sz_t0 = DEM; thickness
     * and temperature maps when given (io.cpp:226-240, 370-398) */
    calSync2D(model);
    const size_t bytes = sizeof(double) * (size_t)rows * cols;
    memcpy(SQ.Sz->current, z0, bytes);
    memcpy(SQ.Sz->next, z0, bytes);
    memcpy(SQ.Sz_t0->current, z0, bytes);
    if (slt0) {
        memcpy(SQ.Slt->current, slt0, bytes);
        memcpy(SQ.Slt->next, slt0, bytes);
    }
    if (st0) {
        memcpy(SQ.St->current, st0, bytes);
        memcpy(SQ.St->next, st0, bytes);
    }
    calMarkHostDirty2D(model);

    struct CALRun2D* run = calRunDef2D(model, 1, max_steps, CAL_UPDATE_IMPLICIT);
    sci_run = run;
    calRunAddInitFunc2D(run, sciara_init);
    calRunAddSteeringFunc2D(run, sciara_steering);
    calRunAddStopConditionFunc2D(run, sciara_stop);
    calRunSetGraph2D(run, graph ? CAL_TRUE : CAL_FALSE);

    cudaStream_t s = (cudaStream_t)calGetStream2D(model);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    calRunInitSimulation2D(run);
    cudaEventRecord(e0, s);
    int done = 0;
    for (run->step = run->initial_step; run->step <= run->final_step || run->final_step == CAL_RUN_LOOP;
         run->step++) {
        done++;
        if (!calRunCAStep2D(run))
            break;
    }
    cudaEventRecord(e1, s);
    calRunFinalizeSimulation2D(run);
    calSync2D(model);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    if (ms)
        *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (steps_done)
        *steps_done = done;
    if (z_out)
        memcpy(z_out, SQ.Sz->current, bytes);
    if (slt_out)
        memcpy(slt_out, SQ.Slt->current, bytes);
    if (st_out)
        memcpy(st_out, SQ.St->current, bytes);
    if (msl_out)
        memcpy(msl_out, SQ.Msl->current, bytes);
    if (n_active)
        *n_active = ac ? model->A.size_current : 0;
    if (cells_out && ac && model->A.cells)
        memcpy(cells_out, model->A.cells, sizeof(int) * 2 * (size_t)model->A.size_current);
    const int err = calGetLastError();
    sci_run = nullptr;
    calRunFinalize2D(run);
    calFinalize2D(model);
    return err;
}
