/*
 * sciddicaT_unsafe.cu -- SCIDDICA-T in the reference's unsafe form:
 * OpenCAL/examples/cal_sciddicaT-unsafe/source/sciddicaT.c:35-107.  The
 * outflows are moved at once into next(h) of the cell and of the receiver
 * (calAddNext2Dr / calAddNextX2Dr: device atomics here, the reference's
 * get-then-set under a lock), one elementary process per step.
 */
#include <string.h>

#include "opencal/cal2D.h"
#include "opencal/cal2DRun.h"
#include "opencal/cal2DUnsafe.h"

static int finish2d(struct CALModel2D* ca, struct CALRun2D* run)
{
    int err = calGetLastError();
    calRunFinalize2D(run);
    calFinalize2D(ca);
    return err;
}

struct SdtuQ {
    struct CALSubstate2Dr* z;
    struct CALSubstate2Dr* h;
    double r, eps;
};
__managed__ struct SdtuQ SU;

CAL_ELEMENTARY_PROCESS_2D(sciddicaT_unsafe_transition)(struct CALModel2D* ca, int i, int j)
{
    bool out[5] = {false, false, false, false, false};
    double u[5];
    const double m = calGet2Dr(ca, SU.h, i, j) - SU.eps;
    u[0] = calGet2Dr(ca, SU.z, i, j) + SU.eps;
    for (int n = 1; n < ca->sizeof_X; n++)
        u[n] = calGetX2Dr(ca, SU.z, i, j, n) + calGetX2Dr(ca, SU.h, i, j, n);
    double avg;
    bool again;
    do {
        again = false;
        avg = m;
        int count = 0;
        for (int n = 0; n < ca->sizeof_X; n++)
            if (!out[n]) {
                avg += u[n];
                count++;
            }
        if (count != 0)
            avg /= count;
        for (int n = 0; n < ca->sizeof_X; n++)
            if (avg <= u[n] && !out[n]) {
                out[n] = true;
                again = true;
            }
    } while (again);
    for (int n = 1; n < ca->sizeof_X; n++)
        if (!out[n]) {
            const double f = (avg - u[n]) * SU.r;
            calAddNext2Dr(ca, SU.h, i, j, -f);
            calAddNextX2Dr(ca, SU.h, i, j, n, f);
        }
}

static void sciddicaT_unsafe_init(struct CALModel2D* ca)
{
    for (int i = 0; i < ca->rows; i++)
        for (int j = 0; j < ca->columns; j++) {
            const double h = calGet2Dr(ca, SU.h, i, j);
            if (h > 0.0)
                calSetCurrent2Dr(ca, SU.z, i, j, calGet2Dr(ca, SU.z, i, j) - h);
        }
}

extern "C" int cal_sciddicaT_unsafe_run(int rows, int cols, int toroidal, int steps, double p_r, double p_eps,
                                        const double* z0, const double* h0, double* z_out, double* h_out, int graph)
{
    calClearError();
    struct CALModel2D* ca = calCADef2D(rows, cols, CAL_VON_NEUMANN_NEIGHBORHOOD_2D,
                                       toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    if (!ca)
        return calGetLastError();
    calSetUnsafe2D(ca);
    struct CALRun2D* run = calRunDef2D(ca, 1, steps, CAL_UPDATE_IMPLICIT);
    calAddElementaryProcess2D(ca, sciddicaT_unsafe_transition);
    SU.z = calAddSubstate2Dr(ca);
    SU.h = calAddSubstate2Dr(ca);
    SU.r = p_r;
    SU.eps = p_eps;
    const size_t bytes = sizeof(double) * (size_t)rows * cols;
    memcpy(SU.z->current, z0, bytes);
    memcpy(SU.z->next, z0, bytes);
    memcpy(SU.h->current, h0, bytes);
    memcpy(SU.h->next, h0, bytes);
    calMarkHostDirty2D(ca);
    calRunAddInitFunc2D(run, sciddicaT_unsafe_init);
    calRunSetGraph2D(run, graph ? CAL_TRUE : CAL_FALSE);
    if (steps > 0)
        calRun2D(run);
    else
        calRunInitSimulation2D(run);
    calSync2D(ca);
    memcpy(z_out, SU.z->current, bytes);
    memcpy(h_out, SU.h->current, bytes);
    return finish2d(ca, run);
}
