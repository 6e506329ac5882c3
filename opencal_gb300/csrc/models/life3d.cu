/*
 * life3d.cu -- the reference's 3D Life example on the C API:
 * OpenCAL/examples/cal_life3D-glut/source/life3D.cpp:61-83 (one CALbyte
 * substate, 3D Moore or von Neumann neighbourhood, survive / birth bounds as
 * arguments), as a device elementary process driven by calRun3D.
 */
#include "opencal/cal3D.h"
#include "opencal/cal3DRun.h"

static int finish3d(struct CALModel3D* ca, struct CALRun3D* run)
{
    int err = calGetLastError();
    calRunFinalize3D(run);
    calFinalize3D(ca);
    return err;
}

__managed__ struct CALSubstate3Db* L3;
__managed__ int L3rule[4];

CAL_ELEMENTARY_PROCESS_3D(life3d_rule)(struct CALModel3D* ca, int i, int j, int k)
{
    int sum = 0, n;
    CALbyte alive = calGet3Db(ca, L3, i, j, k);
    CALbyte nextState = alive;
    for (n = 0; n < ca->sizeof_X; n++)
        sum += calGetX3Db(ca, L3, i, j, k, n);
    if (alive && (sum < L3rule[0] || sum > L3rule[1]))
        nextState = 0;
    else if (!alive && (sum >= L3rule[2] && sum <= L3rule[3]))
        nextState = 1;
    calSet3Db(ca, L3, i, j, k, nextState);
}

extern "C" int cal_life3d_run(int rows, int cols, int slices, int nbhd, int toroidal, int steps, int r1, int r2,
                              int r3, int r4, const unsigned char* s0, unsigned char* s_out, int graph)
{
    calClearError();
    struct CALModel3D* ca = calCADef3D(rows, cols, slices, (enum CALNeighborhood3D)nbhd,
                                       toroidal ? CAL_SPACE_TOROIDAL : CAL_SPACE_FLAT, CAL_NO_OPT);
    if (!ca)
        return calGetLastError();
    struct CALRun3D* run = calRunDef3D(ca, 1, steps, CAL_UPDATE_IMPLICIT);
    L3rule[0] = r1;
    L3rule[1] = r2;
    L3rule[2] = r3;
    L3rule[3] = r4;
    calAddElementaryProcess3D(ca, life3d_rule);
    L3 = calAddSubstate3Db(ca);
    const long long n = (long long)rows * cols * slices;
    for (long long c = 0; c < n; c++)
        L3->current[c] = L3->next[c] = (CALbyte)s0[c];
    calMarkHostDirty3D(ca);
    calRunSetGraph3D(run, graph ? CAL_TRUE : CAL_FALSE);
    if (steps > 0)
        calRun3D(run);
    calSync3D(ca);
    for (long long c = 0; c < n; c++)
        s_out[c] = (unsigned char)L3->current[c];
    return finish3d(ca, run);
}

