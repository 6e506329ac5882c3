/*
 * mbusu_headless_main.c -- headless driver for the reference's mbusu example
 * (OpenCAL/examples/cal_mbusu-glut/source/mbusu.c, compiled unmodified from
 * its sources): mbusu_gui.c's idle loop (step++, calRunCAStep3D until the
 * stop condition) without GLUT, optionally cut after a given number of
 * steps, and the final state written as raw little-endian doubles.
 * Test infrastructure only.
 *
 *   mbusu_ref <steps: 0 = until the stop condition, < 0 = none> <output file>
 * writes teta, moist_cont, psi, k, h, dqdh, convergence, moist_diff (each
 * rows*cols*slices doubles, slice-major), then the step reached, delta_t
 * and delta_t_cum as three doubles.  The example itself appends to
 * ./deltat.txt every step and writes ./ris10g.txt when it stops.
 */
#include <stdio.h>
#include <stdlib.h>

#include "mbusu.h"

extern float delta_t, delta_t_cum;

int main(int argc, char** argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s steps out\n", argv[0]);
        return 2;
    }
    const int steps = atoi(argv[1]);
    mbusuCADef();
    CALbyte again = CAL_TRUE;
    int done = 0;
    while (steps >= 0 && again && (steps == 0 || done < steps)) {
        mbusuSimulation->step++;
        again = calRunCAStep3D(mbusuSimulation);
        done++;
    }
    const size_t n = (size_t)mbusu->rows * mbusu->columns * mbusu->slices;
    FILE* f = fopen(argv[2], "wb");
    if (!f)
        return 1;
    struct CALSubstate3Dr* q[8] = {Q.teta, Q.moist_cont, Q.psi, Q.k, Q.h, Q.dqdh, Q.convergence, Q.moist_diff};
    for (int s = 0; s < 8; s++)
        fwrite(q[s]->current, sizeof(double), n, f);
    double tail[3] = {(double)mbusuSimulation->step, (double)delta_t, (double)delta_t_cum};
    fwrite(tail, sizeof(double), 3, f);
    fclose(f);
    mbusuExit();
    return 0;
}
