/*
 * ac_headless_main.c -- headless stand-in for the GLUT idle loop of the
 * reference's active-cells SCIDDICA-T example
 * (OpenCAL/examples/cal_sciddicaT-activecells-glut/source/gui.c:85-112):
 * step the run with calRunCAStep2D until the stop condition fires, then save.
 * The example's own sciddicaT.c (compiled unmodified) provides the model.
 * Test infrastructure only.
 */
#include <stdio.h>

#include "sciddicaT.h"

extern struct CALRun2D* sciddicaTsimulation;

int main(void)
{
    sciddicaTCADef();
    for (;;) {
        sciddicaTsimulation->step++;
        if (!calRunCAStep2D(sciddicaTsimulation))
            break;
    }
    sciddicaTSaveConfig();
    printf("steps %d active %d\n", sciddicaTsimulation->step, sciddicaTsimulation->ca2D->A.size_current);
    return 0;
}
