/*
 * cal2DRun.h -- simulation run control for 2D models.
 *
 * Drop-in for OpenCAL-OMP/include/cal2DRun.h: the same CALRun2D fields and
 * functions.  Callbacks are host functions, as in the reference; the work
 * they queue through this library (elementary processes, substate
 * initialisation, updates) runs asynchronously on the model's CUDA stream,
 * so a run of N steps is N rounds of kernel launches with no host/device
 * synchronisation unless a callback reads device data through the host
 * accessors.
 *
 * Graph mode (calRunSetGraph2D): the first step is recorded as a CUDA graph
 * and later steps replay it.  Only valid when the callbacks queue the same
 * device work every step (e.g. SCIDDICA-T's steering); the stop condition is
 * still evaluated on the host after every step.
 */
#ifndef cal2DRun_h
#define cal2DRun_h

#include "cal2D.h"

struct CALGpuRun2D;

/* cal2DRun.h:21-33 (+ gpu) */
struct CALRun2D {
    struct CALModel2D* ca2D;
    int step;
    int initial_step;
    int final_step;
    enum CALUpdateMode UPDATE_MODE;
    void (*init)(struct CALModel2D*);
    void (*globalTransition)(struct CALModel2D*);
    void (*steering)(struct CALModel2D*);
    CALbyte (*stopCondition)(struct CALModel2D*);
    void (*finalize)(struct CALModel2D*);
    struct CALGpuRun2D* gpu;
};

#ifdef __cplusplus
extern "C" {
#endif

struct CALRun2D* calRunDef2D(struct CALModel2D* ca2D, int initial_step, int final_step,
                             enum CALUpdateMode UPDATE_MODE);                                       /* cal2DRun.h:42 */
void calRunAddInitFunc2D(struct CALRun2D* simulation, void (*init)(struct CALModel2D*));             /* cal2DRun.h:52 */
void calRunAddGlobalTransitionFunc2D(struct CALRun2D* simulation, void (*globalTransition)(struct CALModel2D*)); /* :59 */
void calRunAddSteeringFunc2D(struct CALRun2D* simulation, void (*steering)(struct CALModel2D*));     /* cal2DRun.h:65 */
void calRunAddStopConditionFunc2D(struct CALRun2D* simulation, CALbyte (*stopCondition)(struct CALModel2D*)); /* :71 */
void calRunAddFinalizeFunc2D(struct CALRun2D* simulation, void (*finalize)(struct CALModel2D*));     /* cal2DRun.h:77 */
void calRunInitSimulation2D(struct CALRun2D* simulation);                                            /* cal2DRun.h:83 */
CALbyte calRunCAStep2D(struct CALRun2D* simulation);                                                 /* cal2DRun.h:90 */
void calRunFinalizeSimulation2D(struct CALRun2D* simulation);                                        /* cal2DRun.h:95 */
void calRun2D(struct CALRun2D* simulation);                                                          /* cal2DRun.h:101 */
void calRunFinalize2D(struct CALRun2D* cal2DRun);                                                    /* cal2DRun.h:108 */

/* ---- opencal-gb300 additions --------------------------------------- */
/* Record the step as a CUDA graph on first use and replay it afterwards.
 * Disabling drops a recorded step, so that a step whose launches change
 * (new parameters baked into its kernels) is recorded again when re-enabled. */
void calRunSetGraph2D(struct CALRun2D* simulation, CALbyte enable);
/* Number of steps whose device work was replayed from the recorded graph. */
long calRunGraphReplays2D(struct CALRun2D* simulation);
/* A stop condition evaluated on the GPU after every step (a function defined
 * with CAL_DEVICE_STOP_CONDITION_2D; on the device it reads the step with
 * calRunGetStep2D).  Used by calRunDevice2D. */
void calRunAddDeviceStopConditionFunc2D(struct CALRun2D* simulation, CALbyte (*stopCondition)(struct CALModel2D*));
/* calRun2D with the step loop on the GPU: init, then ONE graph launch whose
 * conditional WHILE node repeats [step; device stop condition] until the
 * stop condition holds or the final step is done, then finalize.  Needs the
 * step's device work to be recordable (see calRunSetGraph2D) and no host
 * stop condition; otherwise it runs the steps one by one, still deciding
 * with the device stop condition.  On return CALRun2D::step is the step the
 * loop ended on, as after calRun2D. */
void calRunDevice2D(struct CALRun2D* simulation);
/* The device-driven loop alone (no init/finalize) over steps first..last
 * (last = CAL_RUN_LOOP: until the device stop condition); returns the step
 * it ended on (also stored in CALRun2D::step). */
int calRunDeviceSteps2D(struct CALRun2D* simulation, int first_step, int last_step);
/* 1 if the last calRunDevice2D ran as a single device loop, 0 if it fell
 * back to one launch sequence per step. */
int calRunDeviceLoopUsed2D(struct CALRun2D* simulation);

#ifdef __cplusplus
}
#endif

#endif
