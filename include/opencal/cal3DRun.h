/*
 * cal3DRun.h -- simulation run control for 3D models.
 *
 * Drop-in for OpenCAL-OMP/include/cal3DRun.h: the same CALRun3D fields and
 * functions.  Callbacks are host functions, as in the reference; the work
 * they queue through this library (elementary processes, substate
 * initialisation, updates) runs asynchronously on the model's CUDA stream,
 * so a run of N steps is N rounds of kernel launches with no host/device
 * synchronisation unless a callback reads device data through the host
 * accessors.
 *
 * Graph mode (calRunSetGraph3D): the first step is recorded as a CUDA graph
 * and later steps replay it.  Only valid when the callbacks queue the same
 * device work every step (e.g. SCIDDICA-T's steering); the stop condition is
 * still evaluated on the host after every step.
 */
#ifndef cal3DRun_h
#define cal3DRun_h

#include "cal3D.h"

struct CALGpuRun3D;

/* cal3DRun.h:21-33 (+ gpu) */
struct CALRun3D {
    struct CALModel3D* ca3D;
    int step;
    int initial_step;
    int final_step;
    enum CALUpdateMode UPDATE_MODE;
    void (*init)(struct CALModel3D*);
    void (*globalTransition)(struct CALModel3D*);
    void (*steering)(struct CALModel3D*);
    CALbyte (*stopCondition)(struct CALModel3D*);
    void (*finalize)(struct CALModel3D*);
    struct CALGpuRun3D* gpu;
};

#ifdef __cplusplus
extern "C" {
#endif

struct CALRun3D* calRunDef3D(struct CALModel3D* ca3D, int initial_step, int final_step,
                             enum CALUpdateMode UPDATE_MODE);                                       /* cal3DRun.h:42 */
void calRunAddInitFunc3D(struct CALRun3D* simulation, void (*init)(struct CALModel3D*));             /* cal3DRun.h:52 */
void calRunAddGlobalTransitionFunc3D(struct CALRun3D* simulation, void (*globalTransition)(struct CALModel3D*)); /* :59 */
void calRunAddSteeringFunc3D(struct CALRun3D* simulation, void (*steering)(struct CALModel3D*));     /* cal3DRun.h:65 */
void calRunAddStopConditionFunc3D(struct CALRun3D* simulation, CALbyte (*stopCondition)(struct CALModel3D*)); /* :71 */
void calRunAddFinalizeFunc3D(struct CALRun3D* simulation, void (*finalize)(struct CALModel3D*));     /* cal3DRun.h:77 */
void calRunInitSimulation3D(struct CALRun3D* simulation);                                            /* cal3DRun.h:81 */
CALbyte calRunCAStep3D(struct CALRun3D* simulation);                                                 /* cal3DRun.h:87 */
void calRunFinalizeSimulation3D(struct CALRun3D* simulation);                                        /* cal3DRun.h:90 */
void calRun3D(struct CALRun3D* simulation);                                                          /* cal3DRun.h:96 */
void calRunFinalize3D(struct CALRun3D* cal3DRun);                                                    /* cal3DRun.h:103 */

/* ---- opencal-gb300 additions --------------------------------------- */
/* Record the step as a CUDA graph on first use and replay it afterwards.
 * Disabling drops a recorded step, so that a step whose launches change
 * (new parameters baked into its kernels) is recorded again when re-enabled. */
void calRunSetGraph3D(struct CALRun3D* simulation, CALbyte enable);
/* Number of steps whose device work was replayed from the recorded graph. */
long calRunGraphReplays3D(struct CALRun3D* simulation);
/* A stop condition evaluated on the GPU after every step (a function defined
 * with CAL_DEVICE_STOP_CONDITION_3D; on the device it reads the step with
 * calRunGetStep3D).  Used by calRunDevice3D. */
void calRunAddDeviceStopConditionFunc3D(struct CALRun3D* simulation, CALbyte (*stopCondition)(struct CALModel3D*));
/* calRun3D with the step loop on the GPU: init, then ONE graph launch whose
 * conditional WHILE node repeats [step; device stop condition] until the
 * stop condition holds or the final step is done, then finalize.  Needs the
 * step's device work to be recordable (see calRunSetGraph3D) and no host
 * stop condition; otherwise it runs the steps one by one, still deciding
 * with the device stop condition.  On return CALRun3D::step is the step the
 * loop ended on, as after calRun3D. */
void calRunDevice3D(struct CALRun3D* simulation);
/* The device-driven loop alone (no init/finalize) over steps first..last
 * (last = CAL_RUN_LOOP: until the device stop condition); returns the step
 * it ended on (also stored in CALRun3D::step). */
int calRunDeviceSteps3D(struct CALRun3D* simulation, int first_step, int last_step);
/* 1 if the last calRunDevice3D ran as a single device loop, 0 if it fell
 * back to one launch sequence per step. */
int calRunDeviceLoopUsed3D(struct CALRun3D* simulation);

#ifdef __cplusplus
}
#endif

#endif
