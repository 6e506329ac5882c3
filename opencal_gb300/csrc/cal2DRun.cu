/*
 * cal2DRun.cu -- run control (include/opencal/cal2DRun.h).
 *
 * Restates OpenCAL-OMP/source/cal2DRun.c:16-147: init (+ implicit update),
 * steps initial..final inclusive or until the stop condition (final_step ==
 * CAL_RUN_LOOP loops), each step = global transition (+ implicit update
 * after a custom one), steering (+ implicit update), stop condition; then
 * finalize (+ implicit update).
 *
 * Graph mode: the device work one step queues (processes, updates, fills,
 * compactions) is recorded once with stream capture and replayed with
 * cudaGraphLaunch afterwards, which removes the per-kernel launch cost from
 * the host loop.  A step whose recording needed host<->device copies, a host
 * read of device data or a pointer swap cannot be replayed; graph mode then
 * turns itself off and the run continues eagerly.
 */
#define CAL_BUILDING_LIBRARY
#include <stdlib.h>

#include "cal_model_internal.cuh"
#include "opencal/cal2DRun.h"

struct CALGpuRun2D {
    bool graph_enabled = false;
    bool graph_failed = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long replays = 0;
};

static inline cal::CalGrid& G(struct CALModel2D* ca) { return ca->gpu->g; }

extern "C" struct CALRun2D* calRunDef2D(struct CALModel2D* ca2D, int initial_step, int final_step,
                                        enum CALUpdateMode UPDATE_MODE)
{
    struct CALRun2D* sim = (struct CALRun2D*)calloc(1, sizeof(struct CALRun2D));
    if (!sim) {
        cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "calRunDef2D");
        return nullptr;
    }
    sim->ca2D = ca2D;
    sim->step = 0;
    sim->initial_step = initial_step;
    sim->final_step = final_step;
    sim->UPDATE_MODE = UPDATE_MODE;
    sim->gpu = new (std::nothrow) CALGpuRun2D();
    return sim;
}

extern "C" void calRunAddInitFunc2D(struct CALRun2D* s, void (*f)(struct CALModel2D*)) { s->init = f; }
extern "C" void calRunAddGlobalTransitionFunc2D(struct CALRun2D* s, void (*f)(struct CALModel2D*)) { s->globalTransition = f; }
extern "C" void calRunAddSteeringFunc2D(struct CALRun2D* s, void (*f)(struct CALModel2D*)) { s->steering = f; }
extern "C" void calRunAddStopConditionFunc2D(struct CALRun2D* s, CALbyte (*f)(struct CALModel2D*)) { s->stopCondition = f; }
extern "C" void calRunAddFinalizeFunc2D(struct CALRun2D* s, void (*f)(struct CALModel2D*)) { s->finalize = f; }

extern "C" void calRunInitSimulation2D(struct CALRun2D* sim)
{
    if (sim->init) {
        sim->init(sim->ca2D);
        if (sim->UPDATE_MODE == CAL_UPDATE_IMPLICIT)
            calUpdate2D(sim->ca2D);
    }
}

/* the device work of one step (cal2DRun.c:88-105 without the stop test) */
static void step_work(struct CALRun2D* sim)
{
    if (sim->globalTransition) {
        sim->globalTransition(sim->ca2D);
        if (sim->UPDATE_MODE == CAL_UPDATE_IMPLICIT)
            calUpdate2D(sim->ca2D);
    } else {
        calGlobalTransitionFunction2D(sim->ca2D);
    }
    if (sim->steering) {
        sim->steering(sim->ca2D);
        if (sim->UPDATE_MODE == CAL_UPDATE_IMPLICIT)
            calUpdate2D(sim->ca2D);
    }
}

/* record one step as a graph; true when the step has been executed (by
 * launching the fresh graph) */
static bool capture_step(struct CALRun2D* sim)
{
    CALGpuRun2D* gr = sim->gpu;
    cal::CalGrid& g = G(sim->ca2D);
    if (!g.repair_all_stale() || !g.to_device_all())
        return false;
    const int transfers0 = g.transfers;
    const long swaps0 = g.swaps;
    cal::GridState* before = new cal::GridState;
    g.save(before);
    calClearError();
    if (!cal::cuda_ok(cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal), "begin capture")) {
        delete before;
        return false;
    }
    g.capturing = 1;
    step_work(sim);
    g.capturing = 0;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(g.stream, &graph);
    const bool clean = e == cudaSuccess && calGetLastError() == CAL_SUCCESS && g.transfers == transfers0 &&
                       g.swaps == swaps0 && graph != nullptr;
    if (!clean) {
        if (graph)
            cudaGraphDestroy(graph);
        /* nothing of the step ran: undo its host-side bookkeeping and drop
         * the error the abandoned recording left behind */
        (void)cudaGetLastError();
        g.restore(before);
        delete before;
        calClearError();
        gr->graph_failed = true;
        return false;
    }
    delete before;
    cudaGraphExec_t exec = nullptr;
    if (!cal::cuda_ok(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate")) {
        cudaGraphDestroy(graph);
        gr->graph_failed = true;
        return false;
    }
    gr->graph = graph;
    gr->exec = exec;
    return cal::cuda_ok(cudaGraphLaunch(exec, g.stream), "graph launch");
}

extern "C" CALbyte calRunCAStep2D(struct CALRun2D* sim)
{
    CALGpuRun2D* gr = sim->gpu;
    cal::CalGrid& g = G(sim->ca2D);
    bool done = false;
    if (gr && gr->graph_enabled && !gr->graph_failed) {
        if (gr->exec) {
            done = cal::cuda_ok(cudaGraphLaunch(gr->exec, g.stream), "graph launch");
            if (done) {
                gr->replays++;
                g.device_wrote_all();
            }
        } else {
            done = capture_step(sim);
        }
    }
    if (!done)
        step_work(sim);
    if (sim->stopCondition && sim->stopCondition(sim->ca2D))
        return CAL_FALSE;
    return CAL_TRUE;
}

extern "C" void calRunFinalizeSimulation2D(struct CALRun2D* sim)
{
    if (sim->finalize) {
        sim->finalize(sim->ca2D);
        if (sim->UPDATE_MODE == CAL_UPDATE_IMPLICIT)
            calUpdate2D(sim->ca2D);
    }
}

extern "C" void calRun2D(struct CALRun2D* sim)
{
    calRunInitSimulation2D(sim);
    for (sim->step = sim->initial_step; sim->step <= sim->final_step || sim->final_step == CAL_RUN_LOOP; sim->step++)
        if (!calRunCAStep2D(sim))
            break;
    calRunFinalizeSimulation2D(sim);
    G(sim->ca2D).sync();
}

extern "C" void calRunFinalize2D(struct CALRun2D* sim)
{
    if (!sim)
        return;
    if (sim->gpu) {
        if (sim->gpu->exec)
            cudaGraphExecDestroy(sim->gpu->exec);
        if (sim->gpu->graph)
            cudaGraphDestroy(sim->gpu->graph);
        delete sim->gpu;
    }
    free(sim);
}

extern "C" void calRunSetGraph2D(struct CALRun2D* sim, CALbyte enable)
{
    if (sim && sim->gpu)
        sim->gpu->graph_enabled = enable != 0;
}

extern "C" long calRunGraphReplays2D(struct CALRun2D* sim)
{
    return (sim && sim->gpu) ? sim->gpu->replays : 0;
}
