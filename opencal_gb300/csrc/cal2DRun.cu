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
    long rec_epoch = 0; /* the grid's invalidation epoch when the step was recorded */
    /* the grid's invalidation epoch after the last step run launch by launch:
     * a step is recorded only once one step has run that way since the last
     * invalidation, because the first step after one takes one-off host
     * decisions (a substate filled whole before its fills go tile by tile,
     * the skipping bitmaps re-armed) that a replay would repeat every step */
    long eager_epoch = -1;
    CALStopLaunchFunc2D dev_stop = nullptr; /* device stop condition */
    int* d_flag = nullptr;                  /* its decision, for the step-by-step fallback */
    int device_loop_used = 0;
};

bool cal_internal_desc2D(struct CALModel2D* ca, CALDevModel2D* d);
bool cal_prepare_skipping2D(struct CALModel2D* ca);

/* ======================= device stop conditions ========================= */

#define CAL_STOP_REGISTRY_MAX 1024
static CALStopFunc2D g_stop_host[CAL_STOP_REGISTRY_MAX];
static CALStopLaunchFunc2D g_stop_launch[CAL_STOP_REGISTRY_MAX];
static int g_stop_n;

extern "C" int calRegisterDeviceStopCondition2D(CALStopFunc2D host_name, CALStopLaunchFunc2D launch, const char* name)
{
    (void)name;
    for (int r = 0; r < g_stop_n; r++)
        if (g_stop_host[r] == host_name) {
            g_stop_launch[r] = launch;
            return 1;
        }
    if (g_stop_n >= CAL_STOP_REGISTRY_MAX)
        return 0;
    g_stop_host[g_stop_n] = host_name;
    g_stop_launch[g_stop_n] = launch;
    g_stop_n++;
    return 1;
}

/* the condition of a run without a device stop condition: only the final step ends it */
static __device__ CALbyte cal_never_stop(struct CALModel2D*) { return CAL_FALSE; }

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
    /* a new run: pure processes run on every tile again (their parameters
     * may have changed between runs); done here, after the init, so that a
     * first step recorded as a graph does not record the re-arming */
    G(sim->ca2D).nrun = -1;
    cal_prepare_skipping2D(sim->ca2D);
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
    cal_prepare_skipping2D(sim->ca2D); /* any re-arming before the recording, not in it */
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
    gr->rec_epoch = g.inval_epoch;
    return cal::cuda_ok(cudaGraphLaunch(exec, g.stream), "graph launch");
}

extern "C" CALbyte calRunCAStep2D(struct CALRun2D* sim)
{
    CALGpuRun2D* gr = sim->gpu;
    cal::CalGrid& g = G(sim->ca2D);
    bool done = false;
    if (gr && gr->graph_enabled && !gr->graph_failed) {
        if (gr->exec && gr->rec_epoch != g.inval_epoch) {
            /* host-side events since the recording (host writes, copies into
             * a substate, handed-out device pointers) invalidated what it
             * assumed: record the step again */
            cudaGraphExecDestroy(gr->exec);
            gr->exec = nullptr;
            if (gr->graph)
                cudaGraphDestroy(gr->graph);
            gr->graph = nullptr;
        }
        if (gr->exec) {
            done = cal::cuda_ok(cudaGraphLaunch(gr->exec, g.stream), "graph launch");
            if (done) {
                gr->replays++;
                g.device_wrote_all();
            }
        } else if (gr->eager_epoch == g.inval_epoch) {
            done = capture_step(sim);
        }
    }
    if (!done) {
        step_work(sim);
        if (gr)
            gr->eager_epoch = g.inval_epoch;
    }
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
        if (sim->gpu->d_flag)
            cudaFree(sim->gpu->d_flag);
        delete sim->gpu;
    }
    free(sim);
}

extern "C" void calRunAddDeviceStopConditionFunc2D(struct CALRun2D* sim, CALbyte (*stop)(struct CALModel2D*))
{
    for (int r = 0; r < g_stop_n; r++)
        if (g_stop_host[r] == stop) {
            sim->gpu->dev_stop = g_stop_launch[r];
            return;
        }
    cal::set_error(CAL_ERROR_NOT_A_DEVICE_PROCESS,
                   "calRunAddDeviceStopConditionFunc2D: not a device stop condition (CAL_DEVICE_STOP_CONDITION_2D)");
}

/* record [step; stop] as the body of a conditional WHILE node and run it;
 * false (with nothing executed) when the step cannot be recorded */
static bool device_loop(struct CALRun2D* sim, CALStopLaunchFunc2D stop, int have_steps)
{
    CALGpuRun2D* gr = sim->gpu;
    cal::CalGrid& g = G(sim->ca2D);
    if (!g.repair_all_stale() || !g.to_device_all())
        return false;
    CALDevModel2D d;
    if (!cal_internal_desc2D(sim->ca2D, &d))
        return false;
    cudaGraph_t graph = nullptr;
    cudaGraphConditionalHandle handle;
    if (!cal::cuda_ok(cudaGraphCreate(&graph, 0), "cudaGraphCreate"))
        return false;
    if (!cal::cuda_ok(cudaGraphConditionalHandleCreate(&handle, graph, have_steps ? 1u : 0u,
                                                       cudaGraphCondAssignDefault), "conditional handle")) {
        cudaGraphDestroy(graph);
        return false;
    }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (!cal::cuda_ok(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp), "conditional node")) {
        cudaGraphDestroy(graph);
        return false;
    }
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cal_prepare_skipping2D(sim->ca2D); /* any re-arming before the recording, not in it */
    cal::GridState* before = new cal::GridState;
    g.save(before);
    const int transfers0 = g.transfers;
    const long swaps0 = g.swaps;
    calClearError();
    bool clean = cal::cuda_ok(cudaStreamBeginCaptureToGraph(g.stream, body, nullptr, nullptr, 0,
                                                            cudaStreamCaptureModeThreadLocal), "capture body");
    if (clean) {
        g.capturing = 1;
        step_work(sim);
        const int rc = stop(&d, (unsigned long long)handle, 1, sim->final_step, gr->d_flag, (void*)g.stream);
        g.capturing = 0;
        cudaGraph_t out = nullptr;
        const cudaError_t e = cudaStreamEndCapture(g.stream, &out);
        clean = rc == 0 && e == cudaSuccess && calGetLastError() == CAL_SUCCESS && g.transfers == transfers0 &&
                g.swaps == swaps0;
    }
    cudaGraphExec_t exec = nullptr;
    if (clean)
        clean = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
    if (!clean) {
        (void)cudaGetLastError();
        g.restore(before);
        delete before;
        cudaGraphDestroy(graph);
        calClearError();
        return false;
    }
    delete before;
    const bool ok = cal::cuda_ok(cudaGraphLaunch(exec, g.stream), "device loop launch");
    g.device_wrote_all();
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    return ok;
}

/* steps first..last (last == CAL_RUN_LOOP: until the stop condition) with
 * the loop on the device when possible; returns the step the loop ended on */
static int run_device_steps(struct CALRun2D* sim, int first, int last)
{
    CALGpuRun2D* gr = sim->gpu;
    cal::CalGrid& g = G(sim->ca2D);
    if (!gr->d_flag && !cal::cuda_ok(cudaMalloc(&gr->d_flag, sizeof(int)), "cudaMalloc stop flag"))
        return first;
    CALStopLaunchFunc2D stop = gr->dev_stop ? gr->dev_stop : cal_launch_stop2D<cal_never_stop>;
    const int have_steps = last == CAL_RUN_LOOP || first <= last;
    int step = first;
    gr->device_loop_used = 0;
    if (!have_steps)
        return step;
    const int words[2] = {step, 0}; /* step, "gave up at the step limit" */
    cal::cuda_ok(cudaMemcpyAsync(g.d_step, words, sizeof(words), cudaMemcpyHostToDevice, g.stream), "set step");
    g.sync();
    const int saved_final = sim->final_step;
    sim->final_step = last;
    bool settled = gr->eager_epoch == g.inval_epoch;
    bool more = true;
    if (!sim->stopCondition && !settled) {
        /* one step launch by launch before the loop is recorded (see
         * CALGpuRun2D::eager_epoch), with the device's decision */
        calClearError();
        step_work(sim);
        gr->eager_epoch = g.inval_epoch;
        CALDevModel2D d;
        int again = 0;
        more = calGetLastError() == CAL_SUCCESS && cal::cuda_ok(cudaGetLastError(), "step launches") &&
               cal_internal_desc2D(sim->ca2D, &d) && stop(&d, 0ULL, 0, last, gr->d_flag, (void*)g.stream) == 0 &&
               cal::cuda_ok(cudaMemcpyAsync(&again, gr->d_flag, sizeof(int), cudaMemcpyDeviceToHost, g.stream),
                            "read stop flag") &&
               g.sync() && again;
        settled = true;
    }
    if (!more) {
        /* the run ended with that step (or it failed: the error is set) */
    } else if (!sim->stopCondition && device_loop(sim, stop, have_steps)) {
        gr->device_loop_used = 1;
    } else {
        /* one step at a time; the device condition decides, and the host
         * counts the steps too, so that the loop ends even when a failed
         * launch leaves the device's decision stale: at most last - first + 1
         * steps (CAL_DEVICE_LOOP_MAX_STEP with CAL_RUN_LOOP), and at the
         * first error of a step's launches */
        const long long host_limit =
            last == CAL_RUN_LOOP ? (long long)CAL_DEVICE_LOOP_MAX_STEP : (long long)last - first + 1;
        for (long long taken = 0;; taken++) {
            if (taken >= host_limit) {
                cal::set_error(CAL_ERROR_INVALID_ARGUMENT, "device-driven run: host step count reached its limit");
                break;
            }
            calClearError();
            step_work(sim);
            if (calGetLastError() != CAL_SUCCESS || !cal::cuda_ok(cudaGetLastError(), "step launches"))
                break;
            CALDevModel2D d;
            if (!cal_internal_desc2D(sim->ca2D, &d))
                break;
            if (stop(&d, 0ULL, 0, last, gr->d_flag, (void*)g.stream) != 0)
                break;
            int again = 0;
            if (!cal::cuda_ok(cudaMemcpyAsync(&again, gr->d_flag, sizeof(int), cudaMemcpyDeviceToHost, g.stream),
                              "read stop flag") || !g.sync())
                break;
            if (sim->stopCondition) {
                cal::cuda_ok(cudaMemcpyAsync(&sim->step, g.d_step, sizeof(int), cudaMemcpyDeviceToHost, g.stream),
                             "read step");
                g.sync();
                if (sim->stopCondition(sim->ca2D))
                    break;
            }
            if (!again)
                break;
        }
    }
    sim->final_step = saved_final;
    int out[2] = {step, 0};
    cal::cuda_ok(cudaMemcpyAsync(out, g.d_step, sizeof(out), cudaMemcpyDeviceToHost, g.stream), "read step");
    g.sync();
    if (out[1])
        cal::set_error(CAL_ERROR_INVALID_ARGUMENT, "device-driven run stopped at the step limit (CAL_DEVICE_LOOP_MAX_STEP)");
    return out[0];
}

extern "C" void calRunDevice2D(struct CALRun2D* sim)
{
    calRunInitSimulation2D(sim);
    sim->step = run_device_steps(sim, sim->initial_step, sim->final_step);
    calRunFinalizeSimulation2D(sim);
    G(sim->ca2D).sync();
}

extern "C" int calRunDeviceSteps2D(struct CALRun2D* sim, int first_step, int last_step)
{
    sim->step = run_device_steps(sim, first_step, last_step);
    return sim->step;
}

extern "C" int calRunDeviceLoopUsed2D(struct CALRun2D* sim)
{
    return (sim && sim->gpu) ? sim->gpu->device_loop_used : 0;
}

extern "C" void calRunSetGraph2D(struct CALRun2D* sim, CALbyte enable)
{
    if (!sim || !sim->gpu)
        return;
    if (!enable && sim->gpu->exec) {
        /* a recorded step is dropped: the next enabled step records anew */
        cudaGraphExecDestroy(sim->gpu->exec);
        sim->gpu->exec = nullptr;
        if (sim->gpu->graph)
            cudaGraphDestroy(sim->gpu->graph);
        sim->gpu->graph = nullptr;
    }
    sim->gpu->graph_enabled = enable != 0;
}

extern "C" long calRunGraphReplays2D(struct CALRun2D* sim)
{
    return (sim && sim->gpu) ? sim->gpu->replays : 0;
}
