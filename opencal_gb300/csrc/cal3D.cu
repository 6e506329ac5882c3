/*
 * cal3D.cu -- the 3D C API (include/opencal/cal3D.h) on the shared engine.
 *
 * Reference behaviour restated (OpenCAL-OMP/source/cal3D.c):
 *   neighbourhoods VN (7) and Moore (27)      cal3D.c:29-105
 *   calCADef3D                                cal3D.c:205-260
 *   active cells add/remove/update (i,j,k)    cal3D.c:270-370
 *   substates, processes, init/update         cal3D.c:400-655
 *   apply (i, j, k loop), transition, update  cal3D.c:658-714
 *   accessors, layout k*rows*cols+i*cols+j    cal3D.c:720-860, cal3DBuffer.h:131-136
 */
#define CAL_BUILDING_LIBRARY
#include <stdlib.h>
#include <string.h>

#include "cal_model_internal.cuh"
#include "opencal/cal3DUnsafe.h"

using cal::CalGrid;

#define CAL_REGISTRY_MAX 4096
static CALCallbackFunc3D g_reg_host[CAL_REGISTRY_MAX];
static CALLaunchFunc3D g_reg_launch[CAL_REGISTRY_MAX];
static int g_reg_n;

extern "C" int calRegisterElementaryProcess3D(CALCallbackFunc3D host_name, CALLaunchFunc3D launch, const char* name)
{
    (void)name;
    for (int r = 0; r < g_reg_n; r++)
        if (g_reg_host[r] == host_name) {
            g_reg_launch[r] = launch;
            return 1;
        }
    if (g_reg_n >= CAL_REGISTRY_MAX)
        return 0;
    g_reg_host[g_reg_n] = host_name;
    g_reg_launch[g_reg_n] = launch;
    g_reg_n++;
    return 1;
}

static CALLaunchFunc3D find_launch(CALCallbackFunc3D f)
{
    for (int r = 0; r < g_reg_n; r++)
        if (g_reg_host[r] == f)
            return g_reg_launch[r];
    return nullptr;
}

extern "C" void calHostCallOfDeviceProcess3D(const char* name)
{
    cal::set_error(CAL_ERROR_NOT_A_DEVICE_PROCESS,
                   std::string("device elementary process '") + name + "' called as a host function");
}

static inline CalGrid& G(struct CALModel3D* ca) { return ca->gpu->g; }

template <typename Q>
static inline int slot_of(struct CALModel3D* ca, int type, Q* q)
{
    return (int)(((char*)q - (char*)G(ca).pool[type]) / 32);
}

static bool neighbor(const struct CALModel3D* ca, int i, int j, int k, int n, int* oi, int* oj, int* ok)
{
    int a = i + ca->X[n].i, b = j + ca->X[n].j, c = k + ca->X[n].k;
    if (ca->T == CAL_SPACE_TOROIDAL) {
        a = calGetToroidalX(a, ca->rows);
        b = calGetToroidalX(b, ca->columns);
        c = calGetToroidalX(c, ca->slices);
    } else if (a < 0 || a >= ca->rows || b < 0 || b >= ca->columns || c < 0 || c >= ca->slices) {
        return false;
    }
    *oi = a;
    *oj = b;
    *ok = c;
    return true;
}

static bool upload_X(struct CALModel3D* ca)
{
    CALGpuModel3D* gm = ca->gpu;
    const int len = ca->sizeof_X;
    if (gm->d_X_len == len || len == 0)
        return true;
    if (gm->g.capturing) {
        cal::set_error(CAL_ERROR_NOT_CAPTURABLE, "neighbourhood changed during graph capture");
        return false;
    }
    if (!cal::cuda_ok(cudaMemcpy(gm->d_X, ca->X, sizeof(struct CALCell3D) * len, cudaMemcpyHostToDevice), "upload X"))
        return false;
    gm->d_X_len = len;
    return true;
}

static bool build_desc(struct CALModel3D* ca, CALDevModel3D* d)
{
    CalGrid& g = G(ca);
    memset(d, 0, sizeof(*d));
    d->model = *ca;
    d->model.gpu = nullptr;
    d->model.pQb_array = nullptr;
    d->model.pQi_array = nullptr;
    d->model.pQr_array = nullptr;
    d->model.elementary_processes = nullptr;
    d->model.A.size_next = nullptr;
    d->model.A.flags = (CALbyte*)g.d_flags;
    d->model.A.cells = (struct CALCell3D*)g.d_cells;
    if (ca->sizeof_X > CAL_MAX_NEIGHBORS) {
        cal::set_error(CAL_ERROR_LIMIT, "neighbourhood larger than CAL_MAX_NEIGHBORS");
        return false;
    }
    if (!upload_X(ca))
        return false;
    d->model.X = ca->gpu->d_X;
    for (int t = 0; t < CAL_NTYPES; t++) {
        d->pool[t] = (unsigned long long)(uintptr_t)g.pool[t];
        for (int s = 0; s < g.nslot[t]; s++) {
            d->cur[t][s] = g.sub[t][s].layer[0].dev;
            d->nxt[t][s] = g.sub[t][s].single ? nullptr : g.sub[t][s].layer[1].dev;
        }
    }
    d->dirty = g.d_dirty;
    d->step = g.d_step;
    d->flags = (CALbyte*)g.d_flags;
    d->cells = (struct CALCell3D*)g.d_cells;
    d->count = g.d_count;
    d->rows = ca->rows;
    d->cols = ca->columns;
    d->slices = ca->slices;
    d->toroidal = ca->T == CAL_SPACE_TOROIDAL;
    d->use_list = ca->OPTIMIZATION == CAL_OPT_ACTIVE_CELLS;
    d->nx = ca->sizeof_X;
    for (int n = 0; n < ca->sizeof_X; n++) {
        d->xi[n] = ca->X[n].i;
        d->xj[n] = ca->X[n].j;
        d->xk[n] = ca->X[n].k;
    }
    return true;
}

bool cal_internal_desc3D(struct CALModel3D* ca, CALDevModel3D* d)
{
    return build_desc(ca, d);
}

extern "C" struct CALCell3D* calAddNeighbor3D(struct CALModel3D* ca, int i, int j, int k)
{
    if (ca->sizeof_X + 1 > CAL_MAX_NEIGHBORS) {
        cal::set_error(CAL_ERROR_LIMIT, "neighbourhood larger than CAL_MAX_NEIGHBORS");
        return nullptr;
    }
    struct CALCell3D* X = (struct CALCell3D*)realloc(ca->X, sizeof(struct CALCell3D) * (ca->sizeof_X + 1));
    if (!X) {
        cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "calAddNeighbor3D");
        return nullptr;
    }
    X[ca->sizeof_X].i = i;
    X[ca->sizeof_X].j = j;
    X[ca->sizeof_X].k = k;
    ca->X = X;
    ca->sizeof_X++;
    ca->gpu->d_X_len = -1;
    upload_X(ca); /* at definition time, never inside a recorded step */
    return ca->X;
}

extern "C" struct CALModel3D* calCADef3D(int rows, int columns, int slices, enum CALNeighborhood3D nb,
                                         enum CALSpaceBoundaryCondition bc, enum CALOptimization opt)
{
    struct CALModel3D* ca = (struct CALModel3D*)calloc(1, sizeof(struct CALModel3D));
    if (!ca) {
        cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "calCADef3D");
        return nullptr;
    }
    ca->gpu = new (std::nothrow) CALGpuModel3D();
    if (!ca->gpu ||
        !ca->gpu->g.init(3, rows, columns, slices, bc == CAL_SPACE_TOROIDAL, opt == CAL_OPT_ACTIVE_CELLS)) {
        if (ca->gpu) {
            ca->gpu->g.destroy();
            delete ca->gpu;
        }
        free(ca);
        return nullptr;
    }
    if (!cal::cuda_ok(cudaMalloc(&ca->gpu->d_X, sizeof(struct CALCell3D) * CAL_MAX_NEIGHBORS), "cudaMalloc X")) {
        ca->gpu->g.destroy();
        delete ca->gpu;
        free(ca);
        return nullptr;
    }
    ca->rows = rows;
    ca->columns = columns;
    ca->slices = slices;
    ca->T = bc;
    ca->OPTIMIZATION = opt;
    ca->is_safe = CAL_UNSAFE_INACTIVE;
    ca->A.flags = opt == CAL_OPT_ACTIVE_CELLS ? (CALbyte*)ca->gpu->g.h_flags : nullptr;
    ca->A.num_threads = 1;
    ca->A.size_next = (int*)calloc(1, sizeof(int));
    ca->X_id = nb;
    /* index order of cal3D.c:29-105: the 2D plane (VN 5 / Moore 9) of slice
     * 0, then slice -1, then slice +1 */
    static const int plane[9][2] = {{0, 0}, {-1, 0}, {0, -1}, {0, 1}, {1, 0}, {-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    if (nb == CAL_VON_NEUMANN_NEIGHBORHOOD_3D) {
        for (int n = 0; n < 5; n++)
            calAddNeighbor3D(ca, plane[n][0], plane[n][1], 0);
        calAddNeighbor3D(ca, 0, 0, -1);
        calAddNeighbor3D(ca, 0, 0, 1);
    } else if (nb == CAL_MOORE_NEIGHBORHOOD_3D) {
        static const int dk[3] = {0, -1, 1};
        for (int s = 0; s < 3; s++)
            for (int n = 0; n < 9; n++)
                calAddNeighbor3D(ca, plane[n][0], plane[n][1], dk[s]);
    }
    return ca;
}

extern "C" void calSetUnsafe3D(struct CALModel3D* ca) { ca->is_safe = CAL_UNSAFE_ACTIVE; }

template <typename QT, int TYPE>
static QT* add_substate(struct CALModel3D* ca, bool single)
{
    CalGrid& g = G(ca);
    void *cur = nullptr, *next = nullptr;
    int slot = g.add_sub(TYPE, single, &cur, &next);
    if (slot < 0)
        return nullptr;
    QT* q = (QT*)((char*)g.pool[TYPE] + 32 * slot);
    q->current = (decltype(q->current))cur;
    q->next = (decltype(q->next))next;
    q->cal_reserved_[0] = &g; /* lets handle-only calls (getValue*AtIndex) find the grid */
    q->cal_reserved_[1] = (void*)(intptr_t)slot;
    if (!single) {
        QT*** arr = TYPE == 0 ? (QT***)&ca->pQb_array : (TYPE == 1 ? (QT***)&ca->pQi_array : (QT***)&ca->pQr_array);
        int* n = TYPE == 0 ? &ca->sizeof_pQb_array : (TYPE == 1 ? &ca->sizeof_pQi_array : &ca->sizeof_pQr_array);
        QT** na = (QT**)realloc(*arr, sizeof(QT*) * (*n + 1));
        if (!na) {
            cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "substate array");
            return nullptr;
        }
        na[*n] = q;
        *arr = na;
        (*n)++;
    }
    return q;
}

extern "C" struct CALSubstate3Db* calAddSubstate3Db(struct CALModel3D* ca) { return add_substate<struct CALSubstate3Db, 0>(ca, false); }
extern "C" struct CALSubstate3Di* calAddSubstate3Di(struct CALModel3D* ca) { return add_substate<struct CALSubstate3Di, 1>(ca, false); }
extern "C" struct CALSubstate3Dr* calAddSubstate3Dr(struct CALModel3D* ca) { return add_substate<struct CALSubstate3Dr, 2>(ca, false); }
extern "C" struct CALSubstate3Db* calAddSingleLayerSubstate3Db(struct CALModel3D* ca) { return add_substate<struct CALSubstate3Db, 0>(ca, true); }
extern "C" struct CALSubstate3Di* calAddSingleLayerSubstate3Di(struct CALModel3D* ca) { return add_substate<struct CALSubstate3Di, 1>(ca, true); }
extern "C" struct CALSubstate3Dr* calAddSingleLayerSubstate3Dr(struct CALModel3D* ca) { return add_substate<struct CALSubstate3Dr, 2>(ca, true); }

extern "C" CALCallbackFunc3D* calAddElementaryProcess3D(struct CALModel3D* ca, CALCallbackFunc3D ep)
{
    CALLaunchFunc3D launch = find_launch(ep);
    if (!launch) {
        cal::set_error(CAL_ERROR_NOT_A_DEVICE_PROCESS,
                       "calAddElementaryProcess3D: not a device process (define it with CAL_ELEMENTARY_PROCESS_3D)");
        return nullptr;
    }
    if (ca->num_of_elementary_processes >= CAL_MAX_ELEMENTARY_PROCESSES) {
        cal::set_error(CAL_ERROR_LIMIT, "too many elementary processes");
        return nullptr;
    }
    CALCallbackFunc3D* arr = (CALCallbackFunc3D*)realloc(ca->elementary_processes,
                                                         sizeof(CALCallbackFunc3D) * (ca->num_of_elementary_processes + 1));
    if (!arr) {
        cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "calAddElementaryProcess3D");
        return nullptr;
    }
    arr[ca->num_of_elementary_processes] = ep;
    ca->gpu->launch[ca->num_of_elementary_processes] = launch;
    ca->elementary_processes = arr;
    ca->num_of_elementary_processes++;
    return ca->elementary_processes;
}

extern "C" void calAddActiveCell3D(struct CALModel3D* ca, int i, int j, int k)
{
    CalGrid& g = G(ca);
    if (!g.active || i < 0 || i >= ca->rows || j < 0 || j >= ca->columns || k < 0 || k >= ca->slices)
        return;
    if (!g.flags_to_host())
        return;
    g.h_flags[g.lin(i, j, k)] = 1;
    g.flags_dev_valid = false;
}

extern "C" void calAddActiveCellX3D(struct CALModel3D* ca, int i, int j, int k, int n)
{
    int a, b, c;
    if (neighbor(ca, i, j, k, n, &a, &b, &c))
        calAddActiveCell3D(ca, a, b, c);
}

extern "C" void calRemoveActiveCell3D(struct CALModel3D* ca, int i, int j, int k)
{
    CalGrid& g = G(ca);
    if (!g.active || i < 0 || i >= ca->rows || j < 0 || j >= ca->columns || k < 0 || k >= ca->slices)
        return;
    if (!g.flags_to_host())
        return;
    g.h_flags[g.lin(i, j, k)] = 0;
    g.flags_dev_valid = false;
}

extern "C" void calUpdateActiveCells3D(struct CALModel3D* ca) { G(ca).compact(); }

#define CAL_SUBSTATE_OPS_3D(S, T, TC)                                                                   \
    extern "C" void calInitSubstate3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, T value)    \
    {                                                                                                   \
        int s = slot_of(ca, TC, Q);                                                                     \
        if (G(ca).fill(TC, s, 0, &value, true))                                                         \
            G(ca).fill(TC, s, 1, &value, true);                                                         \
    }                                                                                                   \
    extern "C" void calInitSubstateNext3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, T value) \
    {                                                                                                   \
        G(ca).fill(TC, slot_of(ca, TC, Q), 1, &value, true);                                            \
    }                                                                                                   \
    extern "C" void calUpdateSubstate3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q)           \
    {                                                                                                   \
        CalGrid& g = G(ca);                                                                             \
        if (!g.to_device_all())                                                                         \
            return;                                                                                     \
        std::vector<std::pair<int, int>> one(1, std::make_pair(TC, slot_of(ca, TC, Q)));                \
        g.copy_next_to_current(one, false, true);                                                       \
    }                                                                                                   \
    extern "C" void calCopySubstateFromHost3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q,     \
                                                  const T* data)                                        \
    {                                                                                                   \
        G(ca).load_from_host(TC, slot_of(ca, TC, Q), data);                                             \
    }                                                                                                   \
    extern "C" void calCopySubstateToHost3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, T* data) \
    {                                                                                                   \
        G(ca).store_to_host(TC, slot_of(ca, TC, Q), data);                                              \
    }

CAL_SUBSTATE_OPS_3D(b, CALbyte, 0)
CAL_SUBSTATE_OPS_3D(i, CALint, 1)
CAL_SUBSTATE_OPS_3D(r, CALreal, 2)

static void apply_launch(struct CALModel3D* ca, CALLaunchFunc3D launch)
{
    CalGrid& g = G(ca);
    if (!g.repair_all_stale() || !g.to_device_all())
        return;
    CALDevModel3D d;
    if (!build_desc(ca, &d))
        return;
    int gx, gy;
    g.launch_grid(&gx, &gy);
    int rc = launch(&d, gx, gy, (void*)g.stream);
    if (rc != 0) {
        cal::cuda_ok((cudaError_t)rc, "elementary process launch");
        return;
    }
    g.device_wrote_all();
}

extern "C" void calApplyElementaryProcess3D(struct CALModel3D* ca, CALCallbackFunc3D ep)
{
    CALLaunchFunc3D launch = find_launch(ep);
    if (!launch) {
        cal::set_error(CAL_ERROR_NOT_A_DEVICE_PROCESS, "calApplyElementaryProcess3D: not a device process");
        return;
    }
    apply_launch(ca, launch);
}

extern "C" void calUpdate3D(struct CALModel3D* ca) { G(ca).update_all(); }

extern "C" void calGlobalTransitionFunction3D(struct CALModel3D* ca)
{
    for (int b = 0; b < ca->num_of_elementary_processes; b++) {
        apply_launch(ca, ca->gpu->launch[b]);
        calUpdate3D(ca);
    }
}

#define CAL_CELL_OPS_3D(S, T, TC)                                                                            \
    extern "C" T calGet3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k)         \
    {                                                                                                        \
        G(ca).to_host(TC, slot_of(ca, TC, Q), 0);                                                            \
        return Q->current[G(ca).lin(i, j, k)];                                                               \
    }                                                                                                        \
    extern "C" T calGetX3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k, int n) \
    {                                                                                                        \
        int a, b, c;                                                                                         \
        if (!neighbor(ca, i, j, k, n, &a, &b, &c))                                                           \
            return (T)0;                                                                                     \
        return calGet3D##S(ca, Q, a, b, c);                                                                  \
    }                                                                                                        \
    extern "C" void calSet3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k, T v) \
    {                                                                                                        \
        int s = slot_of(ca, TC, Q);                                                                          \
        if (!G(ca).to_host(TC, s, 1))                                                                        \
            return;                                                                                          \
        Q->next[G(ca).lin(i, j, k)] = v;                                                                     \
        G(ca).host_wrote(TC, s, 1);                                                                          \
    }                                                                                                        \
    extern "C" void calSetCurrent3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k, T v) \
    {                                                                                                        \
        int s = slot_of(ca, TC, Q);                                                                          \
        if (!G(ca).to_host(TC, s, 0))                                                                        \
            return;                                                                                          \
        Q->current[G(ca).lin(i, j, k)] = v;                                                                  \
        G(ca).host_wrote(TC, s, 0);                                                                          \
    }                                                                                                        \
    extern "C" void calInit3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k, T v) \
    {                                                                                                        \
        int s = slot_of(ca, TC, Q);                                                                          \
        calSetCurrent3D##S(ca, Q, i, j, k, v);                                                               \
        if (Q->next && G(ca).to_host(TC, s, 1)) {                                                            \
            Q->next[G(ca).lin(i, j, k)] = v;                                                                 \
            G(ca).host_wrote(TC, s, 1);                                                                      \
        }                                                                                                    \
    }

CAL_CELL_OPS_3D(b, CALbyte, 0)
CAL_CELL_OPS_3D(i, CALint, 1)
CAL_CELL_OPS_3D(r, CALreal, 2)

extern "C" void calSync3D(struct CALModel3D* ca)
{
    CalGrid& g = G(ca);
    for (int t = 0; t < CAL_NTYPES; t++)
        for (int s = 0; s < g.nslot[t]; s++) {
            g.to_host(t, s, 0);
            if (!g.sub[t][s].single)
                g.to_host(t, s, 1);
        }
    if (!g.active) {
        g.sync();
        return;
    }
    g.flags_to_host();
    int n = 0;
    if (!cal::cuda_ok(cudaMemcpyAsync(&n, g.d_count, sizeof(int), cudaMemcpyDeviceToHost, g.stream), "read count") ||
        !g.sync())
        return;
    free(ca->A.cells);
    ca->A.cells = nullptr;
    ca->A.size_current = n;
    if (n > 0) {
        ca->A.cells = (struct CALCell3D*)malloc(sizeof(struct CALCell3D) * (size_t)n);
        if (!ca->A.cells) {
            cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "calSync3D active list");
            return;
        }
        /* device cells are packed (i, j, k) ints, the same layout as CALCell3D */
        if (cal::cuda_ok(cudaMemcpyAsync(ca->A.cells, g.d_cells, sizeof(int) * 3 * (size_t)n, cudaMemcpyDeviceToHost,
                                         g.stream), "read active list"))
            g.sync();
    }
}

extern "C" void calMarkHostDirty3D(struct CALModel3D* ca)
{
    /* every layer's host mirror becomes the authoritative copy (the caller
     * either overwrote it entirely or made it current first with calSync) */
    CalGrid& g = G(ca);
    for (int t = 0; t < CAL_NTYPES; t++)
        for (int s = 0; s < g.nslot[t]; s++)
            for (int l = 0; l < (g.sub[t][s].single ? 1 : 2); l++) {
                g.host_wrote(t, s, l);
                g.sub[t][s].layer[l].host_valid = true;
                if (l == 1)
                    g.sub[t][s].next_stale = false;
            }
    if (g.active && g.flags_host_valid)
        g.flags_dev_valid = false;
}

extern "C" void calFinish3D(struct CALModel3D* ca) { G(ca).sync(); }
extern "C" void* calGetStream3D(struct CALModel3D* ca) { return (void*)G(ca).stream; }

extern "C" int calGetActiveCellCount3D(struct CALModel3D* ca)
{
    CalGrid& g = G(ca);
    int n = 0;
    if (cal::cuda_ok(cudaMemcpyAsync(&n, g.d_count, sizeof(int), cudaMemcpyDeviceToHost, g.stream), "read count"))
        g.sync();
    return n;
}

extern "C" void calFinalize3D(struct CALModel3D* ca)
{
    if (!ca)
        return;
    if (ca->gpu) {
        ca->gpu->g.destroy();
        if (ca->gpu->d_X)
            cudaFree(ca->gpu->d_X);
        delete ca->gpu;
    }
    free(ca->A.cells);
    free(ca->A.size_next);
    free(ca->X);
    free(ca->pQb_array);
    free(ca->pQi_array);
    free(ca->pQr_array);
    free(ca->elementary_processes);
    free(ca);
}

/* ======================= unsafe operations (cal3DUnsafe.h) ============== */
/* OpenCAL-OMP/source/cal3DUnsafe.c:18-245, on the host mirrors */

#define CAL_UNSAFE_OPS_3D(S, T, TC)                                                                          \
    extern "C" T calGetNext3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k)     \
    {                                                                                                        \
        if (!G(ca).to_host(TC, slot_of(ca, TC, Q), 1))                                                       \
            return (T)0;                                                                                     \
        return Q->next[G(ca).lin(i, j, k)];                                                                  \
    }                                                                                                        \
    extern "C" T calGetNextX3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k, int n) \
    {                                                                                                        \
        int a, b, c;                                                                                         \
        if (!neighbor(ca, i, j, k, n, &a, &b, &c))                                                           \
            return (T)0;                                                                                     \
        return calGetNext3D##S(ca, Q, a, b, c);                                                              \
    }                                                                                                        \
    extern "C" void calSetX3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k, int n, \
                                 T v)                                                                        \
    {                                                                                                        \
        int a, b, c;                                                                                         \
        if (neighbor(ca, i, j, k, n, &a, &b, &c))                                                            \
            calSet3D##S(ca, Q, a, b, c, v);                                                                  \
    }                                                                                                        \
    extern "C" void calSetCurrentX3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k, \
                                        int n, T v)                                                          \
    {                                                                                                        \
        int a, b, c;                                                                                         \
        if (neighbor(ca, i, j, k, n, &a, &b, &c))                                                            \
            calSetCurrent3D##S(ca, Q, a, b, c, v);                                                           \
    }                                                                                                        \
    extern "C" void calInitX3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k, int n, \
                                  T v)                                                                       \
    {                                                                                                        \
        int a, b, c;                                                                                         \
        if (neighbor(ca, i, j, k, n, &a, &b, &c))                                                            \
            calInit3D##S(ca, Q, a, b, c, v);                                                                 \
    }                                                                                                        \
    extern "C" void calAddNext3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k, T v) \
    {                                                                                                        \
        const int s = slot_of(ca, TC, Q);                                                                    \
        if (!G(ca).to_host(TC, s, 1))                                                                        \
            return;                                                                                          \
        T* p = &Q->next[G(ca).lin(i, j, k)];                                                                 \
        *p = (T)(*p + v);                                                                                    \
        G(ca).host_wrote(TC, s, 1);                                                                          \
    }                                                                                                        \
    extern "C" void calAddNextX3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* Q, int i, int j, int k, int n, \
                                     T v)                                                                    \
    {                                                                                                        \
        int a, b, c;                                                                                         \
        if (neighbor(ca, i, j, k, n, &a, &b, &c))                                                            \
            calAddNext3D##S(ca, Q, a, b, c, v);                                                              \
    }

CAL_UNSAFE_OPS_3D(b, CALbyte, 0)
CAL_UNSAFE_OPS_3D(i, CALint, 1)
CAL_UNSAFE_OPS_3D(r, CALreal, 2)
