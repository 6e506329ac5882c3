/*
 * cal2D.cu -- the 2D C API (include/opencal/cal2D.h) on top of the shared
 * engine (cal_core.cu).
 *
 * Reference behaviour restated (OpenCAL-OMP/source/cal2D.c):
 *   calCADef2D + neighbourhood builders      cal2D.c:28-166, 252-327
 *   active cells add/remove/update           cal2D.c:333-440
 *   substates, single-layer substates        cal2D.c:470-596
 *   elementary-process list                  cal2D.c:600-621
 *   init / init-next / update of substates   cal2D.c:625-713
 *   apply, global transition, update         cal2D.c:717-776
 *   cell accessors (host side)               cal2D.c:780-930
 *   finalize                                 cal2D.c:933-961
 */
#define CAL_BUILDING_LIBRARY
#include <stdlib.h>
#include <string.h>

#include <algorithm>

#include "cal_model_internal.cuh"
#include "cal_tma.cuh"
#include "opencal/cal2DUnsafe.h"

using cal::CalGrid;

/* ======================= process registry =============================== */
/* Filled by static initialisers of the translation units that define
 * processes, possibly before main(): plain zero-initialised arrays. */
#define CAL_REGISTRY_MAX 4096
static CALCallbackFunc2D g_reg_host[CAL_REGISTRY_MAX];
static CALLaunchFunc2D g_reg_launch[CAL_REGISTRY_MAX];
static int g_reg_n;

extern "C" int calRegisterElementaryProcess2D(CALCallbackFunc2D host_name, CALLaunchFunc2D launch, const char* name)
{
    for (int r = 0; r < g_reg_n; r++)
        if (g_reg_host[r] == host_name) {
            g_reg_launch[r] = launch;
            return 1;
        }
    if (g_reg_n >= CAL_REGISTRY_MAX)
        return 0;
    g_reg_host[g_reg_n] = host_name;
    g_reg_launch[g_reg_n] = launch;
    (void)name;
    g_reg_n++;
    return 1;
}

static CALLaunchFunc2D find_launch(CALCallbackFunc2D f)
{
    for (int r = 0; r < g_reg_n; r++)
        if (g_reg_host[r] == f)
            return g_reg_launch[r];
    return nullptr;
}

extern "C" void calHostCallOfDeviceProcess2D(const char* name)
{
    cal::set_error(CAL_ERROR_NOT_A_DEVICE_PROCESS,
                   std::string("device elementary process '") + name +
                       "' called as a host function; apply it with calApplyElementaryProcess2D");
}

/* ======================= helpers ======================================== */

static inline CalGrid& G(struct CALModel2D* ca) { return ca->gpu->g; }

template <typename Q>
static inline int slot_of(struct CALModel2D* ca, int type, Q* q)
{
    return (int)(((char*)q - (char*)G(ca).pool[type]) / 32);
}

static bool neighbor(const struct CALModel2D* ca, int i, int j, int n, int* oi, int* oj)
{
    if ((ca->X_id == CAL_HEXAGONAL_NEIGHBORHOOD_2D && (j % 2) == 1) ||
        (ca->X_id == CAL_HEXAGONAL_NEIGHBORHOOD_ALT_2D && (i % 2) == 1))
        n += CAL_HEXAGONAL_SHIFT;
    int a = i + ca->X[n].i, b = j + ca->X[n].j;
    if (ca->T == CAL_SPACE_TOROIDAL) {
        a = calGetToroidalX(a, ca->rows);
        b = calGetToroidalX(b, ca->columns);
    } else if (a < 0 || a >= ca->rows || b < 0 || b >= ca->columns) {
        return false;
    }
    *oi = a;
    *oj = b;
    return true;
}

static int table_len(const struct CALModel2D* ca);

/* the table only changes through calAddNeighbor2D: upload it when it did */
static bool upload_X(struct CALModel2D* ca)
{
    CALGpuModel2D* gm = ca->gpu;
    const int len = table_len(ca);
    if (gm->d_X_len == len || len == 0)
        return true;
    if (gm->g.capturing) {
        cal::set_error(CAL_ERROR_NOT_CAPTURABLE, "neighbourhood changed during graph capture");
        return false;
    }
    if (!cal::cuda_ok(cudaMemcpy(gm->d_X, ca->X, sizeof(struct CALCell2D) * len, cudaMemcpyHostToDevice), "upload X"))
        return false;
    gm->d_X_len = len;
    return true;
}

static int table_len(const struct CALModel2D* ca)
{
    /* hexagonal models keep 14 entries and report 7 (cal2D.c:115, 160) */
    return (ca->X_id == CAL_HEXAGONAL_NEIGHBORHOOD_2D || ca->X_id == CAL_HEXAGONAL_NEIGHBORHOOD_ALT_2D)
               ? 2 * ca->sizeof_X : ca->sizeof_X;
}

/* launch descriptor for a process kernel */
static bool build_desc(struct CALModel2D* ca, CALDevModel2D* d)
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
    d->model.A.cells = (struct CALCell2D*)g.d_cells;
    const int len = table_len(ca);
    if (len > CAL_MAX_NEIGHBORS) {
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
    d->flags_dirty = g.flags_dirty_word();
    d->step = g.d_step;
    d->flags = (CALbyte*)g.d_flags;
    d->cells = (struct CALCell2D*)g.d_cells;
    d->count = g.d_count;
    d->rows = ca->rows;
    d->cols = ca->columns;
    d->toroidal = ca->T == CAL_SPACE_TOROIDAL;
    d->hex = ca->X_id == CAL_HEXAGONAL_NEIGHBORHOOD_2D ? 1 : (ca->X_id == CAL_HEXAGONAL_NEIGHBORHOOD_ALT_2D ? 2 : 0);
    d->use_list = ca->OPTIMIZATION == CAL_OPT_ACTIVE_CELLS;
    d->nx = ca->sizeof_X;
    for (int n = 0; n < len; n++) {
        d->xi[n] = ca->X[n].i;
        d->xj[n] = ca->X[n].j;
    }
    /* process tiles (every launch) and change tracking (models without
     * active cells) */
    d->tiles_x = (ca->columns + CAL_TILE_W - 1) / CAL_TILE_W;
    d->tiles_y = (ca->rows + CAL_TILE_H - 1) / CAL_TILE_H;
    d->track = g.tracking ? 1 : 0;
    d->tile_words = g.tile_words;
    d->chg = g.d_chg;
    d->untracked = g.d_untracked;
    return true;
}

/* launch descriptor for library-internal kernels (run loop) */
bool cal_internal_desc2D(struct CALModel2D* ca, CALDevModel2D* d)
{
    return build_desc(ca, d);
}

/* ======================= definition ===================================== */

static void add_default_neighborhood(struct CALModel2D* ca)
{
    /* index order of the reference's tables (cal2D.c:28-166) */
    static const int vn[5][2] = {{0, 0}, {-1, 0}, {0, -1}, {0, 1}, {1, 0}};
    static const int moore[9][2] = {{0, 0}, {-1, 0}, {0, -1}, {0, 1}, {1, 0}, {-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    static const int hex[14][2] = {{0, 0}, {-1, 1}, {-1, 0}, {-1, -1}, {0, -1}, {1, 0}, {0, 1},
                                   {0, 0}, {0, 1}, {-1, 0}, {0, -1}, {1, -1}, {1, 0}, {1, 1}};
    static const int hexalt[14][2] = {{0, 0}, {-1, 0}, {-1, -1}, {0, -1}, {1, -1}, {1, 0}, {0, 1},
                                      {0, 0}, {-1, 1}, {-1, 0}, {0, -1}, {1, 0}, {1, 1}, {0, 1}};
    const int(*t)[2] = nullptr;
    int cnt = 0;
    switch (ca->X_id) {
    case CAL_VON_NEUMANN_NEIGHBORHOOD_2D: t = vn; cnt = 5; break;
    case CAL_MOORE_NEIGHBORHOOD_2D: t = moore; cnt = 9; break;
    case CAL_HEXAGONAL_NEIGHBORHOOD_2D: t = hex; cnt = 14; break;
    case CAL_HEXAGONAL_NEIGHBORHOOD_ALT_2D: t = hexalt; cnt = 14; break;
    default: return;
    }
    for (int n = 0; n < cnt; n++)
        calAddNeighbor2D(ca, t[n][0], t[n][1]);
    if (cnt == 14) {
        ca->sizeof_X = 7;
        ca->gpu->d_X_len = -1;
        upload_X(ca);
    }
}

extern "C" struct CALModel2D* calCADef2D(int rows, int columns, enum CALNeighborhood2D nb,
                                         enum CALSpaceBoundaryCondition bc, enum CALOptimization opt)
{
    struct CALModel2D* ca = (struct CALModel2D*)calloc(1, sizeof(struct CALModel2D));
    if (!ca) {
        cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "calCADef2D");
        return nullptr;
    }
    ca->gpu = new (std::nothrow) CALGpuModel2D();
    if (!ca->gpu || !ca->gpu->g.init(2, rows, columns, 1, bc == CAL_SPACE_TOROIDAL, opt == CAL_OPT_ACTIVE_CELLS)) {
        if (ca->gpu) {
            ca->gpu->g.destroy();
            delete ca->gpu;
        }
        free(ca);
        return nullptr;
    }
    if (!cal::cuda_ok(cudaMalloc(&ca->gpu->d_X, sizeof(struct CALCell2D) * CAL_MAX_NEIGHBORS), "cudaMalloc X")) {
        ca->gpu->g.destroy();
        delete ca->gpu;
        free(ca);
        return nullptr;
    }
    ca->rows = rows;
    ca->columns = columns;
    ca->T = bc;
    ca->is_safe = CAL_UNSAFE_INACTIVE;
    ca->OPTIMIZATION = opt;
    ca->A.flags = opt == CAL_OPT_ACTIVE_CELLS ? (CALbyte*)ca->gpu->g.h_flags : nullptr;
    ca->A.num_threads = 1;
    ca->A.size_next = (int*)calloc(1, sizeof(int));
    ca->A.cells = nullptr;
    ca->A.size_current = 0;
    ca->X = nullptr;
    ca->sizeof_X = 0;
    ca->X_id = nb;
    add_default_neighborhood(ca);
    return ca;
}

extern "C" void calSetUnsafe2D(struct CALModel2D* ca2D)
{
    ca2D->is_safe = CAL_UNSAFE_ACTIVE;
}

extern "C" struct CALCell2D* calAddNeighbor2D(struct CALModel2D* ca, int i, int j)
{
    if (table_len(ca) + 1 > CAL_MAX_NEIGHBORS) {
        cal::set_error(CAL_ERROR_LIMIT, "neighbourhood larger than CAL_MAX_NEIGHBORS");
        return nullptr;
    }
    int len = ca->sizeof_X;
    struct CALCell2D* X = (struct CALCell2D*)realloc(ca->X, sizeof(struct CALCell2D) * (len + 1));
    if (!X) {
        cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "calAddNeighbor2D");
        return nullptr;
    }
    X[len].i = i;
    X[len].j = j;
    ca->X = X;
    ca->sizeof_X = len + 1;
    ca->gpu->d_X_len = -1;
    upload_X(ca); /* at definition time, never inside a recorded step */
    return ca->X;
}

template <typename QT, int TYPE>
static QT* add_substate(struct CALModel2D* ca, bool single)
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

extern "C" struct CALSubstate2Db* calAddSubstate2Db(struct CALModel2D* ca) { return add_substate<struct CALSubstate2Db, 0>(ca, false); }
extern "C" struct CALSubstate2Di* calAddSubstate2Di(struct CALModel2D* ca) { return add_substate<struct CALSubstate2Di, 1>(ca, false); }
extern "C" struct CALSubstate2Dr* calAddSubstate2Dr(struct CALModel2D* ca) { return add_substate<struct CALSubstate2Dr, 2>(ca, false); }
extern "C" struct CALSubstate2Db* calAddSingleLayerSubstate2Db(struct CALModel2D* ca) { return add_substate<struct CALSubstate2Db, 0>(ca, true); }
extern "C" struct CALSubstate2Di* calAddSingleLayerSubstate2Di(struct CALModel2D* ca) { return add_substate<struct CALSubstate2Di, 1>(ca, true); }
extern "C" struct CALSubstate2Dr* calAddSingleLayerSubstate2Dr(struct CALModel2D* ca) { return add_substate<struct CALSubstate2Dr, 2>(ca, true); }

extern "C" CALCallbackFunc2D* calAddElementaryProcess2D(struct CALModel2D* ca, CALCallbackFunc2D ep)
{
    CALLaunchFunc2D launch = find_launch(ep);
    if (!launch) {
        cal::set_error(CAL_ERROR_NOT_A_DEVICE_PROCESS,
                       "calAddElementaryProcess2D: not a device process (define it with CAL_ELEMENTARY_PROCESS_2D)");
        return nullptr;
    }
    if (ca->num_of_elementary_processes >= CAL_MAX_ELEMENTARY_PROCESSES) {
        cal::set_error(CAL_ERROR_LIMIT, "too many elementary processes");
        return nullptr;
    }
    CALCallbackFunc2D* arr = (CALCallbackFunc2D*)realloc(ca->elementary_processes,
                                                         sizeof(CALCallbackFunc2D) * (ca->num_of_elementary_processes + 1));
    if (!arr) {
        cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "calAddElementaryProcess2D");
        return nullptr;
    }
    arr[ca->num_of_elementary_processes] = ep;
    ca->gpu->launch[ca->num_of_elementary_processes] = launch;
    ca->elementary_processes = arr;
    ca->num_of_elementary_processes++;
    return ca->elementary_processes;
}

/* ======================= active cells (host side) ======================== */

extern "C" void calAddActiveCell2D(struct CALModel2D* ca, int i, int j)
{
    CalGrid& g = G(ca);
    if (!g.active || i < 0 || i >= ca->rows || j < 0 || j >= ca->columns)
        return;
    if (!g.flags_to_host())
        return;
    g.h_flags[(long long)i * ca->columns + j] = 1;
    g.flags_dev_valid = false;
}

extern "C" void calAddActiveCellX2D(struct CALModel2D* ca, int i, int j, int n)
{
    int a, b;
    if (neighbor(ca, i, j, n, &a, &b))
        calAddActiveCell2D(ca, a, b);
}

extern "C" void calRemoveActiveCell2D(struct CALModel2D* ca, int i, int j)
{
    CalGrid& g = G(ca);
    if (!g.active || i < 0 || i >= ca->rows || j < 0 || j >= ca->columns)
        return;
    if (!g.flags_to_host())
        return;
    g.h_flags[(long long)i * ca->columns + j] = 0;
    g.flags_dev_valid = false;
}

extern "C" void calUpdateActiveCells2D(struct CALModel2D* ca)
{
    G(ca).compact();
}

/* ======================= whole-substate operations ====================== */

#define CAL_SUBSTATE_OPS_2D(S, T, TC)                                                                   \
    extern "C" void calInitSubstate2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, T value)    \
    {                                                                                                   \
        G(ca).fill_both(TC, slot_of(ca, TC, Q), &value);                                                \
    }                                                                                                   \
    extern "C" void calInitSubstateNext2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, T value) \
    {                                                                                                   \
        G(ca).fill(TC, slot_of(ca, TC, Q), 1, &value, true);                                            \
    }                                                                                                   \
    extern "C" void calUpdateSubstate2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q)           \
    {                                                                                                   \
        CalGrid& g = G(ca);                                                                             \
        if (!g.to_device_all())                                                                         \
            return;                                                                                     \
        std::vector<std::pair<int, int>> one(1, std::make_pair(TC, slot_of(ca, TC, Q)));                \
        g.copy_next_to_current(one, false, true);                                                       \
    }                                                                                                   \
    extern "C" void* calGetDeviceBuffer2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int layer) \
    {                                                                                                   \
        CalGrid& g = G(ca);                                                                             \
        int s = slot_of(ca, TC, Q);                                                                     \
        if (!g.to_device_all())                                                                         \
            return nullptr;                                                                             \
        if (layer == 1 && !g.repair_stale(TC, s))                                                       \
            return nullptr;                                                                             \
        g.untrack(TC, s); /* the caller may write it: no change tracking from now on */                \
        return g.sub[TC][s].layer[layer ? 1 : 0].dev;  /* layer 2: next, to be overwritten whole */     \
    }                                                                                                   \
    extern "C" void calCopySubstateFromHost2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q,      \
                                                  const T* data)                                           \
    {                                                                                                      \
        G(ca).load_from_host(TC, slot_of(ca, TC, Q), data);                                                \
    }                                                                                                      \
    extern "C" void calCopySubstateToHost2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, T* data) \
    {                                                                                                      \
        G(ca).store_to_host(TC, slot_of(ca, TC, Q), data);                                                 \
    }                                                                                                      \
    extern "C" void calSyncSubstate2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q)             \
    {                                                                                                   \
        G(ca).to_host(TC, slot_of(ca, TC, Q), 0);                                                       \
    }                                                                                                   \
    extern "C" void calMarkCurrentWritten2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q)       \
    {                                                                                                   \
        G(ca).sub[TC][slot_of(ca, TC, Q)].layer[0].host_valid = false;                                  \
        G(ca).untrack(TC, slot_of(ca, TC, Q));                                                          \
    }                                                                                                   \
    extern "C" void calSwapSubstate2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q)             \
    {                                                                                                   \
        G(ca).swap(TC, slot_of(ca, TC, Q));                                                             \
    }

CAL_SUBSTATE_OPS_2D(b, CALbyte, 0)
CAL_SUBSTATE_OPS_2D(i, CALint, 1)
CAL_SUBSTATE_OPS_2D(r, CALreal, 2)

/* ======================= transition ===================================== */

/* TMA staging of process b's declared reads into the descriptor: one
 * tensor map per substate over its current layer; nothing staged (global
 * reads, same results) when the model keeps an active list, a substate's
 * rows are not a multiple of 16 bytes, the neighbourhood reaches further
 * than the box's halo, or the boxes would not fit in 48 KB */
static void stage_reads(struct CALModel2D* ca, int b, CALDevModel2D* d)
{
    CalGrid& g = G(ca);
    const int n = ca->gpu->nreads[b];
    if (n <= 0 || g.active || g.dim != 2)
        return;
    int ri = 0, rj = 0;
    const int len = table_len(ca);
    for (int k = 0; k < len; k++) {
        ri = std::max(ri, std::abs(ca->X[k].i));
        rj = std::max(rj, std::abs(ca->X[k].j));
    }
    if (ca->X_id == CAL_HEXAGONAL_NEIGHBORHOOD_2D || ca->X_id == CAL_HEXAGONAL_NEIGHBORHOOD_ALT_2D) {
        ri = std::max(ri, 1);
        rj = std::max(rj, 1);
    }
    if (ri > CAL_TILE_H)
        return;
    static const CUtensorMapDataType kType[3] = {CU_TENSOR_MAP_DATA_TYPE_UINT8, CU_TENSOR_MAP_DATA_TYPE_INT32,
                                                 CU_TENSOR_MAP_DATA_TYPE_FLOAT64};
    int off = 0, tx = 0;
    for (int k = 0; k < n; k++) {
        const int t = ca->gpu->read_t[b][k], s = ca->gpu->read_s[b][k];
        const cal::Sub& q = g.sub[t][s];
        const int es = (int)q.elem, hx = 16 / es;
        if (!q.used || rj > hx)
            return;
        const int bw = CAL_TILE_W + 2 * hx, bh = CAL_TILE_H + 2 * ri;
        if (!caltma::encode_2d(&d->stage_map[k], q.layer[0].dev, kType[t], es, ca->rows, ca->columns, bw, bh))
            return;
        d->stage_off[k] = off;
        d->stage_hx[k] = hx;
        d->stage_of[t][s] = (signed char)k;
        off += (bw * bh * es + 127) & ~127;
        tx += bw * bh * es;
    }
    if (2 * off + 128 > 48 * 1024 || !ca->gpu->d_stage_err) /* two buffers in 48 KB */
        return;
    d->nstage = n;
    d->stage_r = ri;
    d->stage_hxmax = 0;
    for (int k = 0; k < n; k++)
        d->stage_hxmax = std::max(d->stage_hxmax, d->stage_hx[k]);
    d->stage_tx = tx;
    d->stage_bytes = off;
    d->stage_err = ca->gpu->d_stage_err;
}

/* run: the process's must-run bitmap when its tiles may be skipped; b: the
 * process's index (its declared reads are staged), -1 for none */
static void apply_launch(struct CALModel2D* ca, CALLaunchFunc2D launch, unsigned* run = nullptr, int b = -1)
{
    CalGrid& g = G(ca);
    if (!g.repair_all_stale() || !g.to_device_all())
        return;
    CALDevModel2D d;
    if (!build_desc(ca, &d))
        return;
    d.run = run;
    for (int t = 0; t < 3; t++)
        for (int s = 0; s < CAL_MAX_SUBSTATES; s++)
            d.stage_of[t][s] = -1;
    if (b >= 0) {
        stage_reads(ca, b, &d);
        d.guard_op = ca->gpu->guard_op[b];
        d.guard_slot = ca->gpu->guard_slot[b];
        d.guard_value = ca->gpu->guard_value[b];
    }
    if (!d.nstage)
        for (int t = 0; t < 3; t++)
            for (int s = 0; s < CAL_MAX_SUBSTATES; s++)
                d.stage_of[t][s] = -1;
    int gx, gy;
    g.launch_grid(&gx, &gy);
    if (g.active) {
        /* the active list, one cell per thread: 608 blocks of 256 threads
         * (four resident per SM) cover 155K cells a pass, and fewer blocks
         * launch faster than the dense grid */
        gx = 1;
        gy = 152 * 4;
    }
    /* a skipping launch deals its busy tiles over the blocks when every
     * block can rank the bitmap (at most 16 words a thread) and keep its
     * share (at most CAL_DEAL_MAX tiles) */
    if (run && g.d_quiet && g.tile_words <= 16 * CAL_EP_THREADS &&
        (long long)g.tiles_x * g.tiles_y <= (long long)CAL_DEAL_MAX * gx * gy) {
        d.quiet = g.d_quiet;
        d.ticket = g.d_ticket;
    }
    int rc = launch(&d, gx, gy, (void*)g.stream);
    if (rc != 0) {
        cal::cuda_ok((cudaError_t)rc, "elementary process launch");
        return;
    }
    g.device_wrote_all();
}

extern "C" void calApplyElementaryProcess2D(struct CALModel2D* ca, CALCallbackFunc2D ep)
{
    CALLaunchFunc2D launch = find_launch(ep);
    if (!launch) {
        cal::set_error(CAL_ERROR_NOT_A_DEVICE_PROCESS, "calApplyElementaryProcess2D: not a device process");
        return;
    }
    apply_launch(ca, launch);
}

extern "C" void calUpdate2D(struct CALModel2D* ca)
{
    G(ca).update_all();
}

/* Whether the pure processes' tiles may be skipped now: change tracking on
 * (no active cells), no unsafe operations, every substate written by the
 * library alone, and a neighbourhood that reaches only the eight tiles
 * around a cell's tile (at most CAL_TILE_H rows and CAL_TILE_W columns; on
 * toroidal grids whose last tile row / column is partial, at most its
 * height / width, so that the wrap stays within the next tile). */
static bool skipping_allowed(struct CALModel2D* ca)
{
    CalGrid& g = G(ca);
    if (!g.tracking || !g.d_run || ca->is_safe == CAL_UNSAFE_ACTIVE)
        return false;
    for (int t = 0; t < CAL_NTYPES; t++)
        for (int s = 0; s < g.nslot[t]; s++)
            if (g.sub[t][s].used && !g.sub[t][s].single && !g.sub[t][s].trackable)
                return false;
    int ri = 0, rj = 0;
    const int len = table_len(ca);
    for (int n = 0; n < len; n++) {
        ri = std::max(ri, std::abs(ca->X[n].i));
        rj = std::max(rj, std::abs(ca->X[n].j));
    }
    if (ca->X_id == CAL_HEXAGONAL_NEIGHBORHOOD_2D || ca->X_id == CAL_HEXAGONAL_NEIGHBORHOOD_ALT_2D) {
        ri = std::max(ri, 1);
        rj = std::max(rj, 1);
    }
    if (ri > CAL_TILE_H || rj > CAL_TILE_W)
        return false;
    if (ca->T == CAL_SPACE_TOROIDAL) {
        const int pr = ca->rows % CAL_TILE_H, pc = ca->columns % CAL_TILE_W;
        if ((pr && ri > pr) || (pc && rj > pc))
            return false;
    }
    return true;
}

/* Bring the skipping state up to date: whether the pure processes' tiles
 * may be skipped, and if the bitmaps were not kept meanwhile (skipping just
 * became possible, or an event the tiles cannot follow happened), every
 * tile runs again.  Returns whether tiles may be skipped. */
bool cal_prepare_skipping2D(struct CALModel2D* ca)
{
    CalGrid& g = G(ca);
    bool any_pure = false;
    for (int b = 0; b < ca->num_of_elementary_processes; b++)
        any_pure = any_pure || ca->gpu->pure[b];
    const bool skip = any_pure && skipping_allowed(ca);
    const int nrun = skip ? ca->num_of_elementary_processes : 0;
    if (nrun != g.nrun || (skip && g.run_epoch != g.inval_epoch)) {
        g.nrun = nrun;
        if (nrun && !g.arm_runs())
            return false;
    }
    return skip;
}

extern "C" void calGlobalTransitionFunction2D(struct CALModel2D* ca)
{
    CalGrid& g = G(ca);
    const bool skip = cal_prepare_skipping2D(ca);
    for (int b = 0; b < ca->num_of_elementary_processes; b++) {
        unsigned* run = (skip && ca->gpu->pure[b]) ? g.d_run + (size_t)b * g.tile_words : nullptr;
        apply_launch(ca, ca->gpu->launch[b], run, b);
        calUpdate2D(ca);
    }
}

extern "C" int calSetElementaryProcessReads2D(struct CALModel2D* ca, CALCallbackFunc2D ep, const void* const* substates,
                                              int count)
{
    if (!ca || !ca->gpu || count < 0 || count > CAL_MAX_STAGED || (count > 0 && !substates)) {
        cal::set_error(CAL_ERROR_INVALID_ARGUMENT, "calSetElementaryProcessReads2D: bad arguments");
        return CAL_ERROR_INVALID_ARGUMENT;
    }
    CalGrid& g = G(ca);
    int b = -1;
    for (int k = 0; k < ca->num_of_elementary_processes; k++)
        if (ca->elementary_processes[k] == ep)
            b = k;
    if (b < 0) {
        cal::set_error(CAL_ERROR_INVALID_ARGUMENT,
                       "calSetElementaryProcessReads2D: not a process added with calAddElementaryProcess2D");
        return CAL_ERROR_INVALID_ARGUMENT;
    }
    int ts[CAL_MAX_STAGED], ss[CAL_MAX_STAGED];
    for (int k = 0; k < count; k++) {
        /* a handle's type is the pool it lies in, its slot its 32-byte record */
        ts[k] = -1;
        for (int t = 0; t < CAL_NTYPES && ts[k] < 0; t++) {
            const uintptr_t h = (uintptr_t)substates[k], p0 = (uintptr_t)g.pool[t];
            if (h >= p0 && h < p0 + 32u * CAL_MAX_SUBSTATES_CORE && ((h - p0) & 31u) == 0 &&
                (int)((h - p0) >> 5) < g.nslot[t] && g.sub[t][(h - p0) >> 5].used) {
                ts[k] = t;
                ss[k] = (int)((h - p0) >> 5);
            }
        }
        if (ts[k] < 0 || g.sub[ts[k]][ss[k]].single) {
            cal::set_error(CAL_ERROR_INVALID_ARGUMENT,
                           "calSetElementaryProcessReads2D: not a (two-layer) substate of this model");
            return CAL_ERROR_INVALID_ARGUMENT;
        }
        for (int j = 0; j < k; j++)
            if (ts[j] == ts[k] && ss[j] == ss[k]) {
                cal::set_error(CAL_ERROR_INVALID_ARGUMENT, "calSetElementaryProcessReads2D: substate listed twice");
                return CAL_ERROR_INVALID_ARGUMENT;
            }
    }
    if (count > 0 && !ca->gpu->d_stage_err &&
        (!cal::cuda_ok(cudaMalloc(&ca->gpu->d_stage_err, sizeof(int)), "cudaMalloc staging flag") ||
         !cal::cuda_ok(cudaMemset(ca->gpu->d_stage_err, 0, sizeof(int)), "memset staging flag")))
        return CAL_ERROR_CUDA;
    ca->gpu->nreads[b] = count;
    for (int k = 0; k < count; k++) {
        ca->gpu->read_t[b][k] = ts[k];
        ca->gpu->read_s[b][k] = ss[k];
    }
    g.inval_epoch++; /* a recorded step holds the old launch */
    return CAL_SUCCESS;
}

extern "C" int calSetElementaryProcessGuard2Dr(struct CALModel2D* ca, CALCallbackFunc2D ep, struct CALSubstate2Dr* Q,
                                               int op, CALreal value)
{
    if (!ca || !ca->gpu || op < CAL_GUARD_NONE || op > CAL_GUARD_NE || (op != CAL_GUARD_NONE && !Q)) {
        cal::set_error(CAL_ERROR_INVALID_ARGUMENT, "calSetElementaryProcessGuard2Dr: bad arguments");
        return CAL_ERROR_INVALID_ARGUMENT;
    }
    int b = -1;
    for (int k = 0; k < ca->num_of_elementary_processes; k++)
        if (ca->elementary_processes[k] == ep)
            b = k;
    if (b < 0) {
        cal::set_error(CAL_ERROR_INVALID_ARGUMENT,
                       "calSetElementaryProcessGuard2Dr: not a process added with calAddElementaryProcess2D");
        return CAL_ERROR_INVALID_ARGUMENT;
    }
    int slot = 0;
    if (op != CAL_GUARD_NONE) {
        CalGrid& g = G(ca);
        const uintptr_t h = (uintptr_t)Q, p0 = (uintptr_t)g.pool[CAL_TYPE_R];
        if (!(h >= p0 && h < p0 + 32u * CAL_MAX_SUBSTATES_CORE && ((h - p0) & 31u) == 0 &&
              (int)((h - p0) >> 5) < g.nslot[CAL_TYPE_R] && g.sub[CAL_TYPE_R][(h - p0) >> 5].used)) {
            cal::set_error(CAL_ERROR_INVALID_ARGUMENT, "calSetElementaryProcessGuard2Dr: not a real substate of this model");
            return CAL_ERROR_INVALID_ARGUMENT;
        }
        slot = (int)((h - p0) >> 5);
    }
    ca->gpu->guard_op[b] = op;
    ca->gpu->guard_slot[b] = slot;
    ca->gpu->guard_value[b] = value;
    G(ca).inval_epoch++; /* a recorded step holds the old launch */
    return CAL_SUCCESS;
}

extern "C" int calSetElementaryProcessPure2D(struct CALModel2D* ca, CALCallbackFunc2D ep, CALbyte pure)
{
    if (!ca || !ca->gpu) {
        cal::set_error(CAL_ERROR_INVALID_ARGUMENT, "calSetElementaryProcessPure2D: no model");
        return CAL_ERROR_INVALID_ARGUMENT;
    }
    for (int b = 0; b < ca->num_of_elementary_processes; b++)
        if (ca->elementary_processes[b] == ep) {
            ca->gpu->pure[b] = pure != 0;
            G(ca).nrun = -1; /* re-armed before the next transition */
            return CAL_SUCCESS;
        }
    cal::set_error(CAL_ERROR_INVALID_ARGUMENT,
                   "calSetElementaryProcessPure2D: not a process added with calAddElementaryProcess2D");
    return CAL_ERROR_INVALID_ARGUMENT;
}

/* ======================= host cell accessors ============================ */

#define CAL_CELL_OPS_2D(S, T, TC)                                                                          \
    extern "C" T calGet2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j)              \
    {                                                                                                      \
        G(ca).to_host(TC, slot_of(ca, TC, Q), 0);                                                          \
        return Q->current[(long long)i * ca->columns + j];                                                 \
    }                                                                                                      \
    extern "C" T calGetX2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j, int n)      \
    {                                                                                                      \
        int a, b;                                                                                          \
        if (!neighbor(ca, i, j, n, &a, &b))                                                                \
            return (T)0;                                                                                   \
        return calGet2D##S(ca, Q, a, b);                                                                   \
    }                                                                                                      \
    extern "C" void calSet2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j, T v)      \
    {                                                                                                      \
        int s = slot_of(ca, TC, Q);                                                                        \
        if (!G(ca).to_host(TC, s, 1))                                                                      \
            return;                                                                                        \
        Q->next[(long long)i * ca->columns + j] = v;                                                       \
        G(ca).host_wrote(TC, s, 1);                                                                        \
    }                                                                                                      \
    extern "C" void calSetCurrent2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j, T v) \
    {                                                                                                      \
        int s = slot_of(ca, TC, Q);                                                                        \
        if (!G(ca).to_host(TC, s, 0))                                                                      \
            return;                                                                                        \
        Q->current[(long long)i * ca->columns + j] = v;                                                    \
        G(ca).host_wrote(TC, s, 0);                                                                        \
    }                                                                                                      \
    extern "C" void calInit2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j, T v)     \
    {                                                                                                      \
        int s = slot_of(ca, TC, Q);                                                                        \
        calSetCurrent2D##S(ca, Q, i, j, v);                                                                \
        if (Q->next && G(ca).to_host(TC, s, 1)) {                                                          \
            Q->next[(long long)i * ca->columns + j] = v;                                                   \
            G(ca).host_wrote(TC, s, 1);                                                                    \
        }                                                                                                  \
    }

CAL_CELL_OPS_2D(b, CALbyte, 0)
CAL_CELL_OPS_2D(i, CALint, 1)
CAL_CELL_OPS_2D(r, CALreal, 2)

/* ======================= additions ===================================== */

extern "C" void calSync2D(struct CALModel2D* ca)
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
        int* tmp = (int*)malloc(sizeof(int) * 2 * (size_t)n);
        ca->A.cells = (struct CALCell2D*)malloc(sizeof(struct CALCell2D) * (size_t)n);
        if (!tmp || !ca->A.cells) {
            free(tmp);
            cal::set_error(CAL_ERROR_OUT_OF_MEMORY, "calSync2D active list");
            return;
        }
        if (cal::cuda_ok(cudaMemcpyAsync(tmp, g.d_cells, sizeof(int) * 2 * (size_t)n, cudaMemcpyDeviceToHost, g.stream),
                         "read active list") && g.sync())
            for (int c = 0; c < n; c++) {
                ca->A.cells[c].i = tmp[2 * c];
                ca->A.cells[c].j = tmp[2 * c + 1];
            }
        free(tmp);
    }
}

extern "C" void calMarkHostDirty2D(struct CALModel2D* ca)
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

extern "C" void calMarkDeviceWritten2D(struct CALModel2D* ca)
{
    CalGrid& g = G(ca);
    g.device_wrote_all();
    g.mark_flags_changed(); /* the active flags may have been written too */
    for (int t = 0; t < CAL_NTYPES; t++)
        for (int s = 0; s < g.nslot[t]; s++)
            g.untrack(t, s); /* written outside the library: no change tracking from now on */
}

extern "C" void calFinish2D(struct CALModel2D* ca)
{
    G(ca).sync();
}

extern "C" void* calGetStream2D(struct CALModel2D* ca)
{
    return (void*)G(ca).stream;
}

extern "C" void calGetDeviceActiveCells2D(struct CALModel2D* ca, CALbyte** flags, struct CALCell2D** cells, int** count)
{
    CalGrid& g = G(ca);
    g.to_device_all();
    if (flags)
        *flags = (CALbyte*)g.d_flags;
    if (cells)
        *cells = (struct CALCell2D*)g.d_cells;
    if (count)
        *count = g.d_count;
}

extern "C" int calGetActiveCellCount2D(struct CALModel2D* ca)
{
    CalGrid& g = G(ca);
    int n = 0;
    if (cal::cuda_ok(cudaMemcpyAsync(&n, g.d_count, sizeof(int), cudaMemcpyDeviceToHost, g.stream), "read count"))
        g.sync();
    return n;
}

extern "C" void calFinalize2D(struct CALModel2D* ca)
{
    if (!ca)
        return;
    if (ca->gpu) {
        ca->gpu->g.destroy();
        if (ca->gpu->d_X)
            cudaFree(ca->gpu->d_X);
        if (ca->gpu->d_stage_err)
            cudaFree(ca->gpu->d_stage_err);
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

/* ======================= unsafe operations (cal2DUnsafe.h) ============== */
/* OpenCAL-OMP/source/cal2DUnsafe.c:17-275, on the host mirrors */

#define CAL_UNSAFE_OPS_2D(S, T, TC)                                                                          \
    extern "C" T calGetNext2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j)            \
    {                                                                                                        \
        if (!G(ca).to_host(TC, slot_of(ca, TC, Q), 1))                                                       \
            return (T)0;                                                                                     \
        return Q->next[(long long)i * ca->columns + j];                                                      \
    }                                                                                                        \
    extern "C" T calGetNextX2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j, int n)    \
    {                                                                                                        \
        int a, b;                                                                                            \
        if (!neighbor(ca, i, j, n, &a, &b))                                                                  \
            return (T)0;                                                                                     \
        return calGetNext2D##S(ca, Q, a, b);                                                                 \
    }                                                                                                        \
    extern "C" void calSetX2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j, int n, T v) \
    {                                                                                                        \
        int a, b;                                                                                            \
        if (neighbor(ca, i, j, n, &a, &b))                                                                   \
            calSet2D##S(ca, Q, a, b, v);                                                                     \
    }                                                                                                        \
    extern "C" void calSetCurrentX2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j, int n, \
                                        T v)                                                                 \
    {                                                                                                        \
        int a, b;                                                                                            \
        if (neighbor(ca, i, j, n, &a, &b))                                                                   \
            calSetCurrent2D##S(ca, Q, a, b, v);                                                              \
    }                                                                                                        \
    extern "C" void calInitX2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j, int n, T v) \
    {                                                                                                        \
        int a, b;                                                                                            \
        if (neighbor(ca, i, j, n, &a, &b))                                                                   \
            calInit2D##S(ca, Q, a, b, v);                                                                    \
    }                                                                                                        \
    extern "C" void calAddNext2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j, T v)    \
    {                                                                                                        \
        const int s = slot_of(ca, TC, Q);                                                                    \
        if (!G(ca).to_host(TC, s, 1))                                                                        \
            return;                                                                                          \
        T* p = &Q->next[(long long)i * ca->columns + j];                                                     \
        *p = (T)(*p + v);                                                                                    \
        G(ca).host_wrote(TC, s, 1);                                                                          \
    }                                                                                                        \
    extern "C" void calAddNextX2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* Q, int i, int j, int n, T v) \
    {                                                                                                        \
        int a, b;                                                                                            \
        if (neighbor(ca, i, j, n, &a, &b))                                                                   \
            calAddNext2D##S(ca, Q, a, b, v);                                                                 \
    }

CAL_UNSAFE_OPS_2D(b, CALbyte, 0)
CAL_UNSAFE_OPS_2D(i, CALint, 1)
CAL_UNSAFE_OPS_2D(r, CALreal, 2)
