/*
 * cal2D.h -- 2D cellular automaton: model definition, substates, elementary
 * processes, the global transition and the cell accessors.
 *
 * Drop-in for OpenCAL-OMP/include/cal2D.h (the C function-pointer API of
 * OpenCAL): every function below keeps the reference's name, argument order
 * and meaning; each cites the declaration it replaces.  The work runs on the
 * GPU:
 *   - substates live in device memory, SoA, one buffer per layer; the
 *     `current`/`next` fields of the substate structs are host mirrors kept
 *     coherent by the library (see calCommon.h);
 *   - elementary processes are __device__ functions written with
 *     CAL_ELEMENTARY_PROCESS_2D (cal2DDevice.cuh) in a .cu file; their host
 *     name is what calAddElementaryProcess2D takes, exactly as in OpenCAL;
 *   - calGet/calGetX/calSet/... work both inside device processes (one GPU
 *     thread per cell) and in host code (init, steering, finalize).
 *
 * Semantics kept from the reference (OpenCAL-OMP/source/cal2D.c):
 *   - after every elementary process the substates are updated: the active
 *     cell list is rebuilt (row-major) and next is copied to current for
 *     every registered substate -- on the active cells only when the list is
 *     non-empty (cal2D.c:738-776);
 *   - with active cells on but an empty list, processes visit every cell
 *     (cal2D.c:723-733 tests A.cells, which is NULL when the list is empty);
 *   - hexagonal neighbourhoods shift the neighbour index by 7 on odd
 *     columns (or odd rows for the alternative layout).
 * One deliberate difference: with CAL_SPACE_FLAT a neighbour outside the grid
 * reads as 0 and adding it as an active cell is ignored (the reference reads
 * and writes outside its buffers there, cal2D.c:866-867).
 */
#ifndef cal2D_h
#define cal2D_h

#include "calCommon.h"

/* cal2D.h:31-37 */
enum CALNeighborhood2D {
    CAL_CUSTOM_NEIGHBORHOOD_2D,
    CAL_VON_NEUMANN_NEIGHBORHOOD_2D,
    CAL_MOORE_NEIGHBORHOOD_2D,
    CAL_HEXAGONAL_NEIGHBORHOOD_2D,
    CAL_HEXAGONAL_NEIGHBORHOOD_ALT_2D
};

#define CAL_HEXAGONAL_SHIFT 7 /* cal2D.h:39 */

/* Limits of this implementation (checked; exceeding one records
 * CAL_ERROR_LIMIT). */
#define CAL_MAX_SUBSTATES 32          /* per type, double- and single-layer together */
#define CAL_MAX_NEIGHBORS 64          /* entries of the neighbourhood table */
#define CAL_MAX_ELEMENTARY_PROCESSES 32
#define CAL_MAX_STAGED 8              /* substates a process may declare it reads (staged by TMA) */

/* cal2D.h:44-50.  flags/cells are host mirrors refreshed by calSync2D. */
struct CALActiveCells2D {
    CALbyte* flags;
    int* size_next;
    struct CALCell2D* cells;
    int size_current;
    int num_threads;
};

struct CALModel2D;
/* cal2D.h:56 */
typedef void (*CALCallbackFunc2D)(struct CALModel2D* ca2D, int i, int j);

struct CALGpuModel2D; /* library-private device state */

/* cal2D.h:61-86: same public fields in the same order; `gpu` is appended. */
struct CALModel2D {
    int rows;
    int columns;
    enum CALSpaceBoundaryCondition T;
    enum CALUnsafeState is_safe;
    enum CALOptimization OPTIMIZATION;
    struct CALActiveCells2D A;
    struct CALCell2D* X;
    int sizeof_X;
    enum CALNeighborhood2D X_id;
    struct CALSubstate2Db** pQb_array;
    struct CALSubstate2Di** pQi_array;
    struct CALSubstate2Dr** pQr_array;
    int sizeof_pQb_array;
    int sizeof_pQi_array;
    int sizeof_pQr_array;
    CALCallbackFunc2D* elementary_processes;
    int num_of_elementary_processes;
    struct CALGpuModel2D* gpu;
};

#ifdef __cplusplus
extern "C" {
#endif

/* ---- the reference API --------------------------------------------- */

struct CALModel2D* calCADef2D(int rows, int columns, enum CALNeighborhood2D CAL_NEIGHBORHOOD_2D,
                              enum CALSpaceBoundaryCondition CAL_TOROIDALITY,
                              enum CALOptimization CAL_OPTIMIZATION);           /* cal2D.h:104 */
void calSetUnsafe2D(struct CALModel2D* ca2D);                                  /* cal2D.h:113 */
void calAddActiveCell2D(struct CALModel2D* ca2D, int i, int j);                /* cal2D.h:118 */
void calAddActiveCellX2D(struct CALModel2D* ca2D, int i, int j, int n);        /* cal2D.h:127 */
void calRemoveActiveCell2D(struct CALModel2D* ca2D, int i, int j);             /* cal2D.h:136 */
void calUpdateActiveCells2D(struct CALModel2D* ca2D);                          /* cal2D.h:145 */
struct CALCell2D* calAddNeighbor2D(struct CALModel2D* ca2D, int i, int j);     /* cal2D.h:152 */
struct CALSubstate2Db* calAddSubstate2Db(struct CALModel2D* ca2D);             /* cal2D.h:161 */
struct CALSubstate2Di* calAddSubstate2Di(struct CALModel2D* ca2D);             /* cal2D.h:166 */
struct CALSubstate2Dr* calAddSubstate2Dr(struct CALModel2D* ca2D);             /* cal2D.h:171 */
struct CALSubstate2Db* calAddSingleLayerSubstate2Db(struct CALModel2D* ca2D);  /* cal2D.h:180 */
struct CALSubstate2Di* calAddSingleLayerSubstate2Di(struct CALModel2D* ca2D);  /* cal2D.h:187 */
struct CALSubstate2Dr* calAddSingleLayerSubstate2Dr(struct CALModel2D* ca2D);  /* cal2D.h:194 */
/* cal2D.h:202.  `elementary_process` must be the host name of a process
 * defined with CAL_ELEMENTARY_PROCESS_2D; a plain host function is rejected
 * (NULL, CAL_ERROR_NOT_A_DEVICE_PROCESS) -- there is no CPU fallback. */
CALCallbackFunc2D* calAddElementaryProcess2D(struct CALModel2D* ca2D, CALCallbackFunc2D elementary_process);
void calInitSubstate2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, CALbyte value);     /* cal2D.h:210 */
void calInitSubstate2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, CALint value);      /* cal2D.h:217 */
void calInitSubstate2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, CALreal value);     /* cal2D.h:224 */
void calInitSubstateNext2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, CALbyte value); /* cal2D.h:233 */
void calInitSubstateNext2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, CALint value);  /* cal2D.h:240 */
void calInitSubstateNext2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, CALreal value); /* cal2D.h:247 */
void calUpdateSubstate2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q);                  /* cal2D.h:256 */
void calUpdateSubstate2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q);                  /* cal2D.h:263 */
void calUpdateSubstate2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q);                  /* cal2D.h:269 */
void calApplyElementaryProcess2D(struct CALModel2D* ca2D, CALCallbackFunc2D elementary_process); /* cal2D.h:277 */
void calGlobalTransitionFunction2D(struct CALModel2D* ca2D);                                   /* cal2D.h:287 */
void calUpdate2D(struct CALModel2D* ca2D);                                                     /* cal2D.h:296 */
void calInit2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j, CALbyte value); /* cal2D.h:303 */
void calInit2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j, CALint value);  /* cal2D.h:312 */
void calInit2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j, CALreal value); /* cal2D.h:321 */
CALbyte calGet2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j);            /* cal2D.h:332 */
CALint calGet2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j);             /* cal2D.h:340 */
CALreal calGet2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j);            /* cal2D.h:348 */
CALbyte calGetX2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j, int n);    /* cal2D.h:358 */
CALint calGetX2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j, int n);     /* cal2D.h:367 */
CALreal calGetX2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j, int n);    /* cal2D.h:376 */
void calSet2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j, CALbyte value); /* cal2D.h:387 */
void calSet2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j, CALint value);  /* cal2D.h:396 */
void calSet2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j, CALreal value); /* cal2D.h:405 */
void calSetCurrent2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j, CALbyte value); /* cal2D.h:417 */
void calSetCurrent2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j, CALint value);  /* cal2D.h:427 */
void calSetCurrent2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j, CALreal value); /* cal2D.h:437 */
void calFinalize2D(struct CALModel2D* ca2D);                                                   /* cal2D.h:448 */

/* ---- opencal-gb300 additions --------------------------------------- */

/* Bring every host mirror up to date with the device: substate layers,
 * A.flags, A.cells, A.size_current.  Synchronises the model's stream. */
void calSync2D(struct CALModel2D* ca2D);
/* A caller's array (rows*columns elements, the buffer layout; host or
 * device memory) becomes both layers of a substate on the device -- what
 * calLoadSubstate2D* does with a file -- without passing through the host
 * mirrors; the mirrors become stale.  From pinned host memory or device
 * memory the copy runs asynchronously on the model's stream: keep the array
 * unchanged until the next synchronising call. */
void calCopySubstateFromHost2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, const CALbyte* data);
void calCopySubstateFromHost2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, const CALint* data);
void calCopySubstateFromHost2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, const CALreal* data);
/* The current layer of a substate into a caller's array (host or device
 * memory; synchronises). */
void calCopySubstateToHost2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, CALbyte* data);
void calCopySubstateToHost2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, CALint* data);
void calCopySubstateToHost2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, CALreal* data);
/* Bring the host mirror of one substate's current layer up to date. */
void calSyncSubstate2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q);
void calSyncSubstate2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q);
void calSyncSubstate2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q);
/* Declare that host code wrote the mirrors directly (Q->current[...] = ...,
 * Q->next[...] = ...): every layer's host mirror becomes the authoritative
 * copy and the next device operation uploads it.  After device work the
 * mirrors are stale: call calSync2D before writing only part of them (a
 * program that overwrites them entirely need not). */
void calMarkHostDirty2D(struct CALModel2D* ca2D);
/* Wait for all device work queued on the model. */
void calFinish2D(struct CALModel2D* ca2D);
/* The CUDA stream (cudaStream_t) the model's work is queued on. */
void* calGetStream2D(struct CALModel2D* ca2D);
/* Device buffers of a substate layer (0 = current, 1 = next, 2 = next for a
 * kernel that will overwrite every cell of it, so stale contents left by a
 * swap need no repair), for custom kernels.  A kernel that writes a layer
 * in place must call calMarkDeviceWritten2D. */
void* calGetDeviceBuffer2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int layer);
void* calGetDeviceBuffer2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int layer);
void* calGetDeviceBuffer2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int layer);
void calMarkDeviceWritten2D(struct CALModel2D* ca2D);
/* A custom kernel rewrote the current layer of one substate in place (every
 * cell it changed, consistently with what an update would leave): only the
 * host mirror becomes stale, no next -> current copy is implied. */
void calMarkCurrentWritten2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q);
void calMarkCurrentWritten2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q);
void calMarkCurrentWritten2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q);
/* current <-> next as a pointer exchange (no copy).  Only valid after a
 * kernel has written EVERY cell of next; next then holds stale data, which
 * the library repairs before any partial write reaches it. */
void calSwapSubstate2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q);
void calSwapSubstate2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q);
void calSwapSubstate2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q);
/* Device pointers of the active-cell state: flags (rows*columns bytes), the
 * compacted list and its length (an int in device memory).  Flags written
 * through the pointer are taken into account by the next
 * calUpdateActiveCells2D, or by the next update after calMarkDeviceWritten2D
 * (the updates that follow a process otherwise keep the list when no process
 * changed a flag). */
void calGetDeviceActiveCells2D(struct CALModel2D* ca2D, CALbyte** flags, struct CALCell2D** cells, int** count);
/* Number of active cells, read from the device (synchronises). */
int calGetActiveCellCount2D(struct CALModel2D* ca2D);

/* Active-cell compaction for callers that cannot allocate device memory.
 * No counterpart in the reference.  It computes what calUpdateActiveCells2D
 * computes -- the cells whose flag is set, in row-major order, their linear
 * indices and their number -- from caller-owned device buffers: `flags`
 * (rows*columns bytes, any alignment), `cells` and `linear` (room for every
 * cell) and `count` (one int), all three 4-byte aligned (otherwise
 * CAL_ERROR_INVALID_ARGUMENT and nothing is launched), queued on `stream`
 * (a cudaStream_t, NULL for the default stream).  It allocates nothing: its
 * scratch is a fixed array in device memory owned by the library, so grids
 * are limited to CAL_NOALLOC_MAX_CELLS cells (larger ones return
 * CAL_ERROR_LIMIT), calls whose kernels overlap on the GPU race on that
 * array, and the first call on each device (which looks the array up)
 * should come before any stream capture; the address it looks up is kept,
 * so a cudaDeviceReset after that first call is not supported.  Returns a
 * CALError code. */
#define CAL_NOALLOC_MAX_CELLS 268435456
int calCompactActiveCellsNoAlloc2D(const CALbyte* flags, int rows, int columns, struct CALCell2D* cells,
                                   int* linear, int* count, void* stream);

/* Declares that an elementary process added with calAddElementaryProcess2D
 * is a pure function of the current values of the model's substates over
 * its cell's neighbourhood and of values that do not change during the run
 * (no step number, no parameters changed by steering, no randomness).  Then,
 * in a model without active cells whose substates the library alone writes
 * (no unsafe operations, no device pointers handed out, no swaps), the
 * process kernel of calGlobalTransitionFunction2D skips every 32 x 8 tile
 * where the process changed nothing the last time it ran and where no
 * substate has changed since in that tile or the eight around it: it would
 * change nothing again.  The results are those of the dense run.  The
 * neighbourhood must reach at most 8 rows and 32 columns; every tile is run
 * again after calRunInitSimulation2D and after any write the library cannot
 * follow tile by tile.  `pure` 0 withdraws the declaration.  No counterpart
 * in the reference (a performance declaration; the reference runs every
 * cell).  Returns a CALError code. */
int calSetElementaryProcessPure2D(struct CALModel2D* ca2D, CALCallbackFunc2D elementary_process, CALbyte pure);

/* Declares the substates (up to CAL_MAX_STAGED handles of any type) whose
 * current layer an elementary process reads with calGet / calGetX, and that
 * it does not write in their current layer.  Then, in a model without
 * active cells, the process kernel stages those substates' 32 x 8 tile plus
 * the neighbourhood's halo into shared memory with one TMA tensor copy per
 * substate and tile (cp.async.bulk.tensor, zero fill outside a flat grid;
 * in a toroidal grid the tiles along the border read global memory), and
 * calGet / calGetX read them there.  Substates whose rows are not a
 * multiple of 16 bytes, or neighbourhoods reaching further than 8 rows or
 * (for 8-, 4-, 1-byte cells) 2, 4, 16 columns, keep global reads.  The
 * results are those of global reads.  count 0 withdraws the declaration.
 * No counterpart in the reference (a performance declaration).  Returns a
 * CALError code. */
int calSetElementaryProcessReads2D(struct CALModel2D* ca2D, CALCallbackFunc2D elementary_process,
                                   const void* const* substates, int count);

/* Declares that an elementary process returns at once, writing and
 * changing nothing, on every cell where the current value v of the real
 * substate Q satisfies `v op value`: the early return its body starts with
 * (SCIDDICA-T's flows process: `if (calGet2Dr(ca, Q.h, i, j) <= P.epsilon)
 * return;` is CAL_GUARD_LE, Q.h, P.epsilon).  Then, in a model without
 * active cells, the process kernel tests the guard for the 256 cells of a
 * tile and runs the process only on those that pass, packed into
 * consecutive threads, so that warps are not held by cells that return at
 * once.  The comparison is the C one (a NaN passes every guard but
 * CAL_GUARD_NE), so the results are those of the plain run whenever the
 * declaration is true.  Not applied to processes whose reads are staged
 * (calSetElementaryProcessReads2D).  `value` is taken at the call: declare
 * again after changing the parameter it stands for.  op CAL_GUARD_NONE
 * withdraws the declaration.  No counterpart in the reference (a
 * performance declaration).  Returns a CALError code. */
#define CAL_GUARD_NONE 0
#define CAL_GUARD_LE 1 /* returns where v <= value */
#define CAL_GUARD_LT 2 /* v < value */
#define CAL_GUARD_GE 3 /* v >= value */
#define CAL_GUARD_GT 4 /* v > value */
#define CAL_GUARD_EQ 5 /* v == value */
#define CAL_GUARD_NE 6 /* v != value */
int calSetElementaryProcessGuard2Dr(struct CALModel2D* ca2D, CALCallbackFunc2D elementary_process,
                                    struct CALSubstate2Dr* Q, int op, CALreal value);

/* Registration of device elementary processes (used by
 * CAL_ELEMENTARY_PROCESS_2D; not called directly). */
struct CALDevModel2D;
typedef int (*CALLaunchFunc2D)(const struct CALDevModel2D* m, int grid_x, int grid_y, void* stream);
int calRegisterElementaryProcess2D(CALCallbackFunc2D host_name, CALLaunchFunc2D launch, const char* name);
typedef CALbyte (*CALStopFunc2D)(struct CALModel2D* ca2D);
typedef int (*CALStopLaunchFunc2D)(const struct CALDevModel2D* m, unsigned long long handle, int use_handle,
                                   int final_step, int* flag, void* stream);
int calRegisterDeviceStopCondition2D(CALStopFunc2D host_name, CALStopLaunchFunc2D launch, const char* name);
void calHostCallOfDeviceProcess2D(const char* name);

#ifdef __cplusplus
}
#endif

#if defined(__CUDACC__)
#include "cal2DDevice.cuh"
#endif

#endif
