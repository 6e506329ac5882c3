/*
 * cal3D.h -- 3D cellular automaton (rows x columns x slices).
 *
 * Drop-in for OpenCAL-OMP/include/cal3D.h; same conventions as cal2D.h.
 * Layout is slice-major, k*rows*columns + i*columns + j
 * (OpenCAL-OMP/include/cal3DBuffer.h:131-136); processes visit cells and the
 * active list is ordered by i, then j, then k (OpenCAL-OMP/source/cal3D.c
 * loop order).
 */
#ifndef cal3D_h
#define cal3D_h

#include "calCommon.h"

#ifndef CAL_MAX_SUBSTATES
#define CAL_MAX_SUBSTATES 32
#define CAL_MAX_NEIGHBORS 64
#define CAL_MAX_ELEMENTARY_PROCESSES 32
#endif

/* cal3D.h:27-31 */
enum CALNeighborhood3D {
    CAL_CUSTOM_NEIGHBORHOOD_3D,
    CAL_VON_NEUMANN_NEIGHBORHOOD_3D,
    CAL_MOORE_NEIGHBORHOOD_3D
};

/* cal3D.h:36-42 */
struct CALActiveCells3D {
    CALbyte* flags;
    int* size_next;
    struct CALCell3D* cells;
    int size_current;
    int num_threads;
};

struct CALModel3D;
struct CALGpuModel3D;

/* cal3D.h:47-70 (+ gpu) */
struct CALModel3D {
    int rows;
    int columns;
    int slices;
    enum CALSpaceBoundaryCondition T;
    enum CALOptimization OPTIMIZATION;
    struct CALActiveCells3D A;
    struct CALCell3D* X;
    int sizeof_X;
    enum CALNeighborhood3D X_id;
    struct CALSubstate3Db** pQb_array;
    struct CALSubstate3Di** pQi_array;
    struct CALSubstate3Dr** pQr_array;
    int sizeof_pQb_array;
    int sizeof_pQi_array;
    int sizeof_pQr_array;
    void (**elementary_processes)(struct CALModel3D* ca3D, int i, int j, int k);
    int num_of_elementary_processes;
    enum CALUnsafeState is_safe;
    struct CALGpuModel3D* gpu;
};

/* cal3D.h:75 */
typedef void (*CALCallbackFunc3D)(struct CALModel3D* ca3D, int i, int j, int k);

#ifdef __cplusplus
extern "C" {
#endif

struct CALModel3D* calCADef3D(int rows, int columns, int slices, enum CALNeighborhood3D CAL_NEIGHBORHOOD_3D,
                              enum CALSpaceBoundaryCondition CAL_TOROIDALITY,
                              enum CALOptimization CAL_OPTIMIZATION);                  /* cal3D.h:100 */
void calSetUnsafe3D(struct CALModel3D* ca3D);                                         /* cal3D.h:116 */
void calAddActiveCell3D(struct CALModel3D* ca3D, int i, int j, int k);                /* cal3D.h:119 */
void calAddActiveCellX3D(struct CALModel3D* ca3D, int i, int j, int k, int n);        /* cal3D.h:129 */
void calRemoveActiveCell3D(struct CALModel3D* ca3D, int i, int j, int k);             /* cal3D.h:139 */
void calUpdateActiveCells3D(struct CALModel3D* ca3D);                                 /* cal3D.h:149 */
struct CALCell3D* calAddNeighbor3D(struct CALModel3D* ca3D, int i, int j, int k);     /* cal3D.h:156 */
struct CALSubstate3Db* calAddSubstate3Db(struct CALModel3D* ca3D);                    /* cal3D.h:166 */
struct CALSubstate3Di* calAddSubstate3Di(struct CALModel3D* ca3D);                    /* cal3D.h:171 */
struct CALSubstate3Dr* calAddSubstate3Dr(struct CALModel3D* ca3D);                    /* cal3D.h:176 */
struct CALSubstate3Db* calAddSingleLayerSubstate3Db(struct CALModel3D* ca3D);         /* cal3D.h:185 */
struct CALSubstate3Di* calAddSingleLayerSubstate3Di(struct CALModel3D* ca3D);         /* cal3D.h:192 */
struct CALSubstate3Dr* calAddSingleLayerSubstate3Dr(struct CALModel3D* ca3D);         /* cal3D.h:199 */
CALCallbackFunc3D* calAddElementaryProcess3D(struct CALModel3D* ca3D, CALCallbackFunc3D elementary_process); /* :206 */
void calInitSubstate3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, CALbyte value);     /* cal3D.h:214 */
void calInitSubstate3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, CALint value);      /* cal3D.h:221 */
void calInitSubstate3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, CALreal value);     /* cal3D.h:228 */
void calInitSubstateNext3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, CALbyte value); /* cal3D.h:237 */
void calInitSubstateNext3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, CALint value);  /* cal3D.h:244 */
void calInitSubstateNext3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, CALreal value); /* cal3D.h:251 */
void calUpdateSubstate3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q);                  /* cal3D.h:261 */
void calUpdateSubstate3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q);                  /* cal3D.h:268 */
void calUpdateSubstate3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q);                  /* cal3D.h:274 */
void calApplyElementaryProcess3D(struct CALModel3D* ca3D, CALCallbackFunc3D elementary_process); /* cal3D.h:282 */
void calGlobalTransitionFunction3D(struct CALModel3D* ca3D);                                   /* cal3D.h:291 */
void calUpdate3D(struct CALModel3D* ca3D);                                                     /* cal3D.h:300 */
void calInit3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k, CALbyte value); /* :307 */
void calInit3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k, CALint value);  /* :317 */
void calInit3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k, CALreal value); /* :327 */
CALbyte calGet3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k);     /* cal3D.h:339 */
CALint calGet3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k);      /* cal3D.h:348 */
CALreal calGet3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k);     /* cal3D.h:357 */
CALbyte calGetX3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k, int n); /* :368 */
CALint calGetX3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k, int n);  /* :378 */
CALreal calGetX3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k, int n); /* :388 */
void calSet3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k, CALbyte value); /* :400 */
void calSet3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k, CALint value);  /* :410 */
void calSet3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k, CALreal value); /* :420 */
void calSetCurrent3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k, CALbyte value); /* :433 */
void calSetCurrent3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k, CALint value);  /* :444 */
void calSetCurrent3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k, CALreal value); /* :455 */
void calFinalize3D(struct CALModel3D* ca3D);                                                   /* cal3D.h:466 */

/* ---- opencal-gb300 additions (see cal2D.h) -------------------------- */
void calSync3D(struct CALModel3D* ca3D);
void calMarkHostDirty3D(struct CALModel3D* ca3D);
void calFinish3D(struct CALModel3D* ca3D);
void* calGetStream3D(struct CALModel3D* ca3D);
int calGetActiveCellCount3D(struct CALModel3D* ca3D);
/* host array (rows*columns*slices, the buffer layout) -> both layers on the
 * device, and the current layer -> host array (see cal2D.h) */
void calCopySubstateFromHost3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, const CALbyte* data);
void calCopySubstateFromHost3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, const CALint* data);
void calCopySubstateFromHost3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, const CALreal* data);
void calCopySubstateToHost3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, CALbyte* data);
void calCopySubstateToHost3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, CALint* data);
void calCopySubstateToHost3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, CALreal* data);

struct CALDevModel3D;
typedef int (*CALLaunchFunc3D)(const struct CALDevModel3D* m, int grid_x, int grid_y, void* stream);
int calRegisterElementaryProcess3D(CALCallbackFunc3D host_name, CALLaunchFunc3D launch, const char* name);
typedef CALbyte (*CALStopFunc3D)(struct CALModel3D* ca3D);
typedef int (*CALStopLaunchFunc3D)(const struct CALDevModel3D* m, unsigned long long handle, int use_handle,
                                   int final_step, int* flag, void* stream);
int calRegisterDeviceStopCondition3D(CALStopFunc3D host_name, CALStopLaunchFunc3D launch, const char* name);
void calHostCallOfDeviceProcess3D(const char* name);

#ifdef __cplusplus
}
#endif

#if defined(__CUDACC__)
#include "cal3DDevice.cuh"
#endif

#endif
