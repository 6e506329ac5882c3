/*
 * calCommon.h -- scalar types, enums and cell/substate structs shared by the
 * 2D and 3D API of opencal-gb300.
 *
 * Drop-in for OpenCAL-OMP/include/calCommon.h:15-222: same type names, same
 * enumerator values, same public struct fields, so that code written against
 * OpenCAL compiles unchanged.  Substate structs carry two reserved pointers
 * after the reference's {current, next} pair (library bookkeeping; do not
 * touch).
 */
#ifndef calCommon_h
#define calCommon_h

#define CAL_FALSE 0 /* calCommon.h:16 */
#define CAL_TRUE 1  /* calCommon.h:17 */

typedef char CALbyte;   /* calCommon.h:20 */
typedef int CALint;     /* calCommon.h:21 */
typedef double CALreal; /* calCommon.h:22 */

typedef CALbyte CALParameterb;
typedef CALint CALParameteri;
typedef CALreal CALParameterr;

/* calCommon.h:32-35 */
enum CALSpaceBoundaryCondition {
    CAL_SPACE_FLAT = 0, /* out-of-grid neighbours read as 0 (see DESIGN notes in cal2D.h) */
    CAL_SPACE_TOROIDAL
};

/* calCommon.h:40-43 */
enum CALUpdateMode {
    CAL_UPDATE_EXPLICIT = 0,
    CAL_UPDATE_IMPLICIT
};

/* calCommon.h:48-51 */
enum CALOptimization {
    CAL_NO_OPT = 0,
    CAL_OPT_ACTIVE_CELLS
};

/* calCommon.h:53-56 */
enum CALUnsafeState {
    CAL_UNSAFE_ACTIVE,
    CAL_UNSAFE_INACTIVE
};

/* calCommon.h:61: wraps an index that is at most one period out of range */
#define calGetToroidalX(index, size) \
    ((index) < 0 ? ((size) + (index)) : ((index) > ((size)-1) ? ((index) - (size)) : (index)))

/* calCommon.h:71-74 */
struct CALCell2D {
    int i; /* row */
    int j; /* column */
};

/* calCommon.h:84-88 */
struct CALCell3D {
    int i; /* row */
    int j; /* column */
    int k; /* slice */
};

/*
 * Double-buffered substates (calCommon.h:102-134 and 150-185).
 * `current` and `next` are HOST mirrors of the device buffers: the library
 * keeps them coherent through its own accessors (calGet/calSet/calInit/
 * calLoad...); code that writes them directly must call
 * calMarkHostDirty2D/3D afterwards, and code that reads them directly after
 * a run must call calSync2D/3D first.
 */
#define CAL_SUBSTATE_RESERVED void* cal_reserved_[2]

struct CALSubstate2Db { CALbyte* current; CALbyte* next; CAL_SUBSTATE_RESERVED; };
struct CALSubstate2Di { CALint* current; CALint* next; CAL_SUBSTATE_RESERVED; };
struct CALSubstate2Dr { CALreal* current; CALreal* next; CAL_SUBSTATE_RESERVED; };
struct CALSubstate3Db { CALbyte* current; CALbyte* next; CAL_SUBSTATE_RESERVED; };
struct CALSubstate3Di { CALint* current; CALint* next; CAL_SUBSTATE_RESERVED; };
struct CALSubstate3Dr { CALreal* current; CALreal* next; CAL_SUBSTATE_RESERVED; };

/* calCommon.h:193: final_step value that turns the run into a loop */
/* Tiles of the 2D process kernels (library internals, shared by the device
 * header and the engine): CAL_TILE_W columns (one warp per tile row) by
 * CAL_TILE_H rows, one cell per thread of a 256-thread block. */
#define CAL_TILE_W 32
#define CAL_TILE_H 8

#define CAL_RUN_LOOP 0

/* calCommon.h:201-213 */
enum REDUCTION_OPERATION {
    REDUCTION_NONE = 0,
    REDUCTION_MAX,
    REDUCTION_MIN,
    REDUCTION_SUM,
    REDUCTION_PROD,
    REDUCTION_LOGICAL_AND,
    REDUCTION_BINARY_AND,
    REDUCTION_LOGICAL_OR,
    REDUCTION_BINARY_OR,
    REDUCTION_LOGICAL_XOR,
    REDUCTION_BINARY_XOR
};

/* ---- opencal-gb300 additions: error reporting ------------------------ */

/* Every C-ABI call records its outcome; allocating calls still return NULL
 * on failure and loaders CAL_FALSE, as in the reference. */
enum CALError {
    CAL_SUCCESS = 0,
    CAL_ERROR_INVALID_ARGUMENT = 1,
    CAL_ERROR_OUT_OF_MEMORY = 2,
    CAL_ERROR_CUDA = 3,
    CAL_ERROR_NOT_A_DEVICE_PROCESS = 4, /* calAddElementaryProcess given a host-only function */
    CAL_ERROR_LIMIT = 5,                /* too many substates / neighbours / processes */
    CAL_ERROR_TIMEOUT = 6,              /* a bounded device wait gave up */
    CAL_ERROR_IO = 7,
    CAL_ERROR_NOT_CAPTURABLE = 8        /* a step could not be recorded as a CUDA graph */
};

#ifdef __cplusplus
extern "C" {
#endif
enum CALError calGetLastError(void);
const char* calGetErrorString(void);
void calClearError(void);
#ifdef __cplusplus
}
#endif

#endif
