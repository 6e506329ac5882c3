/*
 * cal_oracle.h -- CPU restatement of OpenCAL's serial global-transition
 * semantics.  TEST INFRASTRUCTURE ONLY: the parity tests, smoke() and the
 * bench's CPU-baseline leg use it as the checker.  The product library never
 * links or calls it.
 *
 * What is restated (OpenCAL-OMP, built without OpenMP, is the reference):
 *   - model definition and the predefined neighbourhoods
 *       OpenCAL-OMP/source/cal2D.c:28-166, OpenCAL-OMP/source/cal3D.c:29-105
 *   - double-buffered substates, single-layer substates
 *       OpenCAL-OMP/source/cal2D.c:470-596
 *   - apply an elementary process to every cell, or to the active-cell list
 *       OpenCAL-OMP/source/cal2D.c:717-734
 *   - global transition = for each EP { apply; update }  cal2D.c:738-754
 *   - update = rebuild the active list (row-major scan), then copy
 *     next->current of every registered substate (active cells only when the
 *     list is non-empty)                       cal2D.c:758-776, 382-440;
 *                                              cal2DBuffer.c:44-160
 *   - add/remove active cells (count changes only on a real flag change)
 *                                              cal2D.c:333-380
 *   - cell accessors incl. toroidal wrap and the hexagonal odd-column /
 *     odd-row shift of 7                       cal2D.c:780-930, calCommon.h:56
 *   - run loop: init (+update), steps initial..final inclusive, steering
 *     (+update), stop condition, finalize (+update)
 *                                              OpenCAL-OMP/source/cal2DRun.c:77-139
 *
 * One deliberate difference: with CAL_SPACE_FLAT the reference computes
 * (i+di)*columns+(j+dj) unchecked and so reads outside the grid
 * (cal2D.c:866-867).  Here an out-of-grid neighbour reads as 0 and adding an
 * out-of-grid active cell is ignored -- the same definition the CUDA library
 * uses.  On inputs whose non-zero state stays two cells away from the edges
 * both definitions give identical results.
 */
#ifndef CAL_ORACLE_H
#define CAL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_SUBSTATES 64
#define ORC_MAX_X 128
#define ORC_MAX_EP 16
#define ORC_HEX_SHIFT 7

enum { ORC_B = 0, ORC_I = 1, ORC_R = 2 };
enum { ORC_NB_CUSTOM = 0, ORC_NB_VN = 1, ORC_NB_MOORE = 2, ORC_NB_HEX = 3, ORC_NB_HEX_ALT = 4 };

typedef struct orc_sub {
    void* cur;
    void* nxt; /* NULL for single-layer substates */
    int type;
} orc_sub;

struct orc_ca;
typedef void (*orc_ep2)(struct orc_ca*, int, int);
typedef void (*orc_ep3)(struct orc_ca*, int, int, int);

typedef struct orc_ca {
    int dim; /* 2 or 3 */
    int rows, cols, slices;
    int toroidal;
    int nbhd;
    int ac; /* active-cell optimisation on */
    int nx;
    int xo[ORC_MAX_X][3]; /* neighbour offsets (di, dj, dk) */
    orc_sub* sub[ORC_MAX_SUBSTATES];
    int nsub;
    orc_sub* single[ORC_MAX_SUBSTATES];
    int nsingle;
    orc_ep2 ep2[ORC_MAX_EP];
    orc_ep3 ep3[ORC_MAX_EP];
    int nep;
    /* active cells */
    unsigned char* flags;
    long pending;   /* sum of +1/-1 flag transitions since the last rebuild */
    long size;      /* reference's A.size_current */
    int* cells;     /* list, 2 or 3 ints per cell; NULL <=> empty list */
    long ncells;
    int error;      /* set when the flag count and the tracked size disagree */
} orc_ca;

/* definition */
orc_ca* orc_def2d(int rows, int cols, int nbhd, int toroidal, int ac);
orc_ca* orc_def3d(int rows, int cols, int slices, int nbhd, int toroidal, int ac);
void orc_add_neighbor(orc_ca* m, int di, int dj, int dk);
orc_sub* orc_add_sub(orc_ca* m, int type);
orc_sub* orc_add_single(orc_ca* m, int type);
void orc_add_ep2(orc_ca* m, orc_ep2 ep);
void orc_add_ep3(orc_ca* m, orc_ep3 ep);
void orc_free(orc_ca* m);

/* linear index of (i,j,k) in the buffer layout: i*cols+j (2D),
 * k*rows*cols + i*cols + j (3D, OpenCAL-OMP/include/cal3DBuffer.h:136) */
long orc_index(const orc_ca* m, int i, int j, int k);

/* resolve neighbour n of (i,j,k); returns 0 when it lies outside a flat grid */
int orc_neighbor(const orc_ca* m, int i, int j, int k, int n, int* oi, int* oj, int* ok);

/* cell accessors (k ignored in 2D) */
double orc_get(const orc_ca* m, const orc_sub* q, int i, int j, int k);
double orc_getx(const orc_ca* m, const orc_sub* q, int i, int j, int k, int n);
void orc_set(orc_ca* m, orc_sub* q, int i, int j, int k, double v);
void orc_set_cur(orc_ca* m, orc_sub* q, int i, int j, int k, double v);
void orc_init_cell(orc_ca* m, orc_sub* q, int i, int j, int k, double v);

/* unsafe operations (cal2DUnsafe.h / cal3DUnsafe.h) */
double orc_get_next(const orc_ca* m, const orc_sub* q, int i, int j, int k);
double orc_getx_next(const orc_ca* m, const orc_sub* q, int i, int j, int k, int n);
void orc_setx(orc_ca* m, orc_sub* q, int i, int j, int k, int n, double v);
void orc_setx_cur(orc_ca* m, orc_sub* q, int i, int j, int k, int n, double v);
void orc_initx(orc_ca* m, orc_sub* q, int i, int j, int k, int n, double v);
void orc_add_next(orc_ca* m, orc_sub* q, int i, int j, int k, double v);
void orc_add_nextx(orc_ca* m, orc_sub* q, int i, int j, int k, int n, double v);

/* whole-substate operations */
void orc_init_sub(orc_ca* m, orc_sub* q, double v);      /* calInitSubstate2D* */
void orc_init_sub_next(orc_ca* m, orc_sub* q, double v); /* calInitSubstateNext2D* */
void orc_update_sub(orc_ca* m, orc_sub* q);              /* calUpdateSubstate2D* */
void orc_load(orc_ca* m, orc_sub* q, const void* data);  /* current <- data, next <- current */
void orc_store(const orc_ca* m, const orc_sub* q, void* data);

/* active cells */
void orc_add_active(orc_ca* m, int i, int j, int k);
void orc_add_active_x(orc_ca* m, int i, int j, int k, int n);
void orc_remove_active(orc_ca* m, int i, int j, int k);
void orc_update_active(orc_ca* m);

/* transition */
void orc_apply(orc_ca* m, int b);
void orc_update(orc_ca* m);
void orc_transition(orc_ca* m);

/* run loop (cal2DRun.c:16-139), implicit update mode when implicit != 0 */
typedef struct orc_run {
    orc_ca* m;
    int step, initial, final_;
    int implicit;
    void (*init)(orc_ca*);
    void (*transition)(orc_ca*);
    void (*steering)(orc_ca*);
    int (*stop)(orc_ca*);
    void (*finalize)(orc_ca*);
} orc_run;

void orc_run_init(orc_run* r);
int orc_run_step(orc_run* r); /* returns 0 when the stop condition fired */
void orc_run_finalize(orc_run* r);
void orc_run_all(orc_run* r);

#ifdef __cplusplus
}
#endif
/* a reduction of cal2DReduction.h over rows x cols values (kind: 0 byte,
 * 1 int, 2 real) */
int orc_reduce2d(int kind, int rows, int cols, const void* data, int op, double* out);

/* plain SCIDDICA-T on a flat grid with the mass leaving the grid per step
 * (outflux[steps]) and the first step after which the two-cell edge band
 * holds h != 0 (edge_step, -1 if never) */
int orc_sciddicaT_trace(int rows, int cols, int steps, double p_r, double p_eps, const double* z0, const double* h0,
                        double* z_out, double* h_out, double* outflux, int* edge_step);

/* substate text files in the reference's format (dim 2 or 3; kind: 0 byte,
 * 1 int, 2 real; 3D data slice-major) */
int orc_save_text(int dim, int kind, int rows, int cols, int slices, const void* data, const char* path);
int orc_load_text(int dim, int kind, int rows, int cols, int slices, void* data, const char* path);

#endif
