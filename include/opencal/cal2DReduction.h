/*
 * cal2DReduction.h -- global reductions of a 2D substate (steering / stop
 * conditions).  Drop-in for OpenCAL-OMP/include/cal2DReduction.h: the same
 * functions, computed on the GPU over the substate's current layer.
 *
 * Semantics: the reference folds every cell into the value of cell 0
 * (OpenCAL-OMP/source/cal2DReduction.c:15-170); logical operations give 0/1,
 * binary operations on reals act on (CALint) casts.  Two documented
 * differences: (1) every cell is reduced -- the reference's serial branch
 * stops after `rows` elements (cal2DReduction.c:30) -- and (2) real sums and
 * products use a fixed tree order, deterministic but rounded differently
 * from a left-to-right fold (agreement to ~1e-12 relative for well
 * conditioned data).  Integer, byte, min/max, logical and binary results are
 * exact.  Each call synchronises and returns the value to the host; the
 * *Device variants leave it in device memory without synchronising.
 */
#ifndef cal2DReduction_h
#define cal2DReduction_h

#include "cal2D.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CAL_REDUCTION_DECL_2D(OP)                                                              \
    CALbyte calReductionCompute##OP##2Db(struct CALModel2D* model, struct CALSubstate2Db* substate); \
    CALint calReductionCompute##OP##2Di(struct CALModel2D* model, struct CALSubstate2Di* substate);  \
    CALreal calReductionCompute##OP##2Dr(struct CALModel2D* model, struct CALSubstate2Dr* substate);

/* cal2DReduction.h:20-96 */
CAL_REDUCTION_DECL_2D(Max)
CAL_REDUCTION_DECL_2D(Min)
CAL_REDUCTION_DECL_2D(Sum)
CAL_REDUCTION_DECL_2D(Prod)
CAL_REDUCTION_DECL_2D(LogicalAnd)
CAL_REDUCTION_DECL_2D(BinaryAnd)
CAL_REDUCTION_DECL_2D(LogicalOr)
CAL_REDUCTION_DECL_2D(BinaryOr)
CAL_REDUCTION_DECL_2D(LogicalXor)
CAL_REDUCTION_DECL_2D(BinaryXor)

/* cal2DReduction.h:100-112 */
CALbyte calReductionOperation2Db(struct CALModel2D* model, struct CALSubstate2Db* substate, enum REDUCTION_OPERATION operation);
CALint calReductionOperation2Di(struct CALModel2D* model, struct CALSubstate2Di* substate, enum REDUCTION_OPERATION operation);
CALreal calReductionOperation2Dr(struct CALModel2D* model, struct CALSubstate2Dr* substate, enum REDUCTION_OPERATION operation);
/* cal2DReduction.h:114-116: element `index` of the current layer */
CALbyte getValue2DbAtIndex(struct CALSubstate2Db* substate, CALint index);
CALint getValue2DiAtIndex(struct CALSubstate2Di* substate, CALint index);
CALreal getValue2DrAtIndex(struct CALSubstate2Dr* substate, CALint index);

/* opencal-gb300 additions: the result stays in device memory (`result` is a
 * device pointer), queued on the model's stream, no synchronisation -- for
 * device stop conditions and device-driven runs */
void calReductionOperationDevice2Db(struct CALModel2D* model, struct CALSubstate2Db* substate,
                                    enum REDUCTION_OPERATION operation, CALbyte* result);
void calReductionOperationDevice2Di(struct CALModel2D* model, struct CALSubstate2Di* substate,
                                    enum REDUCTION_OPERATION operation, CALint* result);
void calReductionOperationDevice2Dr(struct CALModel2D* model, struct CALSubstate2Dr* substate,
                                    enum REDUCTION_OPERATION operation, CALreal* result);

#ifdef __cplusplus
}
#endif
#endif
