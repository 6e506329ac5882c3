/*
 * cal3DReduction.h -- global reductions of a 3D substate (steering / stop
 * conditions).  Drop-in for OpenCAL-OMP/include/cal3DReduction.h: the same
 * functions, computed on the GPU over the substate's current layer.
 *
 * Semantics: the reference folds every cell into the value of cell 0
 * (OpenCAL-OMP/source/cal3DReduction.c:15-170); logical operations give 0/1,
 * binary operations on reals act on (CALint) casts.  Two documented
 * differences: (1) every cell is reduced -- the reference's serial branch
 * stops after `rows` elements (cal3DReduction.c:30) -- and (2) real sums and
 * products use a fixed tree order, deterministic but rounded differently
 * from a left-to-right fold (agreement to ~1e-12 relative for well
 * conditioned data).  Integer, byte, min/max, logical and binary results are
 * exact.  Each call synchronises and returns the value to the host; the
 * *Device variants leave it in device memory without synchronising.
 */
#ifndef cal3DReduction_h
#define cal3DReduction_h

#include "cal3D.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CAL_REDUCTION_DECL_3D(OP)                                                              \
    CALbyte calReductionCompute##OP##3Db(struct CALModel3D* model, struct CALSubstate3Db* substate); \
    CALint calReductionCompute##OP##3Di(struct CALModel3D* model, struct CALSubstate3Di* substate);  \
    CALreal calReductionCompute##OP##3Dr(struct CALModel3D* model, struct CALSubstate3Dr* substate);

/* cal3DReduction.h:20-96 */
CAL_REDUCTION_DECL_3D(Max)
CAL_REDUCTION_DECL_3D(Min)
CAL_REDUCTION_DECL_3D(Sum)
CAL_REDUCTION_DECL_3D(Prod)
CAL_REDUCTION_DECL_3D(LogicalAnd)
CAL_REDUCTION_DECL_3D(BinaryAnd)
CAL_REDUCTION_DECL_3D(LogicalOr)
CAL_REDUCTION_DECL_3D(BinaryOr)
CAL_REDUCTION_DECL_3D(LogicalXor)
CAL_REDUCTION_DECL_3D(BinaryXor)

/* cal3DReduction.h:100-112 */
CALbyte calReductionOperation3Db(struct CALModel3D* model, struct CALSubstate3Db* substate, enum REDUCTION_OPERATION operation);
CALint calReductionOperation3Di(struct CALModel3D* model, struct CALSubstate3Di* substate, enum REDUCTION_OPERATION operation);
CALreal calReductionOperation3Dr(struct CALModel3D* model, struct CALSubstate3Dr* substate, enum REDUCTION_OPERATION operation);
/* cal3DReduction.h:114-116: element `index` of the current layer */
CALbyte getValue3DbAtIndex(struct CALSubstate3Db* substate, CALint index);
CALint getValue3DiAtIndex(struct CALSubstate3Di* substate, CALint index);
CALreal getValue3DrAtIndex(struct CALSubstate3Dr* substate, CALint index);

/* opencal-gb300 additions: the result stays in device memory (`result` is a
 * device pointer), queued on the model's stream, no synchronisation -- for
 * device stop conditions and device-driven runs */
void calReductionOperationDevice3Db(struct CALModel3D* model, struct CALSubstate3Db* substate,
                                    enum REDUCTION_OPERATION operation, CALbyte* result);
void calReductionOperationDevice3Di(struct CALModel3D* model, struct CALSubstate3Di* substate,
                                    enum REDUCTION_OPERATION operation, CALint* result);
void calReductionOperationDevice3Dr(struct CALModel3D* model, struct CALSubstate3Dr* substate,
                                    enum REDUCTION_OPERATION operation, CALreal* result);

#ifdef __cplusplus
}
#endif
#endif
