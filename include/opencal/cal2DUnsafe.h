/*
 * cal2DUnsafe.h -- unsafe operations: a process writing or reading cells
 * other than its own (OpenCAL-OMP/include/cal2DUnsafe.h; semantics of
 * OpenCAL-OMP/source/cal2DUnsafe.c:17-275).  Enabled per model with
 * calSetUnsafe2D (cal2D.h).
 *
 * Host calls act on the host mirrors (made current first, like calSet2D*).
 * In device processes:
 *   calGetNext*, calGetNextX*     read the next layer (no ordering with
 *                                 concurrent writers, as in the reference);
 *   calSetX*, calSetCurrentX*,    store to a neighbour's next / current /
 *   calInitX*                     both layers (last writer wins when several
 *                                 processes write one cell, as in the
 *                                 reference's OpenMP build);
 *   calAddNext*, calAddNextX*     atomic read-modify-write of next (the
 *                                 reference's per-cell lock): every
 *                                 contribution lands, in an unspecified
 *                                 order -- exact for byte and int, rounding
 *                                 order-dependent for real.
 * A neighbour outside a flat grid is ignored (reads give 0).
 */
#ifndef cal2DUnsafe_h
#define cal2DUnsafe_h

#include "cal2D.h"

#ifdef __cplusplus
extern "C" {
#endif

void calInitX2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j, int n, CALbyte value);     /* cal2DUnsafe.h:23 */
void calInitX2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j, int n, CALint value);      /* cal2DUnsafe.h:35 */
void calInitX2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j, int n, CALreal value);     /* cal2DUnsafe.h:47 */
CALbyte calGetNext2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j);                      /* cal2DUnsafe.h:60 */
CALint calGetNext2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j);                       /* cal2DUnsafe.h:69 */
CALreal calGetNext2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j);                      /* cal2DUnsafe.h:78 */
CALbyte calGetNextX2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j, int n);              /* cal2DUnsafe.h:89 */
CALint calGetNextX2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j, int n);               /* cal2DUnsafe.h:99 */
CALreal calGetNextX2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j, int n);              /* cal2DUnsafe.h:109 */
void calSetX2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j, int n, CALbyte value);      /* cal2DUnsafe.h:121 */
void calSetX2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j, int n, CALint value);       /* cal2DUnsafe.h:132 */
void calSetX2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j, int n, CALreal value);      /* cal2DUnsafe.h:143 */
void calSetCurrentX2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j, int n, CALbyte value); /* :156 */
void calSetCurrentX2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j, int n, CALint value);  /* :167 */
void calSetCurrentX2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j, int n, CALreal value); /* :178 */
void calAddNext2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j, CALreal value);          /* cal2DUnsafe.h:186 */
void calAddNextX2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, int i, int j, int n, CALreal value);  /* cal2DUnsafe.h:188 */
void calAddNext2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j, CALbyte value);          /* cal2DUnsafe.c:234 */
void calAddNextX2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, int i, int j, int n, CALbyte value);  /* cal2DUnsafe.c:244 */
void calAddNext2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j, CALint value);           /* cal2DUnsafe.c:255 */
void calAddNextX2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, int i, int j, int n, CALint value);   /* cal2DUnsafe.c:265 */

#ifdef __cplusplus
}
#endif

#if defined(__CUDACC__)
#include "cal2DDevice.cuh"

#ifndef CAL_UNSAFE_ATOMICS_DEFINED
#define CAL_UNSAFE_ATOMICS_DEFINED
/* atomic add on a byte: compare-and-swap on its aligned 32-bit word
 * (lock-free: each failed attempt means another thread's add landed) */
static __device__ __forceinline__ void cal_atomic_add_byte(CALbyte* p, CALbyte v)
{
    unsigned int* w = reinterpret_cast<unsigned int*>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)3);
    const unsigned int sh = (unsigned int)(reinterpret_cast<uintptr_t>(p) & 3) * 8u;
    unsigned int old = *w, assumed;
    do {
        assumed = old;
        const unsigned int b = ((assumed >> sh) + (unsigned int)(unsigned char)v) & 0xffu;
        old = atomicCAS(w, assumed, (assumed & ~(0xffu << sh)) | (b << sh));
    } while (old != assumed);
}
static __device__ __forceinline__ void cal_atomic_add(CALbyte* p, CALbyte v) { cal_atomic_add_byte(p, v); }
static __device__ __forceinline__ void cal_atomic_add(CALint* p, CALint v) { atomicAdd(p, v); }
static __device__ __forceinline__ void cal_atomic_add(CALreal* p, CALreal v) { atomicAdd(p, v); }
#endif

template <typename T>
static __device__ __forceinline__ T cal_getnext2D(const struct CALModel2D* ca, int t, const void* q, int i, int j)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    return static_cast<const T*>(m->nxt[t][cal_slot2D(m, t, q)])[cal_lin2D(m, i, j)];
}

template <typename T>
static __device__ __forceinline__ T cal_getnextx2D(const struct CALModel2D* ca, int t, const void* q, int i, int j, int n)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    int a, b;
    if (!cal_nbr2D(m, i, j, n, a, b))
        return (T)0;
    return static_cast<const T*>(m->nxt[t][cal_slot2D(m, t, q)])[cal_lin2D(m, a, b)];
}

/* which = 1: next, 0: current, 2: both */
template <typename T, int WHICH>
static __device__ __forceinline__ void cal_storex2D(const struct CALModel2D* ca, int t, const void* q, int i, int j, int n,
                                                    T v)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    int a, b;
    if (!cal_nbr2D(m, i, j, n, a, b))
        return;
    const int s = cal_slot2D(m, t, q);
    const long long c = cal_lin2D(m, a, b);
    if (WHICH != 0 && m->nxt[t][s])
        static_cast<T*>(m->nxt[t][s])[c] = v;
    if (WHICH != 1)
        static_cast<T*>(m->cur[t][s])[c] = v;
    cal_written2D[t * CAL_MAX_SUBSTATES + s] = 1;
    cal_untracked2D[t * CAL_MAX_SUBSTATES + s] = 1; /* another cell's tile: the update copies the whole substate */
}

template <typename T>
static __device__ __forceinline__ void cal_addnext2D(const struct CALModel2D* ca, int t, const void* q, int i, int j, T v)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    const int s = cal_slot2D(m, t, q);
    cal_atomic_add(static_cast<T*>(m->nxt[t][s]) + cal_lin2D(m, i, j), v);
    cal_written2D[t * CAL_MAX_SUBSTATES + s] = 1;
    cal_untracked2D[t * CAL_MAX_SUBSTATES + s] = 1; /* other threads add into the same cell */
}

template <typename T>
static __device__ __forceinline__ void cal_addnextx2D(const struct CALModel2D* ca, int t, const void* q, int i, int j, int n,
                                                      T v)
{
    const struct CALDevModel2D* m = cal_dm2D(ca);
    int a, b;
    if (!cal_nbr2D(m, i, j, n, a, b))
        return;
    const int s = cal_slot2D(m, t, q);
    cal_atomic_add(static_cast<T*>(m->nxt[t][s]) + cal_lin2D(m, a, b), v);
    cal_written2D[t * CAL_MAX_SUBSTATES + s] = 1;
    cal_untracked2D[t * CAL_MAX_SUBSTATES + s] = 1; /* another cell's tile */
}

#ifndef CAL_BUILDING_LIBRARY
#define CAL_HD_UNSAFE_2D(S, T, TC)                                                                            \
    static __host__ __device__ __forceinline__ T cal_hd_getnext2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j) \
    { CAL_HD_BODY((cal_getnext2D<T>(ca, TC, q, i, j)), (calGetNext2D##S(ca, q, i, j))); }                     \
    static __host__ __device__ __forceinline__ T cal_hd_getnextx2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j, int n) \
    { CAL_HD_BODY((cal_getnextx2D<T>(ca, TC, q, i, j, n)), (calGetNextX2D##S(ca, q, i, j, n))); }             \
    static __host__ __device__ __forceinline__ void cal_hd_setx2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j, int n, T v) \
    { CAL_HD_BODY((cal_storex2D<T, 1>(ca, TC, q, i, j, n, v)), (calSetX2D##S(ca, q, i, j, n, v))); }          \
    static __host__ __device__ __forceinline__ void cal_hd_setcurx2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j, int n, T v) \
    { CAL_HD_BODY((cal_storex2D<T, 0>(ca, TC, q, i, j, n, v)), (calSetCurrentX2D##S(ca, q, i, j, n, v))); }   \
    static __host__ __device__ __forceinline__ void cal_hd_initx2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j, int n, T v) \
    { CAL_HD_BODY((cal_storex2D<T, 2>(ca, TC, q, i, j, n, v)), (calInitX2D##S(ca, q, i, j, n, v))); }         \
    static __host__ __device__ __forceinline__ void cal_hd_addnext2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j, T v) \
    { CAL_HD_BODY((cal_addnext2D<T>(ca, TC, q, i, j, v)), (calAddNext2D##S(ca, q, i, j, v))); }               \
    static __host__ __device__ __forceinline__ void cal_hd_addnextx2D##S(struct CALModel2D* ca, struct CALSubstate2D##S* q, int i, int j, int n, T v) \
    { CAL_HD_BODY((cal_addnextx2D<T>(ca, TC, q, i, j, n, v)), (calAddNextX2D##S(ca, q, i, j, n, v))); }

CAL_HD_UNSAFE_2D(b, CALbyte, CAL_TYPE_B)
CAL_HD_UNSAFE_2D(i, CALint, CAL_TYPE_I)
CAL_HD_UNSAFE_2D(r, CALreal, CAL_TYPE_R)

#define calGetNext2Db cal_hd_getnext2Db
#define calGetNext2Di cal_hd_getnext2Di
#define calGetNext2Dr cal_hd_getnext2Dr
#define calGetNextX2Db cal_hd_getnextx2Db
#define calGetNextX2Di cal_hd_getnextx2Di
#define calGetNextX2Dr cal_hd_getnextx2Dr
#define calSetX2Db cal_hd_setx2Db
#define calSetX2Di cal_hd_setx2Di
#define calSetX2Dr cal_hd_setx2Dr
#define calSetCurrentX2Db cal_hd_setcurx2Db
#define calSetCurrentX2Di cal_hd_setcurx2Di
#define calSetCurrentX2Dr cal_hd_setcurx2Dr
#define calInitX2Db cal_hd_initx2Db
#define calInitX2Di cal_hd_initx2Di
#define calInitX2Dr cal_hd_initx2Dr
#define calAddNext2Db cal_hd_addnext2Db
#define calAddNext2Di cal_hd_addnext2Di
#define calAddNext2Dr cal_hd_addnext2Dr
#define calAddNextX2Db cal_hd_addnextx2Db
#define calAddNextX2Di cal_hd_addnextx2Di
#define calAddNextX2Dr cal_hd_addnextx2Dr
#endif /* CAL_BUILDING_LIBRARY */
#endif /* __CUDACC__ */

#endif
