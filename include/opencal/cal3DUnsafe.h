/*
 * cal3DUnsafe.h -- unsafe operations: a process writing or reading cells
 * other than its own (OpenCAL-OMP/include/cal3DUnsafe.h; semantics of
 * OpenCAL-OMP/source/cal3DUnsafe.c:18-245).  Enabled per model with
 * calSetUnsafe3D (cal3D.h).
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
#ifndef cal3DUnsafe_h
#define cal3DUnsafe_h

#include "cal3D.h"

#ifdef __cplusplus
extern "C" {
#endif

void calInitX3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k, int n, CALbyte value);   /* cal3DUnsafe.h:23 */
void calInitX3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k, int n, CALint value);    /* cal3DUnsafe.h:36 */
void calInitX3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k, int n, CALreal value);   /* cal3DUnsafe.h:49 */
CALbyte calGetNext3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k);                    /* cal3DUnsafe.h:63 */
CALint calGetNext3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k);                     /* cal3DUnsafe.h:73 */
CALreal calGetNext3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k);                    /* cal3DUnsafe.h:83 */
CALbyte calGetNextX3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k, int n);            /* cal3DUnsafe.h:95 */
CALint calGetNextX3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k, int n);             /* cal3DUnsafe.h:106 */
CALreal calGetNextX3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k, int n);            /* cal3DUnsafe.h:117 */
void calSetX3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k, int n, CALbyte value);    /* cal3DUnsafe.h:130 */
void calSetX3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k, int n, CALint value);     /* cal3DUnsafe.h:142 */
void calSetX3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k, int n, CALreal value);    /* cal3DUnsafe.h:154 */
void calSetCurrentX3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k, int n, CALbyte value); /* :168 */
void calSetCurrentX3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k, int n, CALint value);  /* :180 */
void calSetCurrentX3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k, int n, CALreal value); /* :192 */
void calAddNext3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k, CALreal value);        /* cal3DUnsafe.c:188 */
void calAddNextX3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, int i, int j, int k, int n, CALreal value); /* cal3DUnsafe.c:198 */
void calAddNext3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k, CALbyte value);        /* cal3DUnsafe.c:207 */
void calAddNextX3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, int i, int j, int k, int n, CALbyte value); /* cal3DUnsafe.c:217 */
void calAddNext3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k, CALint value);         /* cal3DUnsafe.c:227 */
void calAddNextX3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, int i, int j, int k, int n, CALint value);  /* cal3DUnsafe.c:237 */

#ifdef __cplusplus
}
#endif

#if defined(__CUDACC__)
#include "cal3DDevice.cuh"

/* atomic add on a byte: compare-and-swap on its aligned 32-bit word
 * (lock-free: each failed attempt means another thread's add landed) */
#ifndef CAL_UNSAFE_ATOMICS_DEFINED
#define CAL_UNSAFE_ATOMICS_DEFINED
static __device__ __forceinline__ void cal_atomic_add(CALbyte* p, CALbyte v)
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
static __device__ __forceinline__ void cal_atomic_add(CALint* p, CALint v) { atomicAdd(p, v); }
static __device__ __forceinline__ void cal_atomic_add(CALreal* p, CALreal v) { atomicAdd(p, v); }
#endif

template <typename T>
static __device__ __forceinline__ T cal_getnext3D(const struct CALModel3D* ca, int t, const void* q, int i, int j, int k)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    return static_cast<const T*>(m->nxt[t][cal_slot3D(m, t, q)])[cal_lin3D(m, i, j, k)];
}

template <typename T>
static __device__ __forceinline__ T cal_getnextx3D(const struct CALModel3D* ca, int t, const void* q, int i, int j, int k,
                                                   int n)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    int a, b, c;
    if (!cal_nbr3D(m, i, j, k, n, a, b, c))
        return (T)0;
    return static_cast<const T*>(m->nxt[t][cal_slot3D(m, t, q)])[cal_lin3D(m, a, b, c)];
}

/* which = 1: next, 0: current, 2: both */
template <typename T, int WHICH>
static __device__ __forceinline__ void cal_storex3D(const struct CALModel3D* ca, int t, const void* q, int i, int j, int k,
                                                    int n, T v)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    int a, b, c;
    if (!cal_nbr3D(m, i, j, k, n, a, b, c))
        return;
    const int s = cal_slot3D(m, t, q);
    const long long x = cal_lin3D(m, a, b, c);
    if (WHICH != 0 && m->nxt[t][s])
        static_cast<T*>(m->nxt[t][s])[x] = v;
    if (WHICH != 1)
        static_cast<T*>(m->cur[t][s])[x] = v;
    cal_written3D[t * CAL_MAX_SUBSTATES + s] = 1;
}

template <typename T>
static __device__ __forceinline__ void cal_addnext3D(const struct CALModel3D* ca, int t, const void* q, int i, int j, int k,
                                                     T v)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    const int s = cal_slot3D(m, t, q);
    cal_atomic_add(static_cast<T*>(m->nxt[t][s]) + cal_lin3D(m, i, j, k), v);
    cal_written3D[t * CAL_MAX_SUBSTATES + s] = 1;
}

template <typename T>
static __device__ __forceinline__ void cal_addnextx3D(const struct CALModel3D* ca, int t, const void* q, int i, int j, int k,
                                                      int n, T v)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    int a, b, c;
    if (!cal_nbr3D(m, i, j, k, n, a, b, c))
        return;
    const int s = cal_slot3D(m, t, q);
    cal_atomic_add(static_cast<T*>(m->nxt[t][s]) + cal_lin3D(m, a, b, c), v);
    cal_written3D[t * CAL_MAX_SUBSTATES + s] = 1;
}

#ifndef CAL_BUILDING_LIBRARY
#define CAL_HD_UNSAFE_3D(S, T, TC)                                                                            \
    static __host__ __device__ __forceinline__ T cal_hd_getnext3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k) \
    { CAL_HD_BODY((cal_getnext3D<T>(ca, TC, q, i, j, k)), (calGetNext3D##S(ca, q, i, j, k))); }               \
    static __host__ __device__ __forceinline__ T cal_hd_getnextx3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k, int n) \
    { CAL_HD_BODY((cal_getnextx3D<T>(ca, TC, q, i, j, k, n)), (calGetNextX3D##S(ca, q, i, j, k, n))); }       \
    static __host__ __device__ __forceinline__ void cal_hd_setx3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k, int n, T v) \
    { CAL_HD_BODY((cal_storex3D<T, 1>(ca, TC, q, i, j, k, n, v)), (calSetX3D##S(ca, q, i, j, k, n, v))); }    \
    static __host__ __device__ __forceinline__ void cal_hd_setcurx3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k, int n, T v) \
    { CAL_HD_BODY((cal_storex3D<T, 0>(ca, TC, q, i, j, k, n, v)), (calSetCurrentX3D##S(ca, q, i, j, k, n, v))); } \
    static __host__ __device__ __forceinline__ void cal_hd_initx3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k, int n, T v) \
    { CAL_HD_BODY((cal_storex3D<T, 2>(ca, TC, q, i, j, k, n, v)), (calInitX3D##S(ca, q, i, j, k, n, v))); }   \
    static __host__ __device__ __forceinline__ void cal_hd_addnext3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k, T v) \
    { CAL_HD_BODY((cal_addnext3D<T>(ca, TC, q, i, j, k, v)), (calAddNext3D##S(ca, q, i, j, k, v))); }         \
    static __host__ __device__ __forceinline__ void cal_hd_addnextx3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k, int n, T v) \
    { CAL_HD_BODY((cal_addnextx3D<T>(ca, TC, q, i, j, k, n, v)), (calAddNextX3D##S(ca, q, i, j, k, n, v))); }

CAL_HD_UNSAFE_3D(b, CALbyte, CAL_TYPE_B)
CAL_HD_UNSAFE_3D(i, CALint, CAL_TYPE_I)
CAL_HD_UNSAFE_3D(r, CALreal, CAL_TYPE_R)

#define calGetNext3Db cal_hd_getnext3Db
#define calGetNext3Di cal_hd_getnext3Di
#define calGetNext3Dr cal_hd_getnext3Dr
#define calGetNextX3Db cal_hd_getnextx3Db
#define calGetNextX3Di cal_hd_getnextx3Di
#define calGetNextX3Dr cal_hd_getnextx3Dr
#define calSetX3Db cal_hd_setx3Db
#define calSetX3Di cal_hd_setx3Di
#define calSetX3Dr cal_hd_setx3Dr
#define calSetCurrentX3Db cal_hd_setcurx3Db
#define calSetCurrentX3Di cal_hd_setcurx3Di
#define calSetCurrentX3Dr cal_hd_setcurx3Dr
#define calInitX3Db cal_hd_initx3Db
#define calInitX3Di cal_hd_initx3Di
#define calInitX3Dr cal_hd_initx3Dr
#define calAddNext3Db cal_hd_addnext3Db
#define calAddNext3Di cal_hd_addnext3Di
#define calAddNext3Dr cal_hd_addnext3Dr
#define calAddNextX3Db cal_hd_addnextx3Db
#define calAddNextX3Di cal_hd_addnextx3Di
#define calAddNextX3Dr cal_hd_addnextx3Dr
#endif /* CAL_BUILDING_LIBRARY */
#endif /* __CUDACC__ */

#endif
