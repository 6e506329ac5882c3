/*
 * cal3DDevice.cuh -- device side of the 3D API (see cal2DDevice.cuh for the
 * design: handle pools, launch descriptor in constant memory, one thread
 * per cell).  Usage:
 *
 *     CAL_ELEMENTARY_PROCESS_3D(rule)(struct CALModel3D* ca, int i, int j, int k) { ... }
 */
#ifndef cal3DDevice_cuh
#define cal3DDevice_cuh

#include <cuda_runtime.h>
#include <stdint.h>

#ifndef CAL_TYPE_B
#define CAL_TYPE_B 0
#define CAL_TYPE_I 1
#define CAL_TYPE_R 2
#define CAL_HANDLE_SHIFT 5
#define CAL_EP_THREADS 256
#endif

struct CALDevModel3D {
    struct CALModel3D model;
    unsigned long long pool[3];
    void* cur[3][CAL_MAX_SUBSTATES];
    void* nxt[3][CAL_MAX_SUBSTATES];
    unsigned int* dirty;
    int* step; /* current step of a device-driven run (calRunDevice3D) */
    CALbyte* flags;
    struct CALCell3D* cells;
    int* count;
    int rows, cols, slices;
    int toroidal;
    int use_list;
    int nx;
    int xi[CAL_MAX_NEIGHBORS];
    int xj[CAL_MAX_NEIGHBORS];
    int xk[CAL_MAX_NEIGHBORS];
};

#if defined(__CUDACC__)

static __shared__ unsigned char cal_written3D[3 * CAL_MAX_SUBSTATES];

/* A device process receives a kernel-local copy of the model's public part
 * (cal_model_view3D) whose `gpu` field points at the launch descriptor. */
static __device__ __forceinline__ const struct CALDevModel3D* cal_dm3D(const struct CALModel3D* ca)
{
    return reinterpret_cast<const struct CALDevModel3D*>(ca->gpu);
}

/* NX > 0: the neighbourhood's size as a compile-time constant (fixed-count
 * loops over ca->sizeof_X, per-neighbour arrays in registers) */
template <int NX>
static __device__ __forceinline__ struct CALModel3D cal_model_view3D(const struct CALDevModel3D& m)
{
    struct CALModel3D v = m.model;
    if (NX > 0)
        v.sizeof_X = NX;
    v.gpu = reinterpret_cast<struct CALGpuModel3D*>(const_cast<struct CALDevModel3D*>(&m));
    return v;
}

static __device__ __forceinline__ int cal_slot3D(const struct CALDevModel3D* m, int t, const void* q)
{
    return (int)(((unsigned long long)(uintptr_t)q - m->pool[t]) >> CAL_HANDLE_SHIFT);
}

static __device__ __forceinline__ long long cal_lin3D(const struct CALDevModel3D* m, int i, int j, int k)
{
    return ((long long)k * m->rows + i) * m->cols + j;
}

static __device__ __forceinline__ bool cal_nbr3D(const struct CALDevModel3D* m, int i, int j, int k, int n,
                                                 int& ni, int& nj, int& nk)
{
    ni = i + m->xi[n];
    nj = j + m->xj[n];
    nk = k + m->xk[n];
    if (m->toroidal) {
        ni = ni < 0 ? ni + m->rows : (ni >= m->rows ? ni - m->rows : ni);
        nj = nj < 0 ? nj + m->cols : (nj >= m->cols ? nj - m->cols : nj);
        nk = nk < 0 ? nk + m->slices : (nk >= m->slices ? nk - m->slices : nk);
        return true;
    }
    return (unsigned)ni < (unsigned)m->rows && (unsigned)nj < (unsigned)m->cols && (unsigned)nk < (unsigned)m->slices;
}

template <typename T>
static __device__ __forceinline__ T cal_get3D(const struct CALModel3D* ca, int t, const void* q, int i, int j, int k)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    return static_cast<const T*>(m->cur[t][cal_slot3D(m, t, q)])[cal_lin3D(m, i, j, k)];
}

template <typename T>
static __device__ __forceinline__ T cal_getx3D(const struct CALModel3D* ca, int t, const void* q, int i, int j, int k, int n)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    int a, b, c;
    if (!cal_nbr3D(m, i, j, k, n, a, b, c))
        return (T)0;
    return static_cast<const T*>(m->cur[t][cal_slot3D(m, t, q)])[cal_lin3D(m, a, b, c)];
}

template <typename T>
static __device__ __forceinline__ void cal_set3D(const struct CALModel3D* ca, int t, const void* q, int i, int j, int k, T v)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    int s = cal_slot3D(m, t, q);
    static_cast<T*>(m->nxt[t][s])[cal_lin3D(m, i, j, k)] = v;
    cal_written3D[t * CAL_MAX_SUBSTATES + s] = 1;
}

template <typename T>
static __device__ __forceinline__ void cal_setcur3D(const struct CALModel3D* ca, int t, const void* q, int i, int j, int k, T v)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    int s = cal_slot3D(m, t, q);
    static_cast<T*>(m->cur[t][s])[cal_lin3D(m, i, j, k)] = v;
    cal_written3D[t * CAL_MAX_SUBSTATES + s] = 1;
}

template <typename T>
static __device__ __forceinline__ void cal_init3D(const struct CALModel3D* ca, int t, const void* q, int i, int j, int k, T v)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    int s = cal_slot3D(m, t, q);
    long long c = cal_lin3D(m, i, j, k);
    static_cast<T*>(m->cur[t][s])[c] = v;
    if (m->nxt[t][s])
        static_cast<T*>(m->nxt[t][s])[c] = v;
    cal_written3D[t * CAL_MAX_SUBSTATES + s] = 1;
}

static __device__ __forceinline__ void cal_addactive3D(const struct CALModel3D* ca, int i, int j, int k)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    if ((unsigned)i < (unsigned)m->rows && (unsigned)j < (unsigned)m->cols && (unsigned)k < (unsigned)m->slices)
        m->flags[cal_lin3D(m, i, j, k)] = 1;
}

static __device__ __forceinline__ void cal_addactivex3D(const struct CALModel3D* ca, int i, int j, int k, int n)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    int a, b, c;
    if (cal_nbr3D(m, i, j, k, n, a, b, c))
        m->flags[cal_lin3D(m, a, b, c)] = 1;
}

static __device__ __forceinline__ void cal_removeactive3D(const struct CALModel3D* ca, int i, int j, int k)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    m->flags[cal_lin3D(m, i, j, k)] = 0;
}

static __device__ __forceinline__ int calRunGetStep3D(const struct CALModel3D* ca)
{
    return *cal_dm3D(ca)->step;
}

static __device__ __forceinline__ int calGetActiveCellCountDevice3D(const struct CALModel3D* ca)
{
    const struct CALDevModel3D* m = cal_dm3D(ca);
    return m->count ? *m->count : 0;
}

/* device stop condition kernel of a device-driven 3D run (see cal2DDevice.cuh) */
/* the largest step a device-driven run executes: past it the loop ends and
 * the second word of the step counter is set (the host reports an error) */
#ifndef CAL_DEVICE_LOOP_MAX_STEP
#define CAL_DEVICE_LOOP_MAX_STEP (1 << 26)
#endif

template <CALbyte (*STOP)(struct CALModel3D*)>
__global__ void cal_stop3D_kernel(const __grid_constant__ struct CALDevModel3D m, cudaGraphConditionalHandle h,
                                  int use_handle, int final_step, int* flag)
{
    struct CALModel3D view = cal_model_view3D<0>(m);
    const bool stop = STOP(&view) != 0;
    int again = 0;
    if (!stop) {
        const int next = *m.step + 1;
        *m.step = next;
        again = (final_step == CAL_RUN_LOOP || next <= final_step) ? 1 : 0;
        if (again && next > CAL_DEVICE_LOOP_MAX_STEP) {
            again = 0; /* a device-driven run never loops without bound */
            m.step[1] = 1;
        }
    }
    *flag = again;
    if (use_handle)
        cudaGraphSetConditional(h, (unsigned)again);
}

template <CALbyte (*STOP)(struct CALModel3D*)>
static int cal_launch_stop3D(const struct CALDevModel3D* m, unsigned long long handle, int use_handle, int final_step,
                             int* flag, void* stream)
{
    cal_stop3D_kernel<STOP><<<1, 1, 0, (cudaStream_t)stream>>>(*m, (cudaGraphConditionalHandle)handle, use_handle,
                                                                final_step, flag);
    return (int)cudaGetLastError();
}

#define CAL_DEVICE_STOP_CONDITION_3D(NAME)                                                              \
    static __device__ __forceinline__ CALbyte NAME##_cal_device_(struct CALModel3D*);                 \
    extern "C" CALbyte NAME(struct CALModel3D* ca3D_)                                                   \
    {                                                                                                   \
        (void)ca3D_;                                                                                    \
        calHostCallOfDeviceProcess3D(#NAME);                                                            \
        return CAL_FALSE;                                                                               \
    }                                                                                                   \
    static const int NAME##_cal_registered_ =                                                           \
        calRegisterDeviceStopCondition3D(NAME, cal_launch_stop3D<NAME##_cal_device_>, #NAME);           \
    static __device__ __forceinline__ CALbyte NAME##_cal_device_

/* one elementary process over every cell (lines of j for each (k, i)) or
 * over the active list when it is non-empty (cal3D.c:658-674) */
template <void (*EP)(struct CALModel3D*, int, int, int), int NX>
__global__ void __launch_bounds__(CAL_EP_THREADS) cal_ep3D_kernel(const __grid_constant__ struct CALDevModel3D m)
{
    for (int t = threadIdx.x; t < 3 * CAL_MAX_SUBSTATES; t += blockDim.x)
        cal_written3D[t] = 0;
    __syncthreads();
    struct CALModel3D view = cal_model_view3D<NX>(m);
    struct CALModel3D* ca = &view;
    const int listed = m.use_list ? *m.count : 0;
    if (listed > 0) {
        const int stride = gridDim.x * gridDim.y * blockDim.x;
        for (int n = (blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x; n < listed; n += stride) {
            const struct CALCell3D c = m.cells[n];
            EP(ca, c.i, c.j, c.k);
        }
    } else {
        const int lines = m.rows * m.slices;
        for (int q = blockIdx.y; q < lines; q += gridDim.y) {
            const int k = q / m.rows, i = q - k * m.rows;
            for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m.cols; j += gridDim.x * blockDim.x)
                EP(ca, i, j, k);
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 3 * CAL_MAX_SUBSTATES; t += blockDim.x) {
        /* the atomic only where the bit is not already set (every block of a
         * dense launch writes the same bits) */
        const unsigned bit = 1u << (t % CAL_MAX_SUBSTATES);
        if (cal_written3D[t] && !(*(volatile const unsigned*)&m.dirty[t / CAL_MAX_SUBSTATES] & bit))
            atomicOr(&m.dirty[t / CAL_MAX_SUBSTATES], bit);
    }
}

/* one kernel per common neighbourhood size (von Neumann 7, Moore 27) and
 * a generic one for the others */
template <void (*EP)(struct CALModel3D*, int, int, int)>
static int cal_launch_ep3D(const struct CALDevModel3D* m, int gx, int gy, void* stream)
{
    const dim3 grid(gx, gy);
    cudaStream_t st = (cudaStream_t)stream;
    switch (m->model.sizeof_X) {
    case 7: cal_ep3D_kernel<EP, 7><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
    case 27: cal_ep3D_kernel<EP, 27><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
    default: cal_ep3D_kernel<EP, 0><<<grid, CAL_EP_THREADS, 0, st>>>(*m); break;
    }
    return (int)cudaGetLastError();
}

#define CAL_ELEMENTARY_PROCESS_3D(NAME)                                                                 \
    static __device__ __forceinline__ void NAME##_cal_device_(struct CALModel3D*, int, int, int);     \
    extern "C" void NAME(struct CALModel3D* ca3D_, int i_, int j_, int k_)                              \
    {                                                                                                   \
        (void)ca3D_; (void)i_; (void)j_; (void)k_;                                                      \
        calHostCallOfDeviceProcess3D(#NAME);                                                            \
    }                                                                                                   \
    static const int NAME##_cal_registered_ =                                                           \
        calRegisterElementaryProcess3D(NAME, cal_launch_ep3D<NAME##_cal_device_>, #NAME);               \
    static __device__ __forceinline__ void NAME##_cal_device_

#ifndef CAL_BUILDING_LIBRARY
#ifndef CAL_HD_BODY
#ifdef __CUDA_ARCH__
#define CAL_HD_BODY(dev, host) return dev
#else
#define CAL_HD_BODY(dev, host) return host
#endif
#endif

#define CAL_HD_ACCESSORS_3D(S, T, TC)                                                                       \
    static __host__ __device__ __forceinline__ T cal_hd_get3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k) \
    { CAL_HD_BODY((cal_get3D<T>(ca, TC, q, i, j, k)), (calGet3D##S(ca, q, i, j, k))); }                     \
    static __host__ __device__ __forceinline__ T cal_hd_getx3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k, int n) \
    { CAL_HD_BODY((cal_getx3D<T>(ca, TC, q, i, j, k, n)), (calGetX3D##S(ca, q, i, j, k, n))); }             \
    static __host__ __device__ __forceinline__ void cal_hd_set3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k, T v) \
    { CAL_HD_BODY((cal_set3D<T>(ca, TC, q, i, j, k, v)), (calSet3D##S(ca, q, i, j, k, v))); }               \
    static __host__ __device__ __forceinline__ void cal_hd_setcur3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k, T v) \
    { CAL_HD_BODY((cal_setcur3D<T>(ca, TC, q, i, j, k, v)), (calSetCurrent3D##S(ca, q, i, j, k, v))); }     \
    static __host__ __device__ __forceinline__ void cal_hd_init3D##S(struct CALModel3D* ca, struct CALSubstate3D##S* q, int i, int j, int k, T v) \
    { CAL_HD_BODY((cal_init3D<T>(ca, TC, q, i, j, k, v)), (calInit3D##S(ca, q, i, j, k, v))); }

CAL_HD_ACCESSORS_3D(b, CALbyte, CAL_TYPE_B)
CAL_HD_ACCESSORS_3D(i, CALint, CAL_TYPE_I)
CAL_HD_ACCESSORS_3D(r, CALreal, CAL_TYPE_R)

static __host__ __device__ __forceinline__ void cal_hd_addactive3D(struct CALModel3D* ca, int i, int j, int k)
{ CAL_HD_BODY(cal_addactive3D(ca, i, j, k), calAddActiveCell3D(ca, i, j, k)); }
static __host__ __device__ __forceinline__ void cal_hd_addactivex3D(struct CALModel3D* ca, int i, int j, int k, int n)
{ CAL_HD_BODY(cal_addactivex3D(ca, i, j, k, n), calAddActiveCellX3D(ca, i, j, k, n)); }
static __host__ __device__ __forceinline__ void cal_hd_removeactive3D(struct CALModel3D* ca, int i, int j, int k)
{ CAL_HD_BODY(cal_removeactive3D(ca, i, j, k), calRemoveActiveCell3D(ca, i, j, k)); }

#define calGet3Db cal_hd_get3Db
#define calGet3Di cal_hd_get3Di
#define calGet3Dr cal_hd_get3Dr
#define calGetX3Db cal_hd_getx3Db
#define calGetX3Di cal_hd_getx3Di
#define calGetX3Dr cal_hd_getx3Dr
#define calSet3Db cal_hd_set3Db
#define calSet3Di cal_hd_set3Di
#define calSet3Dr cal_hd_set3Dr
#define calSetCurrent3Db cal_hd_setcur3Db
#define calSetCurrent3Di cal_hd_setcur3Di
#define calSetCurrent3Dr cal_hd_setcur3Dr
#define calInit3Db cal_hd_init3Db
#define calInit3Di cal_hd_init3Di
#define calInit3Dr cal_hd_init3Dr
#define calAddActiveCell3D cal_hd_addactive3D
#define calAddActiveCellX3D cal_hd_addactivex3D
#define calRemoveActiveCell3D cal_hd_removeactive3D
#endif /* CAL_BUILDING_LIBRARY */

#endif /* __CUDACC__ */
#endif
