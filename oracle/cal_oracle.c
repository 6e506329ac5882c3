/*
 * cal_oracle.c -- CPU restatement of OpenCAL's serial global transition.
 * TEST INFRASTRUCTURE ONLY (the checker); see cal_oracle.h for the list of
 * reference functions restated here and the one documented FLAT difference.
 */
#include "cal_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static size_t elem_size(int type)
{
    return type == ORC_B ? 1 : (type == ORC_I ? sizeof(int) : sizeof(double));
}

static long ncell(const orc_ca* m)
{
    return (long)m->rows * m->cols * (m->dim == 3 ? m->slices : 1);
}

long orc_index(const orc_ca* m, int i, int j, int k)
{
    if (m->dim == 2)
        return (long)i * m->cols + j;
    return (long)k * m->rows * m->cols + (long)i * m->cols + j;
}

static double load_elem(const void* buf, int type, long c)
{
    switch (type) {
    case ORC_B: return (double)((const signed char*)buf)[c];
    case ORC_I: return (double)((const int*)buf)[c];
    default: return ((const double*)buf)[c];
    }
}

static void store_elem(void* buf, int type, long c, double v)
{
    switch (type) {
    case ORC_B: ((signed char*)buf)[c] = (signed char)v; break;
    case ORC_I: ((int*)buf)[c] = (int)v; break;
    default: ((double*)buf)[c] = v; break;
    }
}

/* ---- neighbourhoods (cal2D.c:28-166, cal3D.c:29-105) ------------------- */

void orc_add_neighbor(orc_ca* m, int di, int dj, int dk)
{
    if (m->nx >= ORC_MAX_X)
        return;
    m->xo[m->nx][0] = di;
    m->xo[m->nx][1] = dj;
    m->xo[m->nx][2] = dk;
    m->nx++;
}

static void build_2d_neighborhood(orc_ca* m)
{
    /* each table lists (di, dj) in the reference's index order */
    static const int vn[5][2] = {{0, 0}, {-1, 0}, {0, -1}, {0, 1}, {1, 0}};
    static const int moore[9][2] = {{0, 0}, {-1, 0}, {0, -1}, {0, 1}, {1, 0},
                                    {-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    /* hexagonal: entries 0-6 for even columns, 7-13 for odd columns */
    static const int hex[14][2] = {{0, 0}, {-1, 1}, {-1, 0}, {-1, -1}, {0, -1}, {1, 0}, {0, 1},
                                   {0, 0}, {0, 1}, {-1, 0}, {0, -1}, {1, -1}, {1, 0}, {1, 1}};
    /* alternative hexagonal: entries 0-6 for even rows, 7-13 for odd rows */
    static const int hexalt[14][2] = {{0, 0}, {-1, 0}, {-1, -1}, {0, -1}, {1, -1}, {1, 0}, {0, 1},
                                      {0, 0}, {-1, 1}, {-1, 0}, {0, -1}, {1, 0}, {1, 1}, {0, 1}};
    const int(*t)[2] = NULL;
    int n, cnt = 0;
    switch (m->nbhd) {
    case ORC_NB_VN: t = vn; cnt = 5; break;
    case ORC_NB_MOORE: t = moore; cnt = 9; break;
    case ORC_NB_HEX: t = hex; cnt = 14; break;
    case ORC_NB_HEX_ALT: t = hexalt; cnt = 14; break;
    default: return;
    }
    for (n = 0; n < cnt; n++)
        orc_add_neighbor(m, t[n][0], t[n][1], 0);
    if (m->nbhd == ORC_NB_HEX || m->nbhd == ORC_NB_HEX_ALT)
        m->nx = 7; /* the reference keeps 14 entries but reports 7 */
}

static void build_3d_neighborhood(orc_ca* m)
{
    static const int plane[9][2] = {{0, 0}, {-1, 0}, {0, -1}, {0, 1}, {1, 0},
                                    {-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    int n, s;
    if (m->nbhd == ORC_NB_VN) {
        for (n = 0; n < 5; n++)
            orc_add_neighbor(m, plane[n][0], plane[n][1], 0);
        orc_add_neighbor(m, 0, 0, -1);
        orc_add_neighbor(m, 0, 0, 1);
    } else if (m->nbhd == ORC_NB_MOORE) {
        static const int dks[3] = {0, -1, 1};
        for (s = 0; s < 3; s++)
            for (n = 0; n < 9; n++)
                orc_add_neighbor(m, plane[n][0], plane[n][1], dks[s]);
    }
}

/* ---- definition ------------------------------------------------------- */

static orc_ca* def_common(int dim, int rows, int cols, int slices, int nbhd, int toroidal, int ac)
{
    orc_ca* m = (orc_ca*)calloc(1, sizeof(orc_ca));
    if (!m)
        return NULL;
    m->dim = dim;
    m->rows = rows;
    m->cols = cols;
    m->slices = dim == 3 ? slices : 1;
    m->nbhd = nbhd;
    m->toroidal = toroidal;
    m->ac = ac;
    if (ac)
        m->flags = (unsigned char*)calloc((size_t)ncell(m), 1);
    return m;
}

orc_ca* orc_def2d(int rows, int cols, int nbhd, int toroidal, int ac)
{
    orc_ca* m = def_common(2, rows, cols, 1, nbhd, toroidal, ac);
    if (m)
        build_2d_neighborhood(m);
    return m;
}

orc_ca* orc_def3d(int rows, int cols, int slices, int nbhd, int toroidal, int ac)
{
    orc_ca* m = def_common(3, rows, cols, slices, nbhd, toroidal, ac);
    if (m)
        build_3d_neighborhood(m);
    return m;
}

static orc_sub* new_sub(orc_ca* m, int type, int layers)
{
    orc_sub* q = (orc_sub*)calloc(1, sizeof(orc_sub));
    size_t bytes = (size_t)ncell(m) * elem_size(type);
    if (!q)
        return NULL;
    q->type = type;
    q->cur = calloc(1, bytes);
    q->nxt = layers == 2 ? calloc(1, bytes) : NULL;
    return q;
}

orc_sub* orc_add_sub(orc_ca* m, int type)
{
    orc_sub* q;
    if (m->nsub >= ORC_MAX_SUBSTATES)
        return NULL;
    q = new_sub(m, type, 2);
    if (q)
        m->sub[m->nsub++] = q;
    return q;
}

orc_sub* orc_add_single(orc_ca* m, int type)
{
    orc_sub* q;
    if (m->nsingle >= ORC_MAX_SUBSTATES)
        return NULL;
    q = new_sub(m, type, 1);
    if (q)
        m->single[m->nsingle++] = q;
    return q;
}

void orc_add_ep2(orc_ca* m, orc_ep2 ep)
{
    if (m->nep < ORC_MAX_EP)
        m->ep2[m->nep++] = ep;
}

void orc_add_ep3(orc_ca* m, orc_ep3 ep)
{
    if (m->nep < ORC_MAX_EP)
        m->ep3[m->nep++] = ep;
}

void orc_free(orc_ca* m)
{
    int s;
    if (!m)
        return;
    for (s = 0; s < m->nsub; s++) {
        free(m->sub[s]->cur);
        free(m->sub[s]->nxt);
        free(m->sub[s]);
    }
    for (s = 0; s < m->nsingle; s++) {
        free(m->single[s]->cur);
        free(m->single[s]);
    }
    free(m->flags);
    free(m->cells);
    free(m);
}

/* ---- neighbour resolution (cal2D.c:859-870, calCommon.h:56) ----------- */

static int wrap(int x, int n)
{
    /* calGetToroidalX only corrects one period, as the reference does */
    return x < 0 ? n + x : (x > n - 1 ? x - n : x);
}

int orc_neighbor(const orc_ca* m, int i, int j, int k, int n, int* oi, int* oj, int* ok)
{
    int ni, nj, nk;
    if (m->dim == 2) {
        if ((m->nbhd == ORC_NB_HEX && (j % 2) == 1) || (m->nbhd == ORC_NB_HEX_ALT && (i % 2) == 1))
            n += ORC_HEX_SHIFT;
        nk = 0;
    } else {
        nk = k + m->xo[n][2];
    }
    ni = i + m->xo[n][0];
    nj = j + m->xo[n][1];
    if (m->toroidal) {
        ni = wrap(ni, m->rows);
        nj = wrap(nj, m->cols);
        if (m->dim == 3)
            nk = wrap(nk, m->slices);
    } else {
        if (ni < 0 || ni >= m->rows || nj < 0 || nj >= m->cols)
            return 0;
        if (m->dim == 3 && (nk < 0 || nk >= m->slices))
            return 0;
    }
    *oi = ni;
    *oj = nj;
    *ok = nk;
    return 1;
}

/* ---- cell accessors ---------------------------------------------------- */

double orc_get(const orc_ca* m, const orc_sub* q, int i, int j, int k)
{
    return load_elem(q->cur, q->type, orc_index(m, i, j, k));
}

double orc_getx(const orc_ca* m, const orc_sub* q, int i, int j, int k, int n)
{
    int a, b, c;
    if (!orc_neighbor(m, i, j, k, n, &a, &b, &c))
        return 0.0;
    return load_elem(q->cur, q->type, orc_index(m, a, b, c));
}

void orc_set(orc_ca* m, orc_sub* q, int i, int j, int k, double v)
{
    store_elem(q->nxt, q->type, orc_index(m, i, j, k), v);
}

void orc_set_cur(orc_ca* m, orc_sub* q, int i, int j, int k, double v)
{
    store_elem(q->cur, q->type, orc_index(m, i, j, k), v);
}

void orc_init_cell(orc_ca* m, orc_sub* q, int i, int j, int k, double v)
{
    long c = orc_index(m, i, j, k);
    store_elem(q->cur, q->type, c, v);
    if (q->nxt)
        store_elem(q->nxt, q->type, c, v);
}

/* ---- whole-substate operations (cal2D.c:625-713, cal2DBuffer.c) -------- */

static long list_index(const orc_ca* m, long n)
{
    const int* c = m->cells + n * m->dim;
    return orc_index(m, c[0], c[1], m->dim == 3 ? c[2] : 0);
}

static void fill(orc_ca* m, void* buf, int type, double v)
{
    long n, total = ncell(m);
    if (m->cells) {
#pragma omp parallel for
        for (n = 0; n < m->ncells; n++)
            store_elem(buf, type, list_index(m, n), v);
    } else {
#pragma omp parallel for
        for (n = 0; n < total; n++)
            store_elem(buf, type, n, v);
    }
}

void orc_init_sub(orc_ca* m, orc_sub* q, double v)
{
    fill(m, q->cur, q->type, v);
    if (q->nxt)
        fill(m, q->nxt, q->type, v);
}

void orc_init_sub_next(orc_ca* m, orc_sub* q, double v)
{
    fill(m, q->nxt, q->type, v);
}

void orc_update_sub(orc_ca* m, orc_sub* q)
{
    size_t es = elem_size(q->type);
    long n;
    if (!q->nxt)
        return;
    if (m->cells) {
#pragma omp parallel for
        for (n = 0; n < m->ncells; n++) {
            long c = list_index(m, n);
            memcpy((char*)q->cur + c * es, (char*)q->nxt + c * es, es);
        }
    } else {
        memcpy(q->cur, q->nxt, (size_t)ncell(m) * es);
    }
}

void orc_load(orc_ca* m, orc_sub* q, const void* data)
{
    size_t bytes = (size_t)ncell(m) * elem_size(q->type);
    memcpy(q->cur, data, bytes);
    if (q->nxt)
        memcpy(q->nxt, q->cur, bytes);
}

void orc_store(const orc_ca* m, const orc_sub* q, void* data)
{
    memcpy(data, q->cur, (size_t)ncell(m) * elem_size(q->type));
}

/* ---- active cells (cal2D.c:333-440, cal3D.c:270-340) ------------------- */

void orc_add_active(orc_ca* m, int i, int j, int k)
{
    long c;
    if (i < 0 || i >= m->rows || j < 0 || j >= m->cols || (m->dim == 3 && (k < 0 || k >= m->slices)))
        return;
    c = orc_index(m, i, j, k);
    /* atomic so that the OpenMP build keeps the count exact */
    if (__atomic_exchange_n(&m->flags[c], 1, __ATOMIC_RELAXED) == 0)
        __atomic_add_fetch(&m->pending, 1, __ATOMIC_RELAXED);
}

void orc_add_active_x(orc_ca* m, int i, int j, int k, int n)
{
    int a, b, c;
    if (orc_neighbor(m, i, j, k, n, &a, &b, &c))
        orc_add_active(m, a, b, c);
}

void orc_remove_active(orc_ca* m, int i, int j, int k)
{
    long c = orc_index(m, i, j, k);
    if (__atomic_exchange_n(&m->flags[c], 0, __ATOMIC_RELAXED) != 0)
        __atomic_sub_fetch(&m->pending, 1, __ATOMIC_RELAXED);
}

void orc_update_active(orc_ca* m)
{
    long n = 0;
    int i, j, k;
    free(m->cells);
    m->cells = NULL;
    m->ncells = 0;
    m->size += m->pending;
    m->pending = 0;
    if (m->size == 0)
        return; /* the reference leaves A.cells NULL: EPs then visit every cell */
    m->cells = (int*)malloc(sizeof(int) * (size_t)m->dim * (size_t)m->size);
    /* 2D: row-major; 3D: i, then j, then k (cal3D.c loop order) */
    for (i = 0; i < m->rows; i++)
        for (j = 0; j < m->cols; j++)
            for (k = 0; k < m->slices; k++)
                if (m->flags[orc_index(m, i, j, k)]) {
                    if (n < m->size) {
                        int* c = m->cells + n * m->dim;
                        c[0] = i;
                        c[1] = j;
                        if (m->dim == 3)
                            c[2] = k;
                    }
                    n++;
                }
    if (n != m->size)
        m->error = 1;
    m->ncells = n < m->size ? n : m->size;
}

/* ---- transition (cal2D.c:717-776) -------------------------------------- */

void orc_apply(orc_ca* m, int b)
{
    long n;
    int i, j, k;
    /* the OpenMP build parallelises exactly where the reference does
     * (cal2D.c:724,729): EPs write only their own cell, so the result does
     * not depend on the thread count */
    if (m->cells) {
#pragma omp parallel for
        for (n = 0; n < m->ncells; n++) {
            const int* c = m->cells + n * m->dim;
            if (m->dim == 2)
                m->ep2[b](m, c[0], c[1]);
            else
                m->ep3[b](m, c[0], c[1], c[2]);
        }
        return;
    }
    if (m->dim == 2) {
#pragma omp parallel for private(j)
        for (i = 0; i < m->rows; i++)
            for (j = 0; j < m->cols; j++)
                m->ep2[b](m, i, j);
    } else {
        /* cal3D.c applies in i, j, k order */
#pragma omp parallel for private(j, k)
        for (i = 0; i < m->rows; i++)
            for (j = 0; j < m->cols; j++)
                for (k = 0; k < m->slices; k++)
                    m->ep3[b](m, i, j, k);
    }
}

void orc_update(orc_ca* m)
{
    int s;
    if (m->ac)
        orc_update_active(m);
    for (s = 0; s < m->nsub; s++)
        orc_update_sub(m, m->sub[s]);
}

void orc_transition(orc_ca* m)
{
    int b;
    for (b = 0; b < m->nep; b++) {
        orc_apply(m, b);
        orc_update(m);
    }
}

/* ---- run loop (cal2DRun.c:77-139) -------------------------------------- */

void orc_run_init(orc_run* r)
{
    if (r->init) {
        r->init(r->m);
        if (r->implicit)
            orc_update(r->m);
    }
}

int orc_run_step(orc_run* r)
{
    if (r->transition) {
        r->transition(r->m);
        if (r->implicit)
            orc_update(r->m);
    } else {
        orc_transition(r->m);
    }
    if (r->steering) {
        r->steering(r->m);
        if (r->implicit)
            orc_update(r->m);
    }
    if (r->stop && r->stop(r->m))
        return 0;
    return 1;
}

void orc_run_finalize(orc_run* r)
{
    if (r->finalize) {
        r->finalize(r->m);
        if (r->implicit)
            orc_update(r->m);
    }
}

void orc_run_all(orc_run* r)
{
    orc_run_init(r);
    for (r->step = r->initial; r->step <= r->final_ || r->final_ == 0; r->step++)
        if (!orc_run_step(r))
            break;
    orc_run_finalize(r);
}

/* unsafe operations, OpenCAL-OMP/source/cal2DUnsafe.c:17-275 and
 * cal3DUnsafe.c:18-245 (serial: the per-cell locks are no-ops) */
double orc_get_next(const orc_ca* m, const orc_sub* q, int i, int j, int k)
{
    return load_elem(q->nxt, q->type, orc_index(m, i, j, k));
}

double orc_getx_next(const orc_ca* m, const orc_sub* q, int i, int j, int k, int n)
{
    int a, b, c;
    if (!orc_neighbor(m, i, j, k, n, &a, &b, &c))
        return 0.0;
    return load_elem(q->nxt, q->type, orc_index(m, a, b, c));
}

void orc_setx(orc_ca* m, orc_sub* q, int i, int j, int k, int n, double v)
{
    int a, b, c;
    if (orc_neighbor(m, i, j, k, n, &a, &b, &c))
        orc_set(m, q, a, b, c, v);
}

void orc_setx_cur(orc_ca* m, orc_sub* q, int i, int j, int k, int n, double v)
{
    int a, b, c;
    if (orc_neighbor(m, i, j, k, n, &a, &b, &c))
        orc_set_cur(m, q, a, b, c, v);
}

void orc_initx(orc_ca* m, orc_sub* q, int i, int j, int k, int n, double v)
{
    int a, b, c;
    if (orc_neighbor(m, i, j, k, n, &a, &b, &c))
        orc_init_cell(m, q, a, b, c, v);
}

void orc_add_next(orc_ca* m, orc_sub* q, int i, int j, int k, double v)
{
    const long c = orc_index(m, i, j, k);
    store_elem(q->nxt, q->type, c, load_elem(q->nxt, q->type, c) + v);
}

void orc_add_nextx(orc_ca* m, orc_sub* q, int i, int j, int k, int n, double v)
{
    int a, b, c;
    if (orc_neighbor(m, i, j, k, n, &a, &b, &c))
        orc_add_next(m, q, a, b, c, v);
}

/* ======================= reductions ===================================== */
/* calReductionOperation2Db/i/r (OpenCAL-OMP/source/cal2DReduction.c:18-500,
 * serial path): start from element 0 of the current layer and fold every
 * other element in index order, in the substate's own type (CALbyte and
 * CALint wrap; the binary operations on reals go through CALint,
 * cal2DReduction.c:437-455).  One deliberate difference: the reference sets
 * the last thread's end index to `model->rows` instead of rows * columns
 * (cal2DReduction.c:45-47), so its serial build folds only elements
 * 0 .. rows-1; here every cell is folded.  Both agree on grids with one
 * column.  kind: 0 byte, 1 int, 2 real; the result is returned as a double. */
#define ORC_FOLD(T, ACC, X, OP)                                                          \
    switch (OP) {                                                                        \
    case 1: if (ACC < X) ACC = X; break;                                                 \
    case 2: if (ACC > X) ACC = X; break;                                                 \
    case 3: ACC += X; break;                                                             \
    case 4: ACC *= X; break;                                                             \
    case 5: ACC = (T)(ACC && X); break;                                                  \
    case 6: ACC = (T)((CALINT_T)ACC & (CALINT_T)X); break;                               \
    case 7: ACC = (T)(ACC || X); break;                                                  \
    case 8: ACC = (T)((CALINT_T)ACC | (CALINT_T)X); break;                               \
    case 9: ACC = (T)(!!ACC != !!X); break;                                              \
    case 10: ACC = (T)((CALINT_T)ACC ^ (CALINT_T)X); break;                              \
    default: break;                                                                      \
    }
#define CALINT_T int

int orc_reduce2d(int kind, int rows, int cols, const void* data, int op, double* out)
{
    long n = (long)rows * cols, i;
    if (n <= 0 || op < 1 || op > 10)
        return 1;
    if (kind == 0) {
        const char* v = (const char*)data;
        char acc = v[0];
        for (i = 1; i < n; i++) {
            char x = v[i];
            ORC_FOLD(char, acc, x, op)
        }
        *out = (double)acc;
    } else if (kind == 1) {
        const int* v = (const int*)data;
        int acc = v[0];
        for (i = 1; i < n; i++) {
            int x = v[i];
            ORC_FOLD(int, acc, x, op)
        }
        *out = (double)acc;
    } else {
        const double* v = (const double*)data;
        double acc = v[0];
        for (i = 1; i < n; i++) {
            double x = v[i];
            ORC_FOLD(double, acc, x, op)
        }
        *out = acc;
    }
    return 0;
}

/* ======================= substate text files ============================ */
/* calfSaveMatrix2D* / calfSaveMatrix3D* (OpenCAL-OMP/source/
 * cal2DBufferIO.c:105-147, cal3DBufferIO.c:110-160): each value printed with
 * "%d " (byte, int) or "%.9f " (2D real) / "%f " (3D real) into a string
 * that is then written followed by one more space; a newline after every
 * row; in 3D slice by slice, with an empty line after every slice.
 * calfLoadMatrix* (cal2DBufferIO.c:17-45): whitespace-separated tokens,
 * atoi / atof, in the same order.  kind: 0 byte, 1 int, 2 real. */
int orc_save_text(int dim, int kind, int rows, int cols, int slices, const void* data, const char* path)
{
    char str[256];
    int i, j, k;
    FILE* f = fopen(path, "w");
    if (!f)
        return 1;
    if (dim == 2)
        slices = 1;
    for (k = 0; k < slices; k++) {
        for (i = 0; i < rows; i++) {
            for (j = 0; j < cols; j++) {
                long c = ((long)k * rows + i) * cols + j;
                if (kind == 0)
                    sprintf(str, "%d ", ((const char*)data)[c]);
                else if (kind == 1)
                    sprintf(str, "%d ", ((const int*)data)[c]);
                else
                    sprintf(str, dim == 2 ? "%.9f " : "%f ", ((const double*)data)[c]);
                fprintf(f, "%s ", str);
            }
            fprintf(f, "\n");
        }
        if (dim == 3)
            fprintf(f, "\n");
    }
    fclose(f);
    return 0;
}

int orc_load_text(int dim, int kind, int rows, int cols, int slices, void* data, const char* path)
{
    char str[256];
    long c, n = (long)rows * cols * (dim == 3 ? slices : 1);
    FILE* f = fopen(path, "r");
    if (!f)
        return 1;
    for (c = 0; c < n; c++) {
        if (fscanf(f, "%255s", str) != 1) {
            fclose(f);
            return 2;
        }
        if (kind == 0)
            ((char*)data)[c] = (char)atoi(str);
        else if (kind == 1)
            ((int*)data)[c] = atoi(str);
        else
            ((double*)data)[c] = atof(str);
    }
    fclose(f);
    return 0;
}
