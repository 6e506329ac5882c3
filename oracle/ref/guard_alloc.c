/*
 * guard_alloc.c -- buffer allocator linked into the reference build in place
 * of the one in OpenCAL-OMP/source/cal2DBuffer.c:16-30 and cal3DBuffer.c.
 *
 * The reference's FLAT boundary computes neighbour indices unchecked
 * (OpenCAL-OMP/source/cal2D.c:866-867): row -1 and row `rows` fall outside
 * the malloc'd buffer.  This allocator surrounds every buffer with zeroed
 * guard cells (one row + one cell in 2D, one slice + one row + one cell in
 * 3D) so those reads return 0 instead of foreign heap bytes and cannot
 * fault.  In-grid behaviour is unchanged.  Test infrastructure only.
 */
#include <stdlib.h>

typedef struct guard_rec {
    void* user;
    void* base;
    struct guard_rec* next;
} guard_rec;

static guard_rec* g_list;

static void* guard_alloc(size_t elem, long cells, long guard)
{
    char* base = (char*)calloc((size_t)(cells + 2 * guard), elem);
    guard_rec* r;
    if (!base)
        return NULL;
    r = (guard_rec*)malloc(sizeof(guard_rec));
    if (!r) {
        free(base);
        return NULL;
    }
    r->base = base;
    r->user = base + (size_t)guard * elem;
    r->next = g_list;
    g_list = r;
    return r->user;
}

static void guard_free(void* user)
{
    guard_rec** p = &g_list;
    if (!user)
        return;
    while (*p) {
        if ((*p)->user == user) {
            guard_rec* r = *p;
            *p = r->next;
            free(r->base);
            free(r);
            return;
        }
        p = &(*p)->next;
    }
}

#define G2(c) ((long)(c) + 1)
#define G3(r, c) ((long)(r) * (c) + (long)(c) + 1)

char* calAllocBuffer2Db(int rows, int columns) { return (char*)guard_alloc(1, (long)rows * columns, G2(columns)); }
int* calAllocBuffer2Di(int rows, int columns) { return (int*)guard_alloc(sizeof(int), (long)rows * columns, G2(columns)); }
double* calAllocBuffer2Dr(int rows, int columns) { return (double*)guard_alloc(sizeof(double), (long)rows * columns, G2(columns)); }
void calDeleteBuffer2Db(char* M) { guard_free(M); }
void calDeleteBuffer2Di(int* M) { guard_free(M); }
void calDeleteBuffer2Dr(double* M) { guard_free(M); }

char* calAllocBuffer3Db(int rows, int columns, int slices) { return (char*)guard_alloc(1, (long)rows * columns * slices, G3(rows, columns)); }
int* calAllocBuffer3Di(int rows, int columns, int slices) { return (int*)guard_alloc(sizeof(int), (long)rows * columns * slices, G3(rows, columns)); }
double* calAllocBuffer3Dr(int rows, int columns, int slices) { return (double*)guard_alloc(sizeof(double), (long)rows * columns * slices, G3(rows, columns)); }
void calDeleteBuffer3Db(char* M) { guard_free(M); }
void calDeleteBuffer3Di(int* M) { guard_free(M); }
void calDeleteBuffer3Dr(double* M) { guard_free(M); }
