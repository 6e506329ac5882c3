/*
 * calIO.cu -- text load/save of substates (include/opencal/cal2DIO.h,
 * cal3DIO.h).  Restates the reference's matrix text format:
 *   load: whitespace-separated tokens, atoi/atof   cal2DBufferIO.c:17-45,
 *                                                  cal3DBufferIO.c (slice-major)
 *   save: "%.9f " (2D reals) / "%f " (3D reals) / "%d " per value, each
 *         followed by one more space; newline per row; 3D adds a blank line
 *         after every slice              cal2DBufferIO.c:118-150, cal3DBufferIO.c
 *   loading a substate also copies current into next   cal2DBufferIO.c:182-194
 */
#define CAL_BUILDING_LIBRARY
#include <stdio.h>
#include <stdlib.h>

#include "cal_model_internal.cuh"
#include "opencal/cal2DIO.h"
#include "opencal/cal3DIO.h"

namespace {

template <typename T>
T parse(const char* s);
template <>
CALbyte parse<CALbyte>(const char* s) { return (CALbyte)atoi(s); }
template <>
CALint parse<CALint>(const char* s) { return (CALint)atoi(s); }
template <>
CALreal parse<CALreal>(const char* s) { return atof(s); }

template <typename T>
void read_matrix(T* M, long long n, FILE* f)
{
    char tok[256];
    for (long long c = 0; c < n; c++) {
        if (fscanf(f, "%255s", tok) != 1) {
            cal::set_error(CAL_ERROR_IO, "substate file ended early");
            return;
        }
        M[c] = parse<T>(tok);
    }
}

inline void write_value(FILE* f, CALbyte v, bool) { fprintf(f, "%d  ", (int)v); }
inline void write_value(FILE* f, CALint v, bool) { fprintf(f, "%d  ", v); }
inline void write_value(FILE* f, CALreal v, bool three_d) { fprintf(f, three_d ? "%f  " : "%.9f  ", v); }

template <typename T>
void load_sub(cal::CalGrid& g, int type, int slot, T* cur, T* next, FILE* f)
{
    read_matrix(cur, g.ncells, f);
    g.host_wrote(type, slot, 0);
    g.sub[type][slot].layer[0].host_valid = true;
    if (next) {
        for (long long c = 0; c < g.ncells; c++)
            next[c] = cur[c];
        g.host_wrote(type, slot, 1);
        g.sub[type][slot].layer[1].host_valid = true;
        g.sub[type][slot].next_stale = false;
    }
}

template <typename T>
void save_sub(cal::CalGrid& g, int type, int slot, const T* cur, FILE* f)
{
    if (!g.to_host(type, slot, 0))
        return;
    const bool three_d = g.dim == 3;
    for (int k = 0; k < g.slices; k++) {
        for (int i = 0; i < g.rows; i++) {
            for (int j = 0; j < g.cols; j++)
                write_value(f, cur[g.lin(i, j, k)], three_d);
            fprintf(f, "\n");
        }
        if (three_d)
            fprintf(f, "\n");
    }
}

template <typename Model>
int slot_of(cal::CalGrid& g, int type, const void* q)
{
    return (int)(((const char*)q - (const char*)g.pool[type]) / 32);
}

} // namespace

#define CAL_IO_OPS(D, S, T, TC)                                                                           \
    extern "C" void calfLoadSubstate##D##S(struct CALModel##D* ca, struct CALSubstate##D##S* Q, FILE* f)    \
    {                                                                                                     \
        cal::CalGrid& g = ca->gpu->g;                                                                     \
        load_sub<T>(g, TC, slot_of<int>(g, TC, Q), Q->current, Q->next, f);                               \
    }                                                                                                     \
    extern "C" CALbyte calLoadSubstate##D##S(struct CALModel##D* ca, struct CALSubstate##D##S* Q, char* path) \
    {                                                                                                     \
        FILE* f = fopen(path, "r");                                                                       \
        if (!f)                                                                                           \
            return CAL_FALSE;                                                                             \
        calfLoadSubstate##D##S(ca, Q, f);                                                                 \
        fclose(f);                                                                                        \
        return CAL_TRUE;                                                                                  \
    }                                                                                                     \
    extern "C" void calfSaveSubstate##D##S(struct CALModel##D* ca, struct CALSubstate##D##S* Q, FILE* f)    \
    {                                                                                                     \
        cal::CalGrid& g = ca->gpu->g;                                                                     \
        save_sub<T>(g, TC, slot_of<int>(g, TC, Q), Q->current, f);                                        \
    }                                                                                                     \
    extern "C" CALbyte calSaveSubstate##D##S(struct CALModel##D* ca, struct CALSubstate##D##S* Q, char* path) \
    {                                                                                                     \
        FILE* f = fopen(path, "w");                                                                       \
        if (!f)                                                                                           \
            return CAL_FALSE;                                                                             \
        calfSaveSubstate##D##S(ca, Q, f);                                                                 \
        fclose(f);                                                                                        \
        return CAL_TRUE;                                                                                  \
    }

CAL_IO_OPS(2D, b, CALbyte, 0)
CAL_IO_OPS(2D, i, CALint, 1)
CAL_IO_OPS(2D, r, CALreal, 2)
CAL_IO_OPS(3D, b, CALbyte, 0)
CAL_IO_OPS(3D, i, CALint, 1)
CAL_IO_OPS(3D, r, CALreal, 2)
