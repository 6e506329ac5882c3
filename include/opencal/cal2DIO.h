/*
 * cal2DIO.h -- text load/save of 2D substates.
 * Drop-in for OpenCAL-OMP/include/cal2DIO.h:21-71.  Format: whitespace
 * separated values in row-major order; saving writes "%.9f " (reals) or
 * "%d " (byte/int) followed by a space per value and a newline per row
 * (OpenCAL-OMP/source/cal2DBufferIO.c:118-150).  Loading fills the host
 * mirror of `current` (and `next`); the device copy is refreshed on the next
 * device operation.  Saving reads the device copy first.
 */
#ifndef cal2DIO_h
#define cal2DIO_h

#include <stdio.h>

#include "cal2D.h"

#ifdef __cplusplus
extern "C" {
#endif
void calfLoadSubstate2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, FILE* f);   /* cal2DIO.h:21 */
void calfLoadSubstate2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, FILE* f);   /* cal2DIO.h:25 */
void calfLoadSubstate2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, FILE* f);   /* cal2DIO.h:29 */
CALbyte calLoadSubstate2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, char* path); /* cal2DIO.h:35 */
CALbyte calLoadSubstate2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, char* path); /* cal2DIO.h:39 */
CALbyte calLoadSubstate2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, char* path); /* cal2DIO.h:43 */
void calfSaveSubstate2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, FILE* f);   /* cal2DIO.h:49 */
void calfSaveSubstate2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, FILE* f);   /* cal2DIO.h:53 */
void calfSaveSubstate2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, FILE* f);   /* cal2DIO.h:57 */
CALbyte calSaveSubstate2Db(struct CALModel2D* ca2D, struct CALSubstate2Db* Q, char* path); /* cal2DIO.h:63 */
CALbyte calSaveSubstate2Di(struct CALModel2D* ca2D, struct CALSubstate2Di* Q, char* path); /* cal2DIO.h:67 */
CALbyte calSaveSubstate2Dr(struct CALModel2D* ca2D, struct CALSubstate2Dr* Q, char* path); /* cal2DIO.h:71 */
#ifdef __cplusplus
}
#endif
#endif
