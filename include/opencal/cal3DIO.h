/*
 * cal3DIO.h -- text load/save of 3D substates.
 * Drop-in for OpenCAL-OMP/include/cal3DIO.h:21-71.  Format: whitespace
 * separated values in slice-major order (one matrix per slice, blank line between); saving writes "%f " (reals) or
 * "%d " (byte/int) followed by a space per value and a newline per row
 * (OpenCAL-OMP/source/cal3DBufferIO.c:150-200).  Loading fills the host
 * mirror of `current` (and `next`); the device copy is refreshed on the next
 * device operation.  Saving reads the device copy first.
 */
#ifndef cal3DIO_h
#define cal3DIO_h

#include <stdio.h>

#include "cal3D.h"

#ifdef __cplusplus
extern "C" {
#endif
void calfLoadSubstate3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, FILE* f);   /* cal3DIO.h:21 */
void calfLoadSubstate3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, FILE* f);   /* cal3DIO.h:25 */
void calfLoadSubstate3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, FILE* f);   /* cal3DIO.h:29 */
CALbyte calLoadSubstate3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, char* path); /* cal3DIO.h:35 */
CALbyte calLoadSubstate3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, char* path); /* cal3DIO.h:39 */
CALbyte calLoadSubstate3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, char* path); /* cal3DIO.h:43 */
void calfSaveSubstate3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, FILE* f);   /* cal3DIO.h:49 */
void calfSaveSubstate3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, FILE* f);   /* cal3DIO.h:53 */
void calfSaveSubstate3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, FILE* f);   /* cal3DIO.h:57 */
CALbyte calSaveSubstate3Db(struct CALModel3D* ca3D, struct CALSubstate3Db* Q, char* path); /* cal3DIO.h:63 */
CALbyte calSaveSubstate3Di(struct CALModel3D* ca3D, struct CALSubstate3Di* Q, char* path); /* cal3DIO.h:67 */
CALbyte calSaveSubstate3Dr(struct CALModel3D* ca3D, struct CALSubstate3Dr* Q, char* path); /* cal3DIO.h:71 */
#ifdef __cplusplus
}
#endif
#endif
