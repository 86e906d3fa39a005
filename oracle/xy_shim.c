/*
 * Build shim for the reference XY library (mcsolver/xyLib.c), used only by the
 * oracle build recipe in this folder.
 *
 * The reference was written for a 15-bit C library rand() (RAND_MAX = 32767).
 * With glibc (RAND_MAX = 2^31-1) two of its lines break as shipped:
 *   - xyLib.c:324 and :384 compute (rand()*RAND_MAX+rand())%totOrbs in int,
 *     which overflows and yields negative site indices;
 *   - xyLib.c:71 declares double gaussian_distr[RAND_MAX], a 16 GiB array.
 * This translation unit restores the 15-bit contract the code assumes and then
 * includes the reference source unchanged: rand() becomes (glibc rand() & 0x7fff)
 * and RAND_MAX becomes 32767.  The reference file is compiled where it lies;
 * nothing of it is copied.
 */
#define PY_SSIZE_T_CLEAN
#include "Python.h"
#include <stdio.h>
#include <stdlib.h>
#include <math.h>

static int mcs_ref_rand15(void) { return rand() & 0x7fff; }

#undef RAND_MAX
#define RAND_MAX 32767
#define rand() mcs_ref_rand15()

#include "xyLib.c"
