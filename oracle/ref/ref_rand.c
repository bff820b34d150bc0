/*
 * ref_rand.c -- the rand() wrapper that the reference's objects call (they are
 * compiled with -Drand=sdmd_ref_rand, see Makefile), for the reference's own
 * executable: glibc's rand() unchanged.  Test infrastructure only.
 */
#include <stdlib.h>

int sdmd_ref_rand(void) { return rand(); }
