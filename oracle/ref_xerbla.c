/*
 * xerbla_ for the reference build in oracle/_ref (test infrastructure only).
 * The reference's Fortran-ABI shims report argument errors through xerbla_
 * (flens/lapack/interface/include/config.h:45 passes name, info, length;
 * flens/blas/interface/blas/config.h:33 passes name, info).  Netlib's xerbla
 * stops the program; this one records the call so tests can read it back.
 */
#include <string.h>

static char ref_last_name[8];
static int ref_last_info;
static int ref_calls;

void xerbla_(const char *name, const int *info)
{
    memset(ref_last_name, 0, sizeof ref_last_name);
    for (int i = 0; i < 6 && name[i]; ++i) ref_last_name[i] = name[i];
    ref_last_info = *info;
    ++ref_calls;
}

int ref_xerbla_calls(void) { return ref_calls; }
int ref_xerbla_info(void) { return ref_last_info; }
const char *ref_xerbla_name(void) { return ref_last_name; }
