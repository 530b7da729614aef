/* Test-infrastructure shim: the reference includes <lapacke.h> but calls no
 * LAPACK routine (its LAPACK_* macros in src/H2ERI_config.h are unused). */
#ifndef ORACLE_LAPACKE_SHIM_H
#define ORACLE_LAPACKE_SHIM_H
#endif
