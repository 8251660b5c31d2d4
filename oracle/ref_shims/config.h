/* Build configuration for compiling the reference sources as a one-rank CPU
 * oracle.  ATRIP_USE_DGEMM is the reference's configure default
 * (configure.ac:96-102); the Makefile beside this file builds a second
 * variant with it undefined (the BLAS-free naive loops,
 * src/atrip/Equations.cxx:685-726). */
#ifndef ORACLE_REF_CONFIG_H
#define ORACLE_REF_CONFIG_H
#ifndef ORACLE_NAIVE_LOOPS
#define ATRIP_USE_DGEMM 1
#endif
#ifndef ATRIP_DEBUG
#define ATRIP_DEBUG 1
#endif
#define ATRIP_NO_OUTPUT 1
#endif
