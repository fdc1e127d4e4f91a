/* Hand-written configuration for building the reference core here:
 * POSIX timing, Bessel jn available, no MPI/HDF5/libctl/MPB/Harminv. */
#ifndef ORACLE_REF_CONFIG_H
#define ORACLE_REF_CONFIG_H
#define HAVE_SYS_TIME_H 1
#define HAVE_GETTIMEOFDAY 1
#define HAVE_JN 1
#define restrict __restrict
#define F77_FUNC(name, NAME) name##_
#define F77_FUNC_(name, NAME) name##_
#define PACKAGE_VERSION "1.34.0"
#define PACKAGE_STRING "meep 1.34.0"
#endif
