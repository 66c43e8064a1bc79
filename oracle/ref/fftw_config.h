/* Stand-in for the configure output of the FFTW 3.3.7 tree vendored with
 * THUNDER (external/packages/fftw-3.3.7), for the oracle's cross-check
 * library only.  It describes the build the reference's own recipe asks for
 * (cmake/BuildFFTW.cmake: double precision, POSIX threads, no SIMD, no
 * Fortran) on a 64-bit Linux host with glibc. */
#ifndef TG3_REF_FFTW_CONFIG_H
#define TG3_REF_FFTW_CONFIG_H

#define PACKAGE "fftw"
#define PACKAGE_NAME "fftw"
#define PACKAGE_TARNAME "fftw"
#define PACKAGE_VERSION "3.3.7"
#define PACKAGE_STRING "fftw 3.3.7"
#define PACKAGE_BUGREPORT "fftw@fftw.org"
#define PACKAGE_URL ""
#define VERSION "3.3.7"
#define FFTW_CC "gcc"

#define DISABLE_FORTRAN 1
#define FFTW_ENABLE_ALLOCA 1
#define HAVE_ALLOCA 1
#define HAVE_ALLOCA_H 1
#define HAVE_ABORT 1
#define HAVE_MEMSET 1
#define HAVE_SQRT 1
#define HAVE_VPRINTF 1
#define HAVE_SNPRINTF 1
#define HAVE_ISNAN 1
#define HAVE_LIBM 1
#define STDC_HEADERS 1

#define HAVE_INTTYPES_H 1
#define HAVE_LIMITS_H 1
#define HAVE_MALLOC_H 1
#define HAVE_MEMORY_H 1
#define HAVE_STDDEF_H 1
#define HAVE_STDINT_H 1
#define HAVE_STDLIB_H 1
#define HAVE_STRINGS_H 1
#define HAVE_STRING_H 1
#define HAVE_SYS_STAT_H 1
#define HAVE_SYS_TIME_H 1
#define HAVE_SYS_TYPES_H 1
#define HAVE_UNISTD_H 1
#define TIME_WITH_SYS_TIME 1
#define HAVE_GETTIMEOFDAY 1

#define HAVE_POSIX_MEMALIGN 1
#define HAVE_MEMALIGN 1
#define HAVE_DRAND48 1
#define HAVE_COSL 1
#define HAVE_SINL 1
#define HAVE_DECL_POSIX_MEMALIGN 1
#define HAVE_DECL_MEMALIGN 1
#define HAVE_DECL_DRAND48 1
#define HAVE_DECL_SRAND48 1
#define HAVE_DECL_COSL 1
#define HAVE_DECL_SINL 1
#define HAVE_DECL_COSQ 0
#define HAVE_DECL_SINQ 0

#define HAVE_THREADS 1
#define USING_POSIX_THREADS 1

#define HAVE_UINTPTR_T 1
#define HAVE_LONG_DOUBLE 1
#define SIZEOF_DOUBLE 8
#define SIZEOF_FLOAT 4
#define SIZEOF_INT 4
#define SIZEOF_LONG 8
#define SIZEOF_LONG_LONG 8
#define SIZEOF_PTRDIFF_T 8
#define SIZEOF_SIZE_T 8
#define SIZEOF_UNSIGNED_INT 4
#define SIZEOF_UNSIGNED_LONG 8
#define SIZEOF_UNSIGNED_LONG_LONG 8
#define SIZEOF_VOID_P 8
#define SIZEOF_FFTW_R2R_KIND 4

#endif
