/* Host configuration the reference's cmake configure step would write (cmpConfiguration.h and
 * cmpTypes.h): a 64-bit Linux host with the POSIX headers and gettimeofday.  Included by the
 * stand-ins for MBIRLib/MBIRLib.h and MXA/MXA.h.  Test infrastructure only. */
#ifndef REF_SHIM_CONFIG_H
#define REF_SHIM_CONFIG_H
#define CMP_HAVE_STDDEF_H 1
#define CMP_HAVE_STDINT_H 1
#define CMP_HAVE_STDLIB_H 1
#define CMP_HAVE_SETJMP_H 1
#define CMP_HAVE_STRING_H 1
#define CMP_HAVE_STDIO_H 1
#define CMP_HAVE_MATH_H 1
#define CMP_HAVE_TIME_H 1
#define CMP_HAVE_SYS_TIME_H 1
#define CMP_HAVE_SYS_TIME_GETTIMEOFDAY 1
#define CMP_HAVE_SYS_TYPES_H 1
#define CMP_HAVE_SYS_STAT_H 1
#define CMP_HAVE_UNISTD_H 1
#define CMP_HAVE_FCNTL_H 1
#define CMP_HAVE_ERRNO_H 1
#define CMP_SIZEOF_CHAR 1
#define CMP_SIZEOF_SHORT 2
#define CMP_SIZEOF_INT 4
#define CMP_SIZEOF_LONG 8
#define CMP_SIZEOF_LONG_LONG 8
#define CMP_SIZEOF_FLOAT 4
#define CMP_SIZEOF_DOUBLE 8
#define CMP_SIZEOF_SIZE_T 8
#define CMP_WORDS_LITTLEENDIAN 1
#define CMP_HAVE_FSEEKO 1
#ifdef __cplusplus
#ifndef __STDC_LIMIT_MACROS
#define __STDC_LIMIT_MACROS 1
#endif
#endif
#include <stdint.h>
#include <stddef.h>
typedef float float32;
typedef double float64;
#endif
