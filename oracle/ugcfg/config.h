/* Hand-written configuration header for compiling the UG 3.12.1 reference
 * library out of tree (it normally comes from autoconf). Used only by
 * oracle/Makefile to build the reference as a CPU oracle; nothing in the
 * ug_gb300 product includes it. */
#ifndef UGREF_CONFIG_H
#define UGREF_CONFIG_H
#define ARCH_CPU "generic"
#define ARCH_VENDOR "pc"
#define ARCH_OS "linux-gnu"
#define ARCHNAME "generic-pc-linux-gnu"
#define DYNAMIC_MEMORY_ALLOCMODEL 1
#define UG_USE_SYSTEM_HEAP 1
#define HAVE_STDLIB_H 1
#define HAVE_STRING_H 1
#define HAVE_UNISTD_H 1
#define HAVE_SYS_PARAM_H 1
#define HAVE_MALLOC_H 1
#define HAVE_TIME_H 1
#define TIME_WITH_SYS_TIME 1
#define NOF77 1
#define HAVE_LIMITS_H 1
#define HAVE_FLOAT_H 1
#define HAVE_STRINGS_H 1
#define HAVE_MEMORY_H 1
#define HAVE_ALLOCA 1
#define HAVE_ALLOCA_H 1
#define HAVE_MALLOC 1
#define HAVE_REALLOC 1
#define HAVE_STRCHR 1
#define HAVE_MEMCPY 1
#define HAVE_MEMSET 1
#define HAVE_MEMMOVE 1
#define HAVE_DIRENT_H 1
#define HAVE_SYS_TIME_H 1
#endif
