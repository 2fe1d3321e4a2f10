/* Configured-header stand-in for the oracle build of the reference
 * (the reference generates this file from include/dendro.h.in with CMake). */
#ifndef __DENDRO_H__
#define __DENDRO_H__
#define DENDRO_VERSION_MAJOR 4
#define DENDRO_VERSION_MINOR 0
#ifndef NULL
#define NULL 0
#endif
#ifdef USE_64BIT_INDICES
#define DendroIntL long long
#else
#define DendroIntL long
#endif
#endif
