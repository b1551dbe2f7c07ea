/* Forced-include shim for compiling the reference Tay CPU path with gcc on Linux.
 *
 * Test infrastructure only: this lets the oracle recipe (oracle/ref/Makefile) build the
 * reference's own C sources where they lie, unmodified, so that the reference CPU path
 * (CpuSimple / CpuGrid / CpuZGrid) can be run in-process as the parity oracle.
 *
 * The reference targets MSVC (tay/tay.vcxproj) and uses the bounds-checked *_s CRT
 * functions (tay/state.c:146 strcpy_s, tay/ocl.c:280 strcpy_s, tay/ocl.c:286 sprintf_s,
 * test/test.c:312 sprintf_s, test/test_basic.c:174 fopen_s).  They are mapped onto their
 * portable equivalents here.  space.h declares `struct TayThreadContext` at prototype
 * scope (tay/space.h:11), so the recipe also force-includes tay/thread.h first. */
#ifndef TAY_REF_SHIM_H
#define TAY_REF_SHIM_H

#include <stddef.h>
#include <stdio.h>
#include <string.h>

#define strcpy_s(dst, cap, src) snprintf((dst), (cap), "%s", (src))
#define sprintf_s(dst, cap, ...) snprintf((dst), (cap), __VA_ARGS__)
#define fopen_s(pfile, name, mode) ((*(pfile) = fopen((name), (mode))) ? 0 : 1)

#endif
