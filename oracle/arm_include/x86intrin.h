/* x86intrin.h stand-in for building the reference's host move generator on a
 * host that is not x86-64 (the GB300 machine is aarch64).
 *
 * TEST INFRASTRUCTURE ONLY (oracle/build_ref.sh puts this directory first on
 * the include path when the host is not x86-64).  The reference's Linux path
 * includes <x86intrin.h> for one thing: the population count behind its
 * popCount() (MoveGeneratorBitboard.h:3-4, 66-75).  The two intrinsics it
 * names are defined here over the compiler's portable builtin; nothing else
 * of the x86 header is used. */
#ifndef PG_ARM_X86INTRIN_SHIM_H
#define PG_ARM_X86INTRIN_SHIM_H
#include <stdint.h>

static inline long long _mm_popcnt_u64(unsigned long long x) { return __builtin_popcountll(x); }
static inline int _mm_popcnt_u32(unsigned int x) { return __builtin_popcount(x); }

#endif
