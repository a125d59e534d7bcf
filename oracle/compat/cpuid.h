/* cpuid.h - TEST INFRASTRUCTURE ONLY: an empty stand-in for the x86 compiler header on hosts that
 * lack it (aarch64).  The reference's src/algorithms/avx2.cpp includes <cpuid.h> for every GNU
 * compiler but uses it only inside its __AVX2__ sections, which are not compiled there; the
 * oracle's reference build adds this directory to the include path on non-x86 hosts only. */
#ifndef IMOP_ORACLE_COMPAT_CPUID_H
#define IMOP_ORACLE_COMPAT_CPUID_H
#endif
