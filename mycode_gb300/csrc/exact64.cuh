// Exact FP64 operations on the integer pipes.
//
// A GB300 SM sub-partition issues one FP64 warp instruction per 64 cycles, and a
// comparison, a min / max or a multiplication by 0.5 occupies the FP64 pipe like an add
// (measured with the pipe's instruction counter: one FP64-pipe instruction each; a square
// root or a divide eight).  The bit-exact FP64 residual is bound by that pipe, so the
// operations whose result is a bit pattern of the operands are done on the integer pipes
// instead, with the same result as the FP64 instruction for every non-NaN operand:
//   half(x)     RN(0.5 x): the exponent lowered by one, or (zero, subnormal, smallest
//               normal) the magnitude halved with round-half-even;
//   twice(x)    RN(2 x);
//   key(x)      a signed integer that orders doubles as < does, with -0 and +0 equal;
//   lt, gt0, lt0, ge0, le0: comparisons through it.
// With a NaN operand a comparison may answer differently from the FP64 one (a NaN state
// is an error either way).  On the host (the harnesses that compile these headers) they
// are the plain FP64 expressions.
#pragma once
#include "dual.cuh"

namespace cfdg {

CFD_HD double half_exact(double x) {
#if defined(__CUDA_ARCH__)
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
    const unsigned long long sign = u & 0x8000000000000000ull;
    const unsigned long long mag = u & 0x7fffffffffffffffull;
    // e in [2, 2046]: 0.5 x is exact, one exponent lower; e = 2047 (inf, NaN): x itself;
    // e <= 1: the magnitude field halved, a dropped half rounded to even
    const unsigned long long tiny = sign | ((mag >> 1) + (mag & (mag >> 1) & 1ull));
    const unsigned long long r = (e - 2u) < 2045u ? u - (1ull << 52) : (e == 0x7ffu ? u : tiny);
    return __longlong_as_double((long long)r);
#else
    return 0.5 * x;
#endif
}

// RN(2 x): the exponent raised by one; zero and subnormals: the magnitude field doubled
// (a carry into the exponent field is the right normal result); the largest binade
// overflows to infinity; inf and NaN unchanged
CFD_HD double twice_exact(double x) {
#if defined(__CUDA_ARCH__)
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
    const unsigned long long sign = u & 0x8000000000000000ull;
    const unsigned long long mag = u & 0x7fffffffffffffffull;
    const unsigned long long r = (e - 1u) < 2045u ? u + (1ull << 52)
                                 : (e == 0u ? (sign | (mag << 1)) : (e == 2046u ? (sign | 0x7ff0000000000000ull) : u));
    return __longlong_as_double((long long)r);
#else
    return 2.0 * x;
#endif
}

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ long long key_exact(double x) {
    const long long u = __double_as_longlong(x);
    const long long mag = u & 0x7fffffffffffffffll;
    return u < 0 ? -mag : mag;
}
#endif

CFD_HD bool lt_exact(double a, double b) {
#if defined(__CUDA_ARCH__)
    return key_exact(a) < key_exact(b);
#else
    return a < b;
#endif
}
CFD_HD bool gt0_exact(double x) {
#if defined(__CUDA_ARCH__)
    return __double_as_longlong(x) > 0;
#else
    return x > 0.0;
#endif
}
CFD_HD bool lt0_exact(double x) {
#if defined(__CUDA_ARCH__)
    const long long u = __double_as_longlong(x);
    return u < 0 && u != (long long)0x8000000000000000ull;
#else
    return x < 0.0;
#endif
}

// generic forms (float, dual numbers: on the values) and the FP64 overloads
template <class S> CFD_HD S half(S x) { return typename real_of<S>::type(0.5) * x; }
CFD_HD double half(double x) { return half_exact(x); }
template <class S> CFD_HD S twice(S x) { return typename real_of<S>::type(2) * x; }
CFD_HD double twice(double x) { return twice_exact(x); }
template <class S, class T> CFD_HD bool lt(S a, T b) { return val(a) < val(b); }
CFD_HD bool lt(double a, double b) { return lt_exact(a, b); }
template <class S> CFD_HD bool gt0(S x) { return val(x) > 0; }
CFD_HD bool gt0(double x) { return gt0_exact(x); }
template <class S> CFD_HD bool lt0(S x) { return val(x) < 0; }
CFD_HD bool lt0(double x) { return lt0_exact(x); }
template <class S> CFD_HD bool ge0(S x) { return val(x) >= 0; }
CFD_HD bool ge0(double x) { return !lt0_exact(x); }
template <class S> CFD_HD bool le0(S x) { return val(x) <= 0; }
CFD_HD bool le0(double x) { return !gt0_exact(x); }

}  // namespace cfdg
