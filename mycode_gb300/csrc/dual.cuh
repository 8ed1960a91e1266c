// Forward-mode dual numbers for the exact linearised residual (J v).
//
// Dual<R> carries a value and one directional derivative.  The residual kernels are
// templated on the scalar type, so instantiating them with Dual<R> differentiates the
// exact same operation sequence the primal uses, branch decisions included (every
// comparison is made on the value through val()).
#pragma once
#include <cmath>

#if defined(__CUDACC__)
#define CFD_HD __host__ __device__ __forceinline__
#else
#define CFD_HD inline
#endif

namespace cfdg {

template <class R>
struct Dual {
    R v, d;
    CFD_HD Dual() : v(0), d(0) {}
    CFD_HD Dual(R value) : v(value), d(0) {}
    CFD_HD Dual(R value, R deriv) : v(value), d(deriv) {}
};

template <class R> struct real_of { typedef R type; };
template <class R> struct real_of<Dual<R>> { typedef R type; };

template <class R> CFD_HD R val(R x) { return x; }
template <class R> CFD_HD R val(Dual<R> x) { return x.v; }

template <class R> CFD_HD Dual<R> operator+(Dual<R> a, Dual<R> b) { return Dual<R>(a.v + b.v, a.d + b.d); }
template <class R> CFD_HD Dual<R> operator-(Dual<R> a, Dual<R> b) { return Dual<R>(a.v - b.v, a.d - b.d); }
template <class R> CFD_HD Dual<R> operator-(Dual<R> a) { return Dual<R>(-a.v, -a.d); }
template <class R> CFD_HD Dual<R> operator*(Dual<R> a, Dual<R> b) { return Dual<R>(a.v * b.v, a.d * b.v + a.v * b.d); }
// Quotients go through one reciprocal (a divide costs about ten FP64 operations on
// GB300); the value may then differ from a plain divide in the last bit.
template <class R> CFD_HD Dual<R> operator/(Dual<R> a, Dual<R> b) {
    R ib = R(1) / b.v;
    R q = a.v * ib;
    return Dual<R>(q, (a.d - q * b.d) * ib);
}
// mixed scalar forms (the scalar is a constant: zero derivative)
template <class R> CFD_HD Dual<R> operator+(Dual<R> a, R b) { return Dual<R>(a.v + b, a.d); }
template <class R> CFD_HD Dual<R> operator+(R a, Dual<R> b) { return Dual<R>(a + b.v, b.d); }
template <class R> CFD_HD Dual<R> operator-(Dual<R> a, R b) { return Dual<R>(a.v - b, a.d); }
template <class R> CFD_HD Dual<R> operator-(R a, Dual<R> b) { return Dual<R>(a - b.v, -b.d); }
template <class R> CFD_HD Dual<R> operator*(Dual<R> a, R b) { return Dual<R>(a.v * b, a.d * b); }
template <class R> CFD_HD Dual<R> operator*(R a, Dual<R> b) { return Dual<R>(a * b.v, a * b.d); }
template <class R> CFD_HD Dual<R> operator/(Dual<R> a, R b) {
    R ib = R(1) / b;
    return Dual<R>(a.v * ib, a.d * ib);
}
template <class R> CFD_HD Dual<R> operator/(R a, Dual<R> b) {
    R ib = R(1) / b.v;
    R q = a * ib;
    return Dual<R>(q, -q * b.d * ib);
}
template <class R> CFD_HD Dual<R>& operator+=(Dual<R>& a, Dual<R> b) { a = a + b; return a; }
template <class R> CFD_HD Dual<R>& operator-=(Dual<R>& a, Dual<R> b) { a = a - b; return a; }

template <class R> CFD_HD Dual<R> sqrt(Dual<R> a) {
    R s = ::sqrt(a.v);
    return Dual<R>(s, a.d / (s + s));
}
template <class R> CFD_HD Dual<R> fabs(Dual<R> a) { return a.v < R(0) ? -a : a; }
template <class R> CFD_HD Dual<R> pow(Dual<R> a, R b) {
    R p = ::pow(a.v, b);
    return Dual<R>(p, b * p / a.v * a.d);
}
template <class R> CFD_HD Dual<R> tanh(Dual<R> a) {
    R t = ::tanh(a.v);
    return Dual<R>(t, (R(1) - t * t) * a.d);
}
template <class R> CFD_HD Dual<R> log(Dual<R> a) { return Dual<R>(::log(a.v), a.d / a.v); }
template <class R> CFD_HD Dual<R> exp(Dual<R> a) {
    R e = ::exp(a.v);
    return Dual<R>(e, e * a.d);
}

}  // namespace cfdg
