// va_dual.cuh — forward-mode dual numbers for the Verilog-A device code emitted
// by cedarsim.jl_gb300/va/emit.py (host and device).
//
// Dual<T, N> carries a value and N partials of type T.  With T = double it is the
// first-order type the emitted models evaluate in (partials with respect to the
// N terminal potentials, as CedarSim seeds ForwardDiff duals on the probed node
// voltages, src/vasim.jl:347-412).  A model that calls ddx() is evaluated in
// Dual<Dual<double, N>, N>: ddx(x, V(a)) reads the outer partial, and the inner
// partials carry its derivative into the Jacobian.
//
// Math functions follow the Verilog-A built-ins (NaN outside the domain, as the
// reference's NaNMath-based environment, src/va_env.jl:35-67); each derivative
// is the textbook one.  limexp continues exp linearly above an exponent of 80.
#pragma once
#ifdef __CUDACC__
#define VA_HD __host__ __device__ __forceinline__
// the model dispatch is called, not inlined: one copy per translation unit
// instead of one per evaluation site keeps the engine kernels' build time and
// register allocation what they are without Verilog-A models
#ifdef CEDAR_VA_SEPARATE
// large models: the dispatch is compiled once, in its own translation unit
// (va_models.cu), and device-linked into the engine kernels
#define VA_CALL __host__ __device__ __noinline__
#define VA_EXTERN __host__ __device__
#else
#define VA_CALL static __host__ __device__ __noinline__
#endif
// the functions a large module is split into are called, not inlined
#define VA_PART __host__ __device__ __noinline__
#else
#define VA_HD inline
#define VA_CALL inline
#define VA_PART inline
#endif
#include <cmath>

namespace cedar {
namespace va {

using ::acos;
using ::asin;
using ::atan;
using ::atan2;
using ::ceil;
using ::cos;
using ::cosh;
using ::exp;
using ::fabs;
using ::floor;
using ::hypot;
using ::log;
using ::log10;
using ::pow;
using ::round;
using ::sin;
using ::sinh;
using ::sqrt;
using ::tan;
using ::tanh;
using ::trunc;

template <class T, int N>
struct Dual {
  T v;
  T d[N];
  VA_HD Dual() : v(0.0) {
    for (int i = 0; i < N; ++i) d[i] = T(0.0);
  }
  VA_HD Dual(double c) : v(c) {  // NOLINT: constants convert implicitly
    for (int i = 0; i < N; ++i) d[i] = T(0.0);
  }
};

// value of a (possibly nested) dual as a double
VA_HD double val(double x) { return x; }
template <class T, int N>
VA_HD double val(const Dual<T, N> &x) { return val(x.v); }

VA_HD bool all_zero(double x) { return x == 0.0; }
template <class T, int N>
VA_HD bool all_zero(const Dual<T, N> &x) {
  if (!all_zero(x.v)) return false;
  for (int i = 0; i < N; ++i)
    if (!all_zero(x.d[i])) return false;
  return true;
}

// f'(x) * dx with a strong zero: a direction x does not move along contributes
// 0 even where f' is infinite (sqrt, pow at 0), instead of 0 * inf = NaN
template <class T>
VA_HD T sz_mul(const T &fp, const T &dx) { return all_zero(dx) ? T(0.0) : fp * dx; }

// r = f(x) with f(x.v) = fv and f'(x.v) = fp
template <class T, int N>
VA_HD Dual<T, N> chain(const Dual<T, N> &x, const T &fv, const T &fp) {
  Dual<T, N> r;
  r.v = fv;
  for (int i = 0; i < N; ++i) r.d[i] = sz_mul(fp, x.d[i]);
  return r;
}

// arithmetic
template <class T, int N>
VA_HD Dual<T, N> operator+(const Dual<T, N> &a, const Dual<T, N> &b) {
  Dual<T, N> r;
  r.v = a.v + b.v;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <class T, int N>
VA_HD Dual<T, N> operator-(const Dual<T, N> &a, const Dual<T, N> &b) {
  Dual<T, N> r;
  r.v = a.v - b.v;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <class T, int N>
VA_HD Dual<T, N> operator-(const Dual<T, N> &a) {
  Dual<T, N> r;
  r.v = -a.v;
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <class T, int N>
VA_HD Dual<T, N> operator*(const Dual<T, N> &a, const Dual<T, N> &b) {
  Dual<T, N> r;
  r.v = a.v * b.v;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <class T, int N>
VA_HD Dual<T, N> operator/(const Dual<T, N> &a, const Dual<T, N> &b) {
  Dual<T, N> r;
  r.v = a.v / b.v;
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v;
  return r;
}
template <class T, int N>
VA_HD Dual<T, N> operator+(const Dual<T, N> &a, double b) { return a + Dual<T, N>(b); }
template <class T, int N>
VA_HD Dual<T, N> operator+(double a, const Dual<T, N> &b) { return Dual<T, N>(a) + b; }
template <class T, int N>
VA_HD Dual<T, N> operator-(const Dual<T, N> &a, double b) { return a - Dual<T, N>(b); }
template <class T, int N>
VA_HD Dual<T, N> operator-(double a, const Dual<T, N> &b) { return Dual<T, N>(a) - b; }
template <class T, int N>
VA_HD Dual<T, N> operator*(const Dual<T, N> &a, double b) {
  Dual<T, N> r;
  r.v = a.v * b;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <class T, int N>
VA_HD Dual<T, N> operator*(double a, const Dual<T, N> &b) { return b * a; }
template <class T, int N>
VA_HD Dual<T, N> operator/(const Dual<T, N> &a, double b) {
  Dual<T, N> r;
  r.v = a.v / b;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b;
  return r;
}
template <class T, int N>
VA_HD Dual<T, N> operator/(double a, const Dual<T, N> &b) { return Dual<T, N>(a) / b; }
template <class T, int N, class U>
VA_HD Dual<T, N> &operator+=(Dual<T, N> &a, const U &b) { return a = a + b; }
template <class T, int N, class U>
VA_HD Dual<T, N> &operator-=(Dual<T, N> &a, const U &b) { return a = a - b; }

// elementary functions
template <class T, int N>
VA_HD Dual<T, N> exp(const Dual<T, N> &x) { const T e = exp(x.v); return chain(x, e, e); }
template <class T, int N>
VA_HD Dual<T, N> log(const Dual<T, N> &x) { return chain(x, log(x.v), T(1.0) / x.v); }
template <class T, int N>
VA_HD Dual<T, N> log10(const Dual<T, N> &x) {
  return chain(x, log10(x.v), T(1.0) / (x.v * 2.30258509299404568402));
}
template <class T, int N>
VA_HD Dual<T, N> sqrt(const Dual<T, N> &x) { const T s = sqrt(x.v); return chain(x, s, T(0.5) / s); }
template <class T, int N>
VA_HD Dual<T, N> sin(const Dual<T, N> &x) { return chain(x, sin(x.v), cos(x.v)); }
template <class T, int N>
VA_HD Dual<T, N> cos(const Dual<T, N> &x) { return chain(x, cos(x.v), -sin(x.v)); }
template <class T, int N>
VA_HD Dual<T, N> tan(const Dual<T, N> &x) { const T t = tan(x.v); return chain(x, t, T(1.0) + t * t); }
template <class T, int N>
VA_HD Dual<T, N> sinh(const Dual<T, N> &x) { return chain(x, sinh(x.v), cosh(x.v)); }
template <class T, int N>
VA_HD Dual<T, N> cosh(const Dual<T, N> &x) { return chain(x, cosh(x.v), sinh(x.v)); }
template <class T, int N>
VA_HD Dual<T, N> tanh(const Dual<T, N> &x) { const T t = tanh(x.v); return chain(x, t, T(1.0) - t * t); }
template <class T, int N>
VA_HD Dual<T, N> atan(const Dual<T, N> &x) { return chain(x, atan(x.v), T(1.0) / (T(1.0) + x.v * x.v)); }
template <class T, int N>
VA_HD Dual<T, N> asin(const Dual<T, N> &x) { return chain(x, asin(x.v), T(1.0) / sqrt(T(1.0) - x.v * x.v)); }
template <class T, int N>
VA_HD Dual<T, N> acos(const Dual<T, N> &x) { return chain(x, acos(x.v), T(-1.0) / sqrt(T(1.0) - x.v * x.v)); }
template <class T, int N>
VA_HD Dual<T, N> fabs(const Dual<T, N> &x) { return val(x) < 0.0 ? -x : x; }
template <class T, int N>
VA_HD Dual<T, N> floor(const Dual<T, N> &x) { return Dual<T, N>(floor(val(x))); }
template <class T, int N>
VA_HD Dual<T, N> ceil(const Dual<T, N> &x) { return Dual<T, N>(ceil(val(x))); }
template <class T, int N>
VA_HD Dual<T, N> atan2(const Dual<T, N> &y, const Dual<T, N> &x) {
  Dual<T, N> r;
  r.v = atan2(y.v, x.v);
  const T den = x.v * x.v + y.v * y.v;
  for (int i = 0; i < N; ++i) r.d[i] = (x.v * y.d[i] - y.v * x.d[i]) / den;
  return r;
}
template <class T, int N>
VA_HD Dual<T, N> hypot(const Dual<T, N> &x, const Dual<T, N> &y) {
  Dual<T, N> r;
  r.v = hypot(x.v, y.v);
  for (int i = 0; i < N; ++i) r.d[i] = (x.v * x.d[i] + y.v * y.d[i]) / r.v;
  return r;
}
// d(x^p)/dx.  CedarSim takes pow's derivative from ChainRules 1.69 (its pow
// frule, src/va_env.jl:57-68): p y / x away from x = 0 and, at x = 0, 1 for
// p = 1, 0 for p = 0 or p > 1, +inf for 0 < p < 1.  p x^(p-1) agrees with that
// (away from 0 up to rounding) except for p = 0, where it is 0 * x^-1, NaN at
// x = 0.  x^0 is constant, so its partials are 0 everywhere (BSIM-CMG raises a
// smoothed V_ds that rounds to exactly 0 to the power DVTP1 = 0); any other p
// takes p x^(p-1), which also keeps second derivatives of nested duals at
// x = 0 (ddx of x^2).
template <class T>
VA_HD T pow_grad_x(const T &x, const T &p) {
  if (all_zero(p)) return T(0.0);
  return p * pow(x, p - T(1.0));
}
// x^y: with a constant exponent the log term is left out (a strong zero, so a
// negative base with an integral exponent keeps finite partials)
template <class T, int N>
VA_HD Dual<T, N> pow(const Dual<T, N> &x, const Dual<T, N> &y) {
  const T p = pow(x.v, y.v);
  Dual<T, N> r;
  r.v = p;
  const T dx = pow_grad_x(x.v, y.v);
  bool ycst = true;
  for (int i = 0; i < N; ++i)
    if (!all_zero(y.d[i])) ycst = false;
  if (ycst) {
    for (int i = 0; i < N; ++i) r.d[i] = sz_mul(dx, x.d[i]);
  } else {
    const T dy = p * log(x.v);
    for (int i = 0; i < N; ++i) r.d[i] = sz_mul(dx, x.d[i]) + sz_mul(dy, y.d[i]);
  }
  return r;
}

// limexp: exp below an exponent of 80, its tangent line above
VA_HD double limexp(double x) {
  const double X = 80.0;
  return x <= X ? exp(x) : exp(X) * (1.0 + (x - X));
}
template <class T, int N>
VA_HD Dual<T, N> limexp(const Dual<T, N> &x) {
  const double X = 80.0;
  if (val(x) <= X) return exp(x);
  const double e = exp(X);
  return Dual<T, N>(e) * (Dual<T, N>(1.0) + (x - Dual<T, N>(X)));
}

// mixed double / dual overloads of the two-argument functions
template <class T, int N>
VA_HD Dual<T, N> pow(const Dual<T, N> &x, double y) { return pow(x, Dual<T, N>(y)); }
template <class T, int N>
VA_HD Dual<T, N> pow(double x, const Dual<T, N> &y) { return pow(Dual<T, N>(x), y); }
template <class T, int N>
VA_HD Dual<T, N> atan2(const Dual<T, N> &y, double x) { return atan2(y, Dual<T, N>(x)); }
template <class T, int N>
VA_HD Dual<T, N> atan2(double y, const Dual<T, N> &x) { return atan2(Dual<T, N>(y), x); }
template <class T, int N>
VA_HD Dual<T, N> hypot(const Dual<T, N> &x, double y) { return hypot(x, Dual<T, N>(y)); }
template <class T, int N>
VA_HD Dual<T, N> hypot(double x, const Dual<T, N> &y) { return hypot(Dual<T, N>(x), y); }

// min / max pick one operand (its partials go with it)
VA_HD double vmin(double a, double b) { return a <= b ? a : b; }
VA_HD double vmax(double a, double b) { return a >= b ? a : b; }
template <class A, class B>
VA_HD auto vmin(const A &a, const B &b) -> decltype(a + b) {
  return val(a) <= val(b) ? decltype(a + b)(a) : decltype(a + b)(b);
}
template <class A, class B>
VA_HD auto vmax(const A &a, const B &b) -> decltype(a + b) {
  return val(a) >= val(b) ? decltype(a + b)(a) : decltype(a + b)(b);
}

// conditional expression c ? a : b with a common type
template <class A, class B>
VA_HD auto vsel(bool c, const A &a, const B &b) -> decltype(a + b) {
  return c ? decltype(a + b)(a) : decltype(a + b)(b);
}

// white_noise(pwr): zero in every analysis but noise; a noise evaluation passes
// nz and collects the source's power there
VA_HD double va_noise(double *nz, int j, double pwr) {
  if (nz) nz[j] += pwr;
  return 0.0;
}

// flicker_noise(pwr, ex): likewise zero outside a noise analysis, where it is a
// source of density pwr / f^ex; nz holds the n sources' powers, then their
// exponents (white sources keep exponent 0)
VA_HD double va_flicker(double *nz, int j, int n, double pwr, double ex) {
  if (nz) { nz[j] += pwr; nz[n + j] = ex; }
  return 0.0;
}

// Real to integer conversion (VA-LRM 4.2.1.1: round half away from zero) and
// integer division (truncation toward zero)
VA_HD double vint(double x) { return round(x); }
VA_HD double vidiv(double a, double b) { return trunc(a / b); }

// seeding and reading.  seed<D>(x, k): the k-th terminal potential.
template <class D>
struct Seed;
template <int N>
struct Seed<Dual<double, N>> {
  VA_HD static Dual<double, N> make(double x, int k) {
    Dual<double, N> r(x);
    r.d[k] = 1.0;
    return r;
  }
};
template <int N>
struct Seed<Dual<Dual<double, N>, N>> {
  VA_HD static Dual<Dual<double, N>, N> make(double x, int k) {
    Dual<Dual<double, N>, N> r(x);
    r.v.d[k] = 1.0;
    r.d[k] = Dual<double, N>(1.0);
    return r;
  }
};

// first partial d/dV_k of a first- or second-order value
template <int N>
VA_HD double part(const Dual<double, N> &x, int k) { return x.d[k]; }
template <int N>
VA_HD double part(const Dual<Dual<double, N>, N> &x, int k) { return x.v.d[k]; }

// ddx(x, V(a)) of a second-order value, as a second-order value: its value and
// first partials are exact, its (unused) second partials are left at zero
template <int N>
VA_HD Dual<Dual<double, N>, N> ddx(const Dual<Dual<double, N>, N> &x, int a) {
  Dual<Dual<double, N>, N> r;
  r.v = x.d[a];
  for (int i = 0; i < N; ++i) r.d[i] = Dual<double, N>(x.d[a].d[i]);
  return r;
}
VA_HD double ddx(double, int) { return 0.0; }

}  // namespace va
}  // namespace cedar
