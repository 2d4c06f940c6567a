// opcount.cpp — host build tool: the FP64 operation count of one device
// evaluation per model, obtained by running the engines' own device code
// (models.cuh and the emitted Verilog-A code) on an op-counting scalar.
//
// Every `double` of that code is compiled here as `Cnt`, a value that counts the
// arithmetic it takes part in: add / sub / mul / div = 1, fma = 2 (a compiled
// a * b + c is one FMA, counted as its multiply and add), exp / log / sqrt and
// the other transcendental calls 1 each.  Comparisons, negation and selections
// are not operations.  The counts are taken at one operating point per model
// (each model's code has no data-dependent loops; the branch taken by the
// diode's limexp and the Verilog-A strong zeros follow the point).
//
// Output (stdout): a C++ header with `kFlopsBuiltin[]` and `kFlopsVA[]`, the
// per-iteration work of a device in the engines' Newton iteration (for V and I
// sources: the cached-value stamp, eval_source_value; the source waveform is
// evaluated once per Newton solve).  cedar_ckt_costs sums them per circuit.
// Build and run: build.py (g++ -std=c++17, before the CUDA units).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

struct Cnt;
static long long g_ops = 0;

struct Cnt {
  double v;
  Cnt() : v(0.0) {}
  Cnt(double x) : v(x) {}  // NOLINT: literals and parameters convert implicitly
  Cnt(int x) : v((double)x) {}
  Cnt(long long x) : v((double)x) {}
  explicit operator int() const { return (int)v; }
  explicit operator long long() const { return (long long)v; }
  explicit operator bool() const { return v != 0.0; }
  // implicit: the dual-number templates construct their values from doubles
  operator double() const { return v; }  // NOLINT
};
static inline Cnt op1(double r) { ++g_ops; return Cnt(r); }
static inline Cnt operator+(Cnt a, Cnt b) { return op1(a.v + b.v); }
static inline Cnt operator-(Cnt a, Cnt b) { return op1(a.v - b.v); }
static inline Cnt operator*(Cnt a, Cnt b) { return op1(a.v * b.v); }
static inline Cnt operator/(Cnt a, Cnt b) { return op1(a.v / b.v); }
static inline Cnt operator-(Cnt a) { return Cnt(-a.v); }
static inline Cnt &operator+=(Cnt &a, Cnt b) { a = a + b; return a; }
static inline Cnt &operator-=(Cnt &a, Cnt b) { a = a - b; return a; }
static inline Cnt &operator*=(Cnt &a, Cnt b) { a = a * b; return a; }
static inline Cnt &operator/=(Cnt &a, Cnt b) { a = a / b; return a; }
static inline bool operator<(Cnt a, Cnt b) { return a.v < b.v; }
static inline bool operator<=(Cnt a, Cnt b) { return a.v <= b.v; }
static inline bool operator>(Cnt a, Cnt b) { return a.v > b.v; }
static inline bool operator>=(Cnt a, Cnt b) { return a.v >= b.v; }
static inline bool operator==(Cnt a, Cnt b) { return a.v == b.v; }
static inline bool operator!=(Cnt a, Cnt b) { return a.v != b.v; }
static inline bool operator!(Cnt a) { return a.v == 0.0; }
// mixed with plain doubles (literals): exact overloads, so no conversion is ambiguous
#define CEDAR_CNT_MIX(op)                                                   \
  static inline Cnt operator op(Cnt a, double b) { return a op Cnt(b); }   \
  static inline Cnt operator op(double a, Cnt b) { return Cnt(a) op b; }   \
  static inline Cnt operator op(Cnt a, int b) { return a op Cnt(b); }      \
  static inline Cnt operator op(int a, Cnt b) { return Cnt(a) op b; }
CEDAR_CNT_MIX(+) CEDAR_CNT_MIX(-) CEDAR_CNT_MIX(*) CEDAR_CNT_MIX(/)
#undef CEDAR_CNT_MIX
#define CEDAR_CNT_CMP(op)                                                        \
  static inline bool operator op(Cnt a, double b) { return a.v op b; }          \
  static inline bool operator op(double a, Cnt b) { return a op b.v; }          \
  static inline bool operator op(Cnt a, int b) { return a.v op (double)b; }     \
  static inline bool operator op(int a, Cnt b) { return (double)a op b.v; }
CEDAR_CNT_CMP(<) CEDAR_CNT_CMP(<=) CEDAR_CNT_CMP(>) CEDAR_CNT_CMP(>=) CEDAR_CNT_CMP(==) CEDAR_CNT_CMP(!=)
#undef CEDAR_CNT_CMP
#define CEDAR_CNT_F1(f) static inline Cnt f(Cnt a) { return op1(std::f(a.v)); }
CEDAR_CNT_F1(exp) CEDAR_CNT_F1(log) CEDAR_CNT_F1(log10) CEDAR_CNT_F1(sqrt) CEDAR_CNT_F1(sin) CEDAR_CNT_F1(cos)
CEDAR_CNT_F1(tan) CEDAR_CNT_F1(asin) CEDAR_CNT_F1(acos) CEDAR_CNT_F1(atan) CEDAR_CNT_F1(sinh) CEDAR_CNT_F1(cosh)
CEDAR_CNT_F1(tanh)
#undef CEDAR_CNT_F1
static inline Cnt fabs(Cnt a) { return Cnt(std::fabs(a.v)); }
static inline Cnt floor(Cnt a) { return Cnt(std::floor(a.v)); }
static inline Cnt ceil(Cnt a) { return Cnt(std::ceil(a.v)); }
static inline Cnt trunc(Cnt a) { return Cnt(std::trunc(a.v)); }
static inline Cnt round(Cnt a) { return Cnt(std::round(a.v)); }
static inline Cnt fmod(Cnt a, Cnt b) { return op1(std::fmod(a.v, b.v)); }
static inline Cnt pow(Cnt a, Cnt b) { return op1(std::pow(a.v, b.v)); }
static inline Cnt atan2(Cnt a, Cnt b) { return op1(std::atan2(a.v, b.v)); }
static inline Cnt hypot(Cnt a, Cnt b) { return op1(std::hypot(a.v, b.v)); }
static inline Cnt fmin(Cnt a, Cnt b) { return Cnt(std::fmin(a.v, b.v)); }
static inline Cnt fmax(Cnt a, Cnt b) { return Cnt(std::fmax(a.v, b.v)); }
static inline Cnt fma(Cnt a, Cnt b, Cnt c) { g_ops += 2; return Cnt(std::fma(a.v, b.v, c.v)); }
// two-argument functions with one plain double (a literal exponent, as BSIM-CMG's
// pow(x, 0.719)): exact overloads, as for the operators above
#define CEDAR_CNT_F2MIX(f)                                             \
  static inline Cnt f(Cnt a, double b) { return f(a, Cnt(b)); }        \
  static inline Cnt f(double a, Cnt b) { return f(Cnt(a), b); }
CEDAR_CNT_F2MIX(pow) CEDAR_CNT_F2MIX(atan2) CEDAR_CNT_F2MIX(hypot) CEDAR_CNT_F2MIX(fmod)
#undef CEDAR_CNT_F2MIX
static inline bool isfinite(Cnt a) { return std::isfinite(a.v); }
static inline bool isnan(Cnt a) { return std::isnan(a.v); }
static inline long long llround(Cnt a) { return std::llround(a.v); }

// Helpers the dual-number templates find by argument-dependent lookup.
static inline double val(Cnt x) { return x.v; }
static inline bool all_zero(Cnt x) { return x.v == 0.0; }

// The library header and the dual-number templates keep real doubles (their
// constants and interfaces); the device code itself -- built-in models and the
// emitted Verilog-A bodies -- is compiled with every double an op-counting scalar.
#include <stddef.h>
#include "../../include/cedar.h"
#include "va_dual.cuh"

// seeding and reading of counting duals (va_dual.cuh specialises them for double)
namespace cedar {
namespace va {
template <int N>
struct Seed<Dual<Cnt, N>> {
  static Dual<Cnt, N> make(Cnt x, int k) { Dual<Cnt, N> r; r.v = x; r.d[k] = Cnt(1.0); return r; }
};
template <int N>
struct Seed<Dual<Dual<Cnt, N>, N>> {
  static Dual<Dual<Cnt, N>, N> make(Cnt x, int k) {
    Dual<Dual<Cnt, N>, N> r;
    r.v.v = x;
    r.v.d[k] = Cnt(1.0);
    r.d[k].v = Cnt(1.0);
    return r;
  }
};
template <int N>
Cnt part(const Dual<Cnt, N> &x, int k) { return x.d[k]; }
template <int N>
Cnt part(const Dual<Dual<Cnt, N>, N> &x, int k) { return x.v.d[k]; }
template <int N>
Dual<Dual<Cnt, N>, N> ddx(const Dual<Dual<Cnt, N>, N> &x, int a) {
  Dual<Dual<Cnt, N>, N> r;
  r.v = x.d[a];
  for (int i = 0; i < N; ++i) r.d[i].v = x.d[a].d[i];
  return r;
}
inline double va_noise(Cnt *, int, double) { return 0.0; }
inline double va_flicker(Cnt *, int, int, double, double) { return 0.0; }
}  // namespace va
}  // namespace cedar

#define double Cnt
#include "models.cuh"
#undef double

using cedar::EvalCtx;

// terminal values for the counting point of a model with nt inputs
static void point(int nt, Cnt *v) {
  const double vals[] = {0.9, 0.55, 0.05, 0.0, 0.3, -0.2, 0.7, 0.1};
  for (int k = 0; k < nt; ++k) v[k] = Cnt(vals[k % 8]);
}

int main() {
  using namespace cedar;
  const int nb = CEDAR_NMODELS;
  Cnt dp[64], raw[64], v[16], out[4096];
  std::printf("// Generated by cedarsim.jl_gb300/csrc/opcount.cpp at build time; do not edit.\n");
  std::printf("// FP64 operations of one device evaluation in the engines' Newton iteration,\n");
  std::printf("// counted by running the device code on an op-counting scalar.\n#pragma once\n");
  std::printf("namespace cedar { namespace flops {\n");
  std::printf("static const int kBuiltin[%d] = {0", nb);
  for (int m = 1; m < nb; ++m) {
    for (int k = 0; k < 64; ++k) raw[k] = Cnt(1.0);
    // parameters that keep each model in its ordinary region: MOS1 n-type on,
    // sources at a DC value, diode forward below the limexp knee
    if (m == CEDAR_MOS1) { raw[0] = 1.0; raw[1] = 2e-6; raw[2] = 1e-6; raw[3] = 2e-4; raw[4] = 0.45; raw[5] = 0.0; }
    if (m == CEDAR_DIODE) { raw[0] = 1e-14; raw[1] = 1.0; raw[2] = 1.0; }
    if (m == CEDAR_V || m == CEDAR_I) { raw[2] = 0.0; }
    derive_one(m, raw, 1, dp, 1, 0.025852);
    // terminal values per built-in model (terminals + branch current)
    static const int kIn[CEDAR_NMODELS] = {0, 2, 2, 3, 3, 2, 5, 4, 4, 2, 3};
    point(kIn[m], v);
    EvalCtx ctx{1e-9, 1e12, 1.0, 1e-12, false, false};
    g_ops = 0;
    if (m == CEDAR_V || m == CEDAR_I) eval_source_value(m, dp, v, Cnt(0.8), out, 1);
    else eval_device(m, dp, 1, v, nullptr, ctx, nullptr, out, 1);
    std::printf(", %lld", g_ops);
  }
  std::printf("};\n");
  std::printf("static const int kVA[%d] = {", va::kCount > 0 ? va::kCount : 1);
  for (int k = 0; k < va::kCount; ++k) {
    const int np = va::kNPar[k];
    for (int q = 0; q < 64; ++q) raw[q] = Cnt(0.0);
    for (int q = 0; q < np; ++q) raw[q] = Cnt(1.0);
    derive_one(va::kBase + k, raw, 1, dp, 1, 0.025852);
    point(va::kNTerm[k] + va::kHasBr[k], v);
    g_ops = 0;
    va::eval(k, dp, 1, v, nullptr, false, Cnt(1e12), Cnt(1e-12), out, 1);
    std::printf("%s%lld", k ? ", " : "", g_ops);
  }
  if (va::kCount == 0) std::printf("0");
  std::printf("};\n} }\n");
  return 0;
}
