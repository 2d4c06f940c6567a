// models.cuh — FP64 device-model evaluation (host + device), per-model outputs.
//
// Each device writes `nout` outputs (layout fixed per model, multiplicity folded
// in), output k at out[k * os]: a group's outputs are stored output-major (output
// k of device i at out_off + k * n_inst + i), so the devices a warp evaluates
// store each output contiguously.  The stamp programs built by compile.cpp then
// add signed outputs into J slots and residual rows.  Equations follow CedarSim:
//   R  I - V/res = 0                      src/simpledevices.jl:66-77
//   C  I - C ddt(V) = 0                   src/simpledevices.jl:105-109
//   L  V - L ddt(I) = 0                   src/simpledevices.jl:128-132
//   V  V - Vab = 0, I  I - Iab = 0        src/simpledevices.jl:280-300,325-339
//   E  V - gain (Vc+ - Vc-) = 0           src/simpledevices.jl:351-356
//   G  I - gain (Vc+ - Vc-) = 0           src/simpledevices.jl:368-373
//   MOS1 / DIODE / NLVCR: Verilog-A current contributions I(a,b) <+ expr, lowered
//   as in src/vasim.jl:128-180,836-839 (current leaves a, enters b).
// Derivatives are written out analytically (the CPU oracle differentiates the
// same equations with dual numbers, so the two are independent).
#pragma once
#ifdef __CUDACC__
#define CEDAR_HD __host__ __device__ __forceinline__
#else
#define CEDAR_HD inline
#include <cmath>
#endif
#include "../../include/cedar.h"
// Verilog-A models compiled by cedarsim.jl_gb300/va (the build writes this
// header into its own directory and puts it on the include path)
#include "va_models.gen.h"
// terminal values (terminals + branch current) the engines stage per device:
// 5 for the built-in models, more when a compiled Verilog-A model needs them
// (the generated header defines it then)
#ifndef CEDAR_MAX_TERM
#define CEDAR_MAX_TERM 5
#endif

namespace cedar {

// outputs / derived params / raw params / terminals(+branch) per model
// (must match kModels in compile.cpp)
CEDAR_HD int model_nout(int m) {
  switch (m) { case 1: return 2; case 2: return 3; case 3: return 6; case 4: return 4; case 5: return 1;
               case 6: return 5; case 7: return 2; case 8: return 4; case 9: return 2; case 10: return 4; }
  return va::nout(m - va::kBase);
}

// built-in models followed by the Verilog-A models (ids CEDAR_NMODELS ...)
static_assert(va::kBase == CEDAR_NMODELS, "Verilog-A model ids must follow the built-in ones");
constexpr int kNumModels = CEDAR_NMODELS + va::kCount;

// models whose devices carry charges (evaluated again for the integrator history)
CEDAR_HD bool model_has_q(int m) { return m == CEDAR_C || m == CEDAR_L || va::has_q(m - va::kBase); }

// thermal voltage k T / q at temperature temp_c (Celsius), $temperature = T+273.15
CEDAR_HD double thermal_voltage(double temp_c) {
  return 1.380649e-23 * (temp_c + 273.15) / 1.602176634e-19;
}

// raw (stride rs) -> derived (stride ds) parameters of one device
CEDAR_HD void derive_one(int model, const double *raw, int rs, double *dp, int ds, double vt) {
  switch (model) {
    case CEDAR_R: dp[0] = raw[rs] / raw[0]; break;                 // m / r
    case CEDAR_C: dp[0] = raw[rs] * raw[0]; break;                 // m * c
    case CEDAR_L: dp[0] = raw[rs]; dp[ds] = raw[0]; break;         // m, l
    case CEDAR_V: case CEDAR_I: for (int k = 0; k < 10; ++k) dp[k * ds] = raw[k * rs]; break;
    case CEDAR_E: dp[0] = raw[0]; dp[ds] = raw[rs]; break;         // gain, m
    case CEDAR_G: dp[0] = raw[rs] * raw[0]; break;                 // m * gain
    case CEDAR_MOS1: {
      double type = raw[0], W = raw[rs], L = raw[2 * rs], KP = raw[3 * rs], VTO = raw[4 * rs];
      dp[0] = type; dp[ds] = KP * W / L; dp[2 * ds] = type * VTO; dp[3 * ds] = raw[5 * rs]; dp[4 * ds] = raw[6 * rs];
    } break;
    case CEDAR_DIODE: dp[0] = raw[0] * raw[2 * rs]; dp[ds] = 1.0 / (raw[rs] * vt); dp[2 * ds] = raw[3 * rs]; break;
    case CEDAR_NLVCR: dp[0] = 2.0 * raw[0]; dp[ds] = raw[rs]; break;
    default: va::derive(model - va::kBase, raw, rs, dp, ds, vt); break;
  }
}

#if defined(__CUDA_ARCH__)
#define DADD(a, b) __dadd_rn((a), (b))
#define DMUL(a, b) __dmul_rn((a), (b))
#else
#define DADD(a, b) ((a) + (b))
#define DMUL(a, b) ((a) * (b))
#endif

// pwl_at_time (src/spectre_env.jl:43-69): index of the first point strictly after t
CEDAR_HD double pwl_at(const double *tv, int npts, double t) {
  int i = 0;
  while (i < npts && tv[2 * i] <= t) ++i;
  if (i <= 0) return tv[1];
  if (i >= npts) return tv[2 * (npts - 1) + 1];
  double y0 = tv[2 * (i - 1) + 1], y1 = tv[2 * i + 1], t0 = tv[2 * (i - 1)], t1 = tv[2 * i];
  if (y0 == y1) return y1;
  if (t1 == t0) return (y0 + y1) / 2;
  double slope = (y1 - y0) / (t1 - t0);
  return y0 + (t - t0) * slope;
}

// source value; p = derived params of the source (stride s): m dc kind a0..a6
CEDAR_HD double source_value(const double *p, int s, double t, bool dc, const double *pwl) {
  double dcv = p[s];
  if (dc) return dcv;
  int kind = (int)p[2 * s];
  if (kind == CEDAR_WAVE_PULSE) {
    double v1 = p[3 * s], v2 = p[4 * s], td = p[5 * s], tr = p[6 * s], tf = p[7 * s], pw = p[8 * s], per = p[9 * s];
    double tv[8] = {td, v1, td + tr, v2, td + tr + pw, v2, td + tr + pw + tf, v1};
    return pwl_at(tv, 4, fmod(t, per));
  }
  if (kind == CEDAR_WAVE_PWL) return pwl_at(pwl + (long long)p[3 * s], (int)p[4 * s], t);
  if (kind == CEDAR_WAVE_SIN) {
    double vo = p[3 * s], va = p[4 * s], freq = p[5 * s], td = p[6 * s], theta = p[7 * s], phase = p[8 * s], nc = p[9 * s];
    const double d2r = 3.14159265358979323846 / 180.0;
    if (td < t && t < nc / freq) return vo + va * exp(-(t - td) * theta) * sin((360.0 * freq * (t - td) + phase) * d2r);
    return vo + va * sin(phase * d2r);
  }
  return dcv;
}

// next corner of one source strictly after t + eps (time_periodic_singularity!)
CEDAR_HD double source_next_bp(const double *p, int s, double t, double eps, const double *pwl) {
  double best = 1e300;
  int kind = (int)p[2 * s];
  double te = DADD(t, eps);
  if (kind == CEDAR_WAVE_PULSE) {
    double td = p[5 * s], tr = p[6 * s], tf = p[7 * s], pw = p[8 * s], per = p[9 * s];
    double cs[4] = {td, td + tr, td + tr + pw, td + tr + pw + tf};
    for (int j = 0; j < 4; ++j) {
      double c = cs[j], bp;
      if (c > te) bp = c;
      else if (per > 0 && per < 1e300) {
        double k = floor((te - c) / per) + 1.0;
        bp = DADD(c, DMUL(k, per));
        if (!(bp > te)) bp = DADD(c, DMUL(k + 1.0, per));
      } else continue;
      best = bp < best ? bp : best;
    }
  } else if (kind == CEDAR_WAVE_PWL) {
    const double *tv = pwl + (long long)p[3 * s];
    int np = (int)p[4 * s];
    for (int k = 0; k < np; ++k) if (tv[2 * k] > te) { best = tv[2 * k] < best ? tv[2 * k] : best; break; }
  } else if (kind == CEDAR_WAVE_SIN) {
    double td = p[6 * s];
    if (td > te) best = td < best ? td : best;
  }
  return best;
}

struct EvalCtx {
  double t, cj, src_scale, gmin;
  bool dc;      // DC analysis: sources at dc values
  bool xdot;    // F part of charges = C * xdot (cedar_eval) instead of cj * Q (Newton)
};

// V / I source outputs given the source value vs (already scaled); same layout
// as eval_device.  Used when vs is cached once per Newton solve.
CEDAR_HD void eval_source_value(int model, const double *dp, const double *v, double vs, double *out, int os) {
  double m = dp[0];
  if (model == CEDAR_V) { out[0] = m * v[2]; out[os] = (v[0] - v[1]) - vs; out[2 * os] = m; out[3 * os] = 1.0; }
  else out[0] = m * vs;
}

// level-1 forward-mode current and partials (vds >= 0).  Both regions share one
// expression: with a = vds in triode (vds < vov) and a = vov in saturation,
//   id = beta clm (vov - a/2) a,  gm = beta clm a,
//   gds = beta clm (vov - a) + beta lam (vov - a/2) a,   clm = 1 + lam vds,
// which is the triode formula at a = vds and the saturation one (beta/2 vov^2 clm,
// beta vov clm, beta lam vov^2/2) at a = vov.  The region only selects a, so a warp
// whose lanes sit in different regions runs one instruction stream, and about
// half the FP64 operations of forming both regions' expressions are saved.
CEDAR_HD void mos1_fwd(double vgs, double vds, double vth, double beta, double lam,
                       double &id, double &gm, double &gds) {
  const double vov = vgs - vth;
  const double clm = 1.0 + lam * vds;
  const bool off = vov <= 0, tri = vds < vov;
  const double a = tri ? vds : vov;
  const double A = (vov - 0.5 * a) * a;
  const double bc = beta * clm;
  const double i = bc * A, g = bc * a, d = bc * (vov - a) + (beta * lam) * A;
  const double zero = 0.0;
  id = off ? zero : i;
  gm = off ? zero : g;
  gds = off ? zero : d;
}

// Sign and unit tests and the sign flip, on the bit patterns on the device (the
// integer pipe, not the FP64 pipe).  x * s for s = +1 or -1 is exact in IEEE
// arithmetic, so neg_if(x, s < 0) has the bits of the product.
CEDAR_HD double neg_if(double x, bool neg) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)((unsigned long long)neg << 63));
#else
  return neg ? -x : x;
#endif
}
CEDAR_HD bool is_unit(double a) {  // a is exactly +1 or -1
#ifdef __CUDA_ARCH__
  return (__double_as_longlong(a) & 0x7fffffffffffffffLL) == 0x3ff0000000000000LL;
#else
  return a == 1.0 || a == -1.0;
#endif
}
CEDAR_HD bool sign_set(double a) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(a) < 0;
#else
  return a < 0;
#endif
}
CEDAR_HD bool is_one(double a) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(a) == 0x3ff0000000000000LL;
#else
  return a == 1.0;
#endif
}

// Level-1 MOSFET terminal current and partials (outputs: Ids, dIds/dVg,
// dIds/dVd + gmin, -dIds/dVs + gmin, each times m).  gsum = gm + gds is formed
// without cancellation in reverse mode; the source/drain exchange for vds < 0 is
// a selection (no divergent branch).  UNIT: type is +-1 and m is 1 (the usual
// case), so the products by type are sign flips and those by m are left out;
// both are exact, so the outputs have the bits of the general form.
template <bool UNIT>
CEDAR_HD void mos1_device(double type, double beta, double vth, double lam, double m, const double *v, double gmin,
                          double *out, int os) {
  const bool pt = UNIT && sign_set(type);
  auto tm = [&](double x) -> double {
    if constexpr (UNIT) return neg_if(x, pt);
    else return type * x;
  };
  auto mm = [&](double x) -> double {
    if constexpr (UNIT) return x;
    else return m * x;
  };
  const double vgs = tm(v[1] - v[2]), vds = tm(v[0] - v[2]);
  const bool fwd = vds >= 0;
  double i1, g1, g2;
  // the reversed-mode negations as sign flips (integer ops, exact)
  mos1_fwd(fwd ? vgs : vgs - vds, neg_if(vds, !fwd), vth, beta, lam, i1, g1, g2);
  const double s12 = g1 + g2;
  const double id = neg_if(i1, !fwd), gm = neg_if(g1, !fwd), gds = fwd ? g2 : s12, gsum = fwd ? s12 : g2;
  const double ids = fma(gmin, v[0] - v[2], tm(id));
  out[0] = mm(ids); out[os] = mm(gm); out[2 * os] = mm(gds + gmin); out[3 * os] = mm(gsum + gmin);
}

// The source waveform out of line: the batched engines take time-varying sources'
// values from a per-solve cache, so the waveform code on the Newton iteration's
// path only serves constant sources; a call keeps its code out of the hot loop.
#if defined(__CUDACC__)
static __host__ __device__ __noinline__
#else
static inline
#endif
double source_value_cold(const double *p, int s, double t, bool dc, const double *pwl) {
  return source_value(p, s, t, dc, pwl);
}

// Evaluate one device.  v[k]: terminal (+branch) unknown values, vd[k]: their
// time derivatives (only when ctx.xdot).  dp: derived params with stride ds.
// HOT_SRC false: V / I source values through source_value_cold.
template <bool HOT_SRC = true>
CEDAR_HD void eval_device(int model, const double *dp, int ds, const double *v, const double *vd,
                          const EvalCtx &ctx, const double *pwl, double *out, int os) {
  switch (model) {
    case CEDAR_R: {
      double gm = dp[0];
      out[0] = gm * (v[0] - v[1]); out[os] = gm;
    } break;
    case CEDAR_C: {
      double mc = dp[0];
      double Q = mc * (v[0] - v[1]);
      out[0] = ctx.xdot ? mc * (vd[0] - vd[1]) : ctx.cj * Q;
      out[os] = ctx.cj * mc; out[2 * os] = Q;
    } break;
    case CEDAR_L: {
      double m = dp[0], l = dp[ds], I = v[2];
      out[0] = m * I;
      out[os] = (v[0] - v[1]) - (ctx.xdot ? l * vd[2] : ctx.cj * (l * I));
      out[2 * os] = m; out[3 * os] = 1.0; out[4 * os] = ctx.cj * l; out[5 * os] = l * I;
    } break;
    case CEDAR_V: {
      double m = dp[0];
      double vs = (HOT_SRC ? source_value(dp, ds, ctx.t, ctx.dc, pwl) : source_value_cold(dp, ds, ctx.t, ctx.dc, pwl)) *
                  ctx.src_scale;
      out[0] = m * v[2]; out[os] = (v[0] - v[1]) - vs; out[2 * os] = m; out[3 * os] = 1.0;
    } break;
    case CEDAR_I: {
      double m = dp[0];
      out[0] = m * ((HOT_SRC ? source_value(dp, ds, ctx.t, ctx.dc, pwl) : source_value_cold(dp, ds, ctx.t, ctx.dc, pwl)) *
                    ctx.src_scale);
    } break;
    case CEDAR_E: {
      double gain = dp[0], m = dp[ds];
      out[0] = m * v[4]; out[os] = (v[0] - v[1]) - gain * (v[2] - v[3]); out[2 * os] = m; out[3 * os] = 1.0; out[4 * os] = gain;
    } break;
    case CEDAR_G: {
      double mg = dp[0];
      out[0] = mg * (v[2] - v[3]); out[os] = mg;
    } break;
    case CEDAR_MOS1: {
      const double type = dp[0], beta = dp[ds], vth = dp[2 * ds], lam = dp[3 * ds], m = dp[4 * ds];
      if (is_unit(type) && is_one(m)) mos1_device<true>(type, beta, vth, lam, m, v, ctx.gmin, out, os);
      else mos1_device<false>(type, beta, vth, lam, m, v, ctx.gmin, out, os);
    } break;
    case CEDAR_DIODE: {
      double isat = dp[0], invnvt = dp[ds], m = dp[2 * ds];
      double vv = v[0] - v[1], a = vv * invnvt, e, I, gd;
      if (a <= 80.0) { e = exp(a); I = isat * (e - 1.0); gd = isat * e * invnvt; }
      else { e = exp(80.0); I = isat * (e * (1.0 + (a - 80.0)) - 1.0); gd = isat * e * invnvt; }
      I += ctx.gmin * vv; gd += ctx.gmin;
      out[0] = m * I; out[os] = m * gd;
    } break;
    case CEDAR_NLVCR: {
      double tR = dp[0], m = dp[ds];
      double vgs = v[1] - v[2], vds = v[0] - v[2];
      out[0] = m * (vds * (tR * vgs)); out[os] = m * (tR * vgs); out[2 * os] = m * (tR * vds); out[3 * os] = m * (tR * (vgs + vds));
    } break;
    default:  // Verilog-A models
      va::eval(model - va::kBase, dp, ds, v, vd, ctx.xdot, ctx.cj, ctx.gmin, out, os);
      break;
  }
}

}  // namespace cedar
