// k_ac.cu — small-signal AC and noise analysis about an operating point.
//
// CedarSim linearises the circuit at its DC operating point and evaluates the
// descriptor system (jωE − A)⁻¹B per frequency (src/ac.jl:73-104 ACSol,
// src/ac.jl:251-258 freqresp, src/ac.jl:107-171 NoiseSol, src/ac.jl:263-283 PSD).
// In this build's residual form F = Fi(x) + d/dt Fq(x) that system is
//   (G + jω C) X = b,   G = ∂Fi/∂x, C = ∂Fq/∂x at x_op,   b = −∂Fi/∂ε,
// which has the pattern of the transient Jacobian G + cj C.  The static pivot
// order, the fill pattern and the level-scheduled task lists of the LU and of
// the substitutions (plain and transposed) are therefore reused unchanged, in
// complex FP64.
//
//   ac_split_kernel   one thread per LU slot: G and C values of the slot, from
//                     the device outputs at x_op (cj = 1), split by out_q
//   ac_lane_kernel    one lane per frequency, 32 frequencies per warp in lockstep
//                     (circuits whose per-frequency workspace is small): the
//                     work of ac_kernel below with every FP64 instruction
//                     serving 32 frequencies
//   ac_kernel<false>  one warp per frequency: assemble G + jωC, LU, forward and
//                     back substitution of b, probed unknowns out
//   ac_kernel<true>   one warp per frequency: LU, then (G + jωC)ᵀ y = e_probe by
//                     the transposed substitutions (Uᵀ, then Lᵀ); the output PSD
//                     is Σ_r w_r |y_a − y_b|² over the thermal noise currents of
//                     the resistors (one transposed solve per frequency instead
//                     of one solve per noise source)
//   ac_dense_kernel   the static pivot order was chosen for the structure, not
//                     the values: at a metastable operating point (nodes held by
//                     gmin alone) and low ω its pivots can grow without bound.
//                     Every sparse solve is therefore checked by the residual of
//                     the assembled matrix; a frequency that fails it (or meets
//                     a zero pivot) is solved again, one warp per frequency, by a
//                     dense LU with partial pivoting (n ≤ kAcDenseNmax)
//
// Every warp runs the task lists in the same lane order and reduces with the
// same butterfly, so the result of a frequency does not depend on which warp
// ran it or on the grid: reruns are bitwise identical.
#include "kernels.cuh"

namespace cedar {

__device__ __forceinline__ double2 c_fms(double2 a, double2 b, double2 c) {   // a − b c
  return make_double2(a.x - (b.x * c.x - b.y * c.y), a.y - (b.x * c.y + b.y * c.x));
}
__device__ __forceinline__ double2 c_mul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double c_abs1(double2 a) { return fabs(a.x) + fabs(a.y); }
// 1 / z by Smith's method (R. L. Smith, "Algorithm 116: Complex division",
// CACM 5(8), 1962): scale by the larger component so neither |z|² nor the
// quotients overflow or underflow for representable z.
__device__ __forceinline__ double2 c_rcp(double2 z) {
  if (fabs(z.x) >= fabs(z.y)) {
    const double r = z.y / z.x, d = z.x + z.y * r;
    return make_double2(1.0 / d, -r / d);
  }
  const double r = z.x / z.y, d = z.x * r + z.y;
  return make_double2(r / d, -1.0 / d);
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double2 slot_val(const AcDev &a, int s, double w) {
  return make_double2(a.gval[s], w * a.cval[s]);
}
__device__ __forceinline__ double nan_value() { return __longlong_as_double(0x7ff8000000000000ll); }

__global__ void ac_split_kernel(DTpl T, const double *dout, double *gval, double *cval) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= T.nnz_lu) return;
  double g = 0.0, c = 0.0;
  for (int k = T.jlu_ptr[s]; k < T.jlu_ptr[s + 1]; ++k) {
    const int e = T.jlu_ent[k], o = e >> 1;
    const double v = (e & 1) ? -dout[o] : dout[o];
    if (T.out_q[o]) c += v; else g += v;
  }
  gval[s] = g;
  cval[s] = c;
}

// Backward error of a solve of M x = rhs (NOISE: Mᵀ x = rhs), M = G + jωC in
// internal order: ‖rhs − M x‖∞ against 1e-10 (‖M‖∞ ‖x‖∞ + ‖rhs‖∞) in the
// ν(z) = |Re z| + |Im z| norm.  True when the solve fails it or is not finite.
constexpr double kAcResidTol = 1e-10;

template <bool NOISE>
__device__ bool ac_solve_suspect(const AcDev &a, double w, const double2 *x, const double2 *rhs, int lane) {
  const DTpl &T = a.T;
  double rmax = 0.0, amax = 0.0, xmax = 0.0, bmax = 0.0;
  bool nonfinite = false;
  for (int i = lane; i < T.n; i += 32) {
    double2 r = rhs[i];
    double arow = 0.0;
    if (!NOISE) {
      for (int s = T.lu_rowptr[i]; s < T.lu_rowptr[i + 1]; ++s) {
        const double2 m = slot_val(a, s, w);
        r = c_fms(r, m, x[T.lu_colidx[s]]);
        arow += c_abs1(m);
      }
    } else {
      for (int k = T.lu_cptr[i]; k < T.lu_cptr[i + 1]; ++k) {
        const int s = T.lu_cslot[k];
        const double2 m = slot_val(a, s, w);
        r = c_fms(r, m, x[T.lu_srow[s]]);
        arow += c_abs1(m);
      }
    }
    const double ra = c_abs1(r), xa = c_abs1(x[i]);
    if (!(ra <= 1e300) || !(xa <= 1e300)) nonfinite = true;
    rmax = fmax(rmax, ra); amax = fmax(amax, arow); xmax = fmax(xmax, xa); bmax = fmax(bmax, c_abs1(rhs[i]));
  }
  nonfinite = __any_sync(0xffffffffu, nonfinite);
  rmax = warp_max(rmax); amax = warp_max(amax); xmax = warp_max(xmax); bmax = warp_max(bmax);
  return nonfinite || rmax > kAcResidTol * (amax * xmax + bmax);
}

// output PSD of frequency f from y (internal rows): Σ_r w_r / hz^e_r |y_a − y_b|²,
// hz = omega / 2π, e_r = 0 for white sources (noise_e null when all are white);
// fixed butterfly
__device__ double noise_sum(const AcDev &a, const double2 *y, long long f, int lane) {
  const DTpl &T = a.T;
  double acc = 0.0;
  for (int r = lane; r < a.n_noise; r += 32) {
    const int na = a.noise_a[r], nb = a.noise_b[r];
    const double2 ya = na < 0 ? make_double2(0.0, 0.0) : y[T.eq_pos[na]];
    const double2 yb = nb < 0 ? make_double2(0.0, 0.0) : y[T.eq_pos[nb]];
    const double hr = ya.x - yb.x, hi = ya.y - yb.y;
    double w = a.noise_w[r];
    if (a.noise_e) {
      const double e = a.noise_e[r];
      if (e != 0.0) w /= pow(a.omega[f] / 6.283185307179586, e);
    }
    acc += w * (hr * hr + hi * hi);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return acc;
}

// rhs of frequency f in internal order: b at its rows (AC), e at the probe's column (noise)
template <bool NOISE>
__device__ void ac_rhs(const AcDev &a, double2 *v, int lane) {
  const DTpl &T = a.T;
  if (!NOISE) {
    for (int e = lane; e < T.n; e += 32) v[T.eq_pos[e]] = make_double2(a.b[e], 0.0);
  } else {
    const int c = T.iorder[a.probe[0]];
    for (int u = lane; u < T.n; u += 32) v[u] = make_double2(u == c ? 1.0 : 0.0, 0.0);
  }
}

template <bool NOISE>
__device__ void ac_write_nan(const AcDev &a, long long f) {
  const double nan = nan_value();
  if (NOISE) a.psd[f] = nan;
  else for (int k = 0; k < a.n_probe; ++k) reinterpret_cast<double2 *>(a.resp)[f * a.n_probe + k] = make_double2(nan, nan);
}

template <bool NOISE>
__global__ void __launch_bounds__(128) ac_kernel(AcDev a) {
  const DTpl &T = a.T;
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (wid >= a.n_warps) return;            // a.ws holds n_warps workspaces
  double2 *lu = a.ws + wid * a.ws_stride, *rd = lu + T.nnz_lu, *v = rd + T.n, *rhs = v + T.n;
  for (long long f = wid; f < a.n_freq; f += a.n_warps) {
    const double w = a.omega[f];
    for (int s = lane; s < T.nnz_lu; s += 32) lu[s] = slot_val(a, s, w);
    __syncwarp();
    bool bad = false;
    for (int l = 0; l < T.lu_nlev; ++l) {
      for (int t = T.lu_lvl[l] + lane; t < T.lu_lvl[l + 1]; t += 32) {
        const int4 tk = T.lu_task[t];
        double2 acc = lu[tk.x];
        for (int p = tk.z; p < tk.w; ++p) { const int2 pr = T.lu_pair[p]; acc = c_fms(acc, lu[pr.x], lu[pr.y]); }
        const int kind = tk.y & 3, j = tk.y >> 2;
        if (kind == 2) acc = c_mul(acc, rd[j]);
        else if (kind == 1) {
          const double m = fmax(fabs(acc.x), fabs(acc.y));
          if (!(m > 1e-300) || !(m < 1e300)) bad = true;
          rd[j] = c_rcp(acc);
        }
        lu[tk.x] = acc;
      }
      __syncwarp();
    }
    bad = __any_sync(0xffffffffu, bad);
    if (!bad) {
      ac_rhs<NOISE>(a, v, lane);
      ac_rhs<NOISE>(a, rhs, lane);
      __syncwarp();
      if (!NOISE) {
        for (int l = 0; l < T.fw_nlev; ++l) {          // L y = b (unit diagonal)
          for (int t = T.fw_lvl[l] + lane; t < T.fw_lvl[l + 1]; t += 32) {
            const int4 tk = T.fw_task[t];
            double2 acc = v[tk.x];
            for (int p = tk.y; p < tk.z; ++p) { const int2 pr = T.fw_pair[p]; acc = c_fms(acc, lu[pr.x], v[pr.y]); }
            v[tk.x] = acc;
          }
          __syncwarp();
        }
        for (int l = 0; l < T.bw_nlev; ++l) {          // U x = y
          for (int t = T.bw_lvl[l] + lane; t < T.bw_lvl[l + 1]; t += 32) {
            const int4 tk = T.bw_task[t];
            double2 acc = v[tk.x];
            for (int p = tk.y; p < tk.z; ++p) { const int2 pr = T.bw_pair[p]; acc = c_fms(acc, lu[pr.x], v[pr.y]); }
            v[tk.x] = c_mul(acc, rd[tk.x]);
          }
          __syncwarp();
        }
      } else {
        for (int l = 0; l < T.tf_nlev; ++l) {          // Uᵀ z = e_probe
          for (int t = T.tf_lvl[l] + lane; t < T.tf_lvl[l + 1]; t += 32) {
            const int4 tk = T.tf_task[t];
            double2 acc = v[tk.x];
            for (int p = tk.y; p < tk.z; ++p) { const int2 pr = T.tf_pair[p]; acc = c_fms(acc, lu[pr.x], v[pr.y]); }
            v[tk.x] = c_mul(acc, rd[tk.x]);
          }
          __syncwarp();
        }
        for (int l = 0; l < T.tb_nlev; ++l) {          // Lᵀ y = z (unit diagonal)
          for (int t = T.tb_lvl[l] + lane; t < T.tb_lvl[l + 1]; t += 32) {
            const int4 tk = T.tb_task[t];
            double2 acc = v[tk.x];
            for (int p = tk.y; p < tk.z; ++p) { const int2 pr = T.tb_pair[p]; acc = c_fms(acc, lu[pr.x], v[pr.y]); }
            v[tk.x] = acc;
          }
          __syncwarp();
        }
      }
      bad = ac_solve_suspect<NOISE>(a, w, v, rhs, lane);
    }
    if (!bad) {
      if (!NOISE) {
        double2 *out = reinterpret_cast<double2 *>(a.resp) + f * a.n_probe;
        for (int k = lane; k < a.n_probe; k += 32) out[k] = v[T.iorder[a.probe[k]]];
      } else {
        const double p = noise_sum(a, v, f, lane);
        if (lane == 0) a.psd[f] = p;
      }
    } else if (lane == 0) {
      ac_write_nan<NOISE>(a, f);
      atomicAdd(a.n_dense, 1);
    }
    if (lane == 0) a.status[f] = bad ? kAcDense : CEDAR_ST_OK;
    __syncwarp();   // the workspace is reused by this warp's next frequency
  }
}

// One lane per frequency (circuits whose per-frequency workspace is small): a
// warp runs 32 frequencies through the same task lists in lockstep, so every
// task record and slot index is a broadcast load and every FP64 instruction
// serves 32 frequencies (on this part an FP64 warp instruction costs the same
// whatever its active mask).  The per-lane workspaces are interleaved, element e
// of lane l at ws[e * 32 + l], so each access of the warp is one contiguous
// 512-byte line.  Each task is summed in the pair order of ac_kernel and the
// residual check takes the same norms, so a frequency's response has the bits
// ac_kernel gives it; the noise PSD sums its sources in order (ac_kernel sums
// them lane-strided, then by a butterfly).
template <bool NOISE>
__global__ void __launch_bounds__(128) ac_lane_kernel(AcDev a) {
  const DTpl &T = a.T;
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (wid >= a.n_warps) return;
  double2 *const base = a.ws + wid * a.ws_stride * 32 + lane;
  const int n = T.n, nlu = T.nnz_lu;
  auto LU = [&](int s) -> double2 & { return base[(size_t)s * 32]; };
  auto RD = [&](int i) -> double2 & { return base[(size_t)(nlu + i) * 32]; };
  auto V = [&](int i) -> double2 & { return base[(size_t)(nlu + n + i) * 32]; };
  auto RHS = [&](int i) -> double2 & { return base[(size_t)(nlu + 2 * n + i) * 32]; };
  const int n_lu = T.lu_lvl[T.lu_nlev];
  for (long long f0 = wid * 32; f0 < a.n_freq; f0 += a.n_warps * 32) {
    const long long f = f0 + lane;
    const bool on = f < a.n_freq;
    const double w = a.omega[on ? f : f0];
    for (int s = 0; s < nlu; ++s) LU(s) = slot_val(a, s, w);
    bool bad = false;
    for (int t = 0; t < n_lu; ++t) {                   // level order: a level's tasks are independent
      const int4 tk = T.lu_task[t];
      double2 acc = LU(tk.x);
      for (int p = tk.z; p < tk.w; ++p) { const int2 pr = T.lu_pair[p]; acc = c_fms(acc, LU(pr.x), LU(pr.y)); }
      const int kind = tk.y & 3, j = tk.y >> 2;
      if (kind == 2) acc = c_mul(acc, RD(j));
      else if (kind == 1) {
        const double m = fmax(fabs(acc.x), fabs(acc.y));
        if (!(m > 1e-300) || !(m < 1e300)) bad = true;
        RD(j) = c_rcp(acc);
      }
      LU(tk.x) = acc;
    }
    if (!NOISE) {
      for (int e = 0; e < n; ++e) { const double2 b = make_double2(a.b[e], 0.0); V(T.eq_pos[e]) = b; RHS(T.eq_pos[e]) = b; }
      const int n_fw = T.fw_lvl[T.fw_nlev], n_bw = T.bw_lvl[T.bw_nlev];
      for (int t = 0; t < n_fw; ++t) {                 // L y = b (unit diagonal)
        const int4 tk = T.fw_task[t];
        double2 acc = V(tk.x);
        for (int p = tk.y; p < tk.z; ++p) { const int2 pr = T.fw_pair[p]; acc = c_fms(acc, LU(pr.x), V(pr.y)); }
        V(tk.x) = acc;
      }
      for (int t = 0; t < n_bw; ++t) {                 // U x = y
        const int4 tk = T.bw_task[t];
        double2 acc = V(tk.x);
        for (int p = tk.y; p < tk.z; ++p) { const int2 pr = T.bw_pair[p]; acc = c_fms(acc, LU(pr.x), V(pr.y)); }
        V(tk.x) = c_mul(acc, RD(tk.x));
      }
    } else {
      const int c = T.iorder[a.probe[0]];
      for (int u = 0; u < n; ++u) { const double2 e = make_double2(u == c ? 1.0 : 0.0, 0.0); V(u) = e; RHS(u) = e; }
      const int n_tf = T.tf_lvl[T.tf_nlev], n_tb = T.tb_lvl[T.tb_nlev];
      for (int t = 0; t < n_tf; ++t) {                 // U^T z = e_probe
        const int4 tk = T.tf_task[t];
        double2 acc = V(tk.x);
        for (int p = tk.y; p < tk.z; ++p) { const int2 pr = T.tf_pair[p]; acc = c_fms(acc, LU(pr.x), V(pr.y)); }
        V(tk.x) = c_mul(acc, RD(tk.x));
      }
      for (int t = 0; t < n_tb; ++t) {                 // L^T y = z (unit diagonal)
        const int4 tk = T.tb_task[t];
        double2 acc = V(tk.x);
        for (int p = tk.y; p < tk.z; ++p) { const int2 pr = T.tb_pair[p]; acc = c_fms(acc, LU(pr.x), V(pr.y)); }
        V(tk.x) = acc;
      }
    }
    // backward error of the solve (the norms of ac_solve_suspect, taken by one lane)
    double rmax = 0.0, amax = 0.0, xmax = 0.0, bmax = 0.0;
    bool nonfinite = false;
    for (int i = 0; i < n; ++i) {
      double2 r = RHS(i);
      double arow = 0.0;
      if (!NOISE) {
        for (int s = T.lu_rowptr[i]; s < T.lu_rowptr[i + 1]; ++s) {
          const double2 m = slot_val(a, s, w);
          r = c_fms(r, m, V(T.lu_colidx[s]));
          arow += c_abs1(m);
        }
      } else {
        for (int k = T.lu_cptr[i]; k < T.lu_cptr[i + 1]; ++k) {
          const int s = T.lu_cslot[k];
          const double2 m = slot_val(a, s, w);
          r = c_fms(r, m, V(T.lu_srow[s]));
          arow += c_abs1(m);
        }
      }
      const double ra = c_abs1(r), xa = c_abs1(V(i));
      if (!(ra <= 1e300) || !(xa <= 1e300)) nonfinite = true;
      rmax = fmax(rmax, ra); amax = fmax(amax, arow); xmax = fmax(xmax, xa); bmax = fmax(bmax, c_abs1(RHS(i)));
    }
    if (!bad) bad = nonfinite || rmax > kAcResidTol * (amax * xmax + bmax);
    if (on) {
      if (!bad) {
        if (!NOISE) {
          double2 *out = reinterpret_cast<double2 *>(a.resp) + f * a.n_probe;
          for (int k = 0; k < a.n_probe; ++k) out[k] = V(T.iorder[a.probe[k]]);
        } else {
          double acc = 0.0;
          for (int r = 0; r < a.n_noise; ++r) {
            const int na = a.noise_a[r], nb = a.noise_b[r];
            const double2 ya = na < 0 ? make_double2(0.0, 0.0) : V(T.eq_pos[na]);
            const double2 yb = nb < 0 ? make_double2(0.0, 0.0) : V(T.eq_pos[nb]);
            const double hr = ya.x - yb.x, hi = ya.y - yb.y;
            double wr = a.noise_w[r];
            if (a.noise_e) {
              const double e = a.noise_e[r];
              if (e != 0.0) wr /= pow(w / 6.283185307179586, e);
            }
            acc += wr * (hr * hr + hi * hi);
          }
          a.psd[f] = acc;
        }
      } else {
        ac_write_nan<NOISE>(a, f);
        atomicAdd(a.n_dense, 1);
      }
      a.status[f] = bad ? kAcDense : CEDAR_ST_OK;
    }
  }
}

// Dense rerun of the frequencies marked kAcDense: LU with partial pivoting (row
// interchanges of whole rows, pivot = largest ν in the column, lowest row on a
// tie), one warp per frequency; P M = L U.
template <bool NOISE>
__global__ void __launch_bounds__(128) ac_dense_kernel(AcDev a) {
  const DTpl &T = a.T;
  const int n = T.n, lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (wid >= a.n_dwarps) return;
  double2 *A = a.dws + wid * a.dws_stride, *r = A + (size_t)n * n;
  int *piv = a.dpiv + wid * n;
  for (long long f = wid; f < a.n_freq; f += a.n_dwarps) {
    if (a.status[f] != kAcDense) continue;            // the same value for every lane
    const double w = a.omega[f];
    for (long long i = lane; i < (long long)n * n; i += 32) A[i] = make_double2(0.0, 0.0);
    __syncwarp();
    for (int p = lane; p < n; p += 32)
      for (int s = T.lu_rowptr[p]; s < T.lu_rowptr[p + 1]; ++s) A[(size_t)p * n + T.lu_colidx[s]] = slot_val(a, s, w);
    ac_rhs<NOISE>(a, r, lane);
    __syncwarp();
    bool sing = false;
    for (int k = 0; k < n; ++k) {
      double best = -1.0; int bi = n;
      for (int i = k + lane; i < n; i += 32) { const double m = c_abs1(A[(size_t)i * n + k]); if (m > best) { best = m; bi = i; } }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (!(best > 0.0) || !(best < 1e300)) { sing = true; break; }
      if (lane == 0) piv[k] = bi;
      if (bi != k)
        for (int j = lane; j < n; j += 32) {
          const double2 t = A[(size_t)k * n + j]; A[(size_t)k * n + j] = A[(size_t)bi * n + j]; A[(size_t)bi * n + j] = t;
        }
      __syncwarp();
      const double2 inv = c_rcp(A[(size_t)k * n + k]);
      for (int i = k + 1 + lane; i < n; i += 32) {
        double2 *Ai = A + (size_t)i * n;
        const double2 l = c_mul(Ai[k], inv);
        Ai[k] = l;
        if (l.x == 0.0 && l.y == 0.0) continue;
        const double2 *Ak = A + (size_t)k * n;
        for (int j = k + 1; j < n; ++j) Ai[j] = c_fms(Ai[j], l, Ak[j]);
      }
      __syncwarp();
    }
    if (!sing) {
      if (!NOISE) {                                    // L U x = P b
        if (lane == 0)
          for (int k = 0; k < n; ++k) if (piv[k] != k) { const double2 t = r[k]; r[k] = r[piv[k]]; r[piv[k]] = t; }
        __syncwarp();
        for (int k = 0; k < n; ++k) {
          const double2 bk = r[k];
          for (int i = k + 1 + lane; i < n; i += 32) r[i] = c_fms(r[i], A[(size_t)i * n + k], bk);
          __syncwarp();
        }
        for (int k = n - 1; k >= 0; --k) {
          if (lane == 0) r[k] = c_mul(r[k], c_rcp(A[(size_t)k * n + k]));
          __syncwarp();
          const double2 bk = r[k];
          for (int i = lane; i < k; i += 32) r[i] = c_fms(r[i], A[(size_t)i * n + k], bk);
          __syncwarp();
        }
        double2 *out = reinterpret_cast<double2 *>(a.resp) + f * a.n_probe;
        for (int k = lane; k < a.n_probe; k += 32) out[k] = r[T.iorder[a.probe[k]]];
      } else {                                         // Mᵀ = Uᵀ Lᵀ P: Uᵀ w = e, Lᵀ u = w, y = Pᵀ u
        for (int k = 0; k < n; ++k) {
          if (lane == 0) r[k] = c_mul(r[k], c_rcp(A[(size_t)k * n + k]));
          __syncwarp();
          const double2 wk = r[k];
          for (int j = k + 1 + lane; j < n; j += 32) r[j] = c_fms(r[j], A[(size_t)k * n + j], wk);
          __syncwarp();
        }
        for (int k = n - 1; k >= 0; --k) {
          const double2 uk = r[k];
          for (int j = lane; j < k; j += 32) r[j] = c_fms(r[j], A[(size_t)k * n + j], uk);
          __syncwarp();
        }
        if (lane == 0)
          for (int k = n - 1; k >= 0; --k) if (piv[k] != k) { const double2 t = r[k]; r[k] = r[piv[k]]; r[piv[k]] = t; }
        __syncwarp();
        const double p = noise_sum(a, r, f, lane);
        if (lane == 0) a.psd[f] = p;
      }
    } else if (lane == 0) {
      ac_write_nan<NOISE>(a, f);
    }
    if (lane == 0) a.status[f] = sing ? CEDAR_ST_ZERO_PIVOT : CEDAR_ST_OK;
    __syncwarp();
  }
}

cudaError_t launch_ac_split(const DTpl &T, const double *dout, double *gval, double *cval, cudaStream_t s) {
  if (T.nnz_lu <= 0) return cudaSuccess;
  const int th = 256;
  ac_split_kernel<<<(T.nnz_lu + th - 1) / th, th, 0, s>>>(T, dout, gval, cval);
  return cudaGetLastError();
}

constexpr int kAcWarpsPerCta = 4;

cudaError_t launch_ac(const AcDev &a, bool noise, cudaStream_t s) {
  if (a.n_freq <= 0 || a.n_warps <= 0) return cudaSuccess;
  const long long grid = (a.n_warps + kAcWarpsPerCta - 1) / kAcWarpsPerCta;
  if (a.lane_mode) {
    if (noise) ac_lane_kernel<true><<<(unsigned)grid, 32 * kAcWarpsPerCta, 0, s>>>(a);
    else ac_lane_kernel<false><<<(unsigned)grid, 32 * kAcWarpsPerCta, 0, s>>>(a);
  } else {
    if (noise) ac_kernel<true><<<(unsigned)grid, 32 * kAcWarpsPerCta, 0, s>>>(a);
    else ac_kernel<false><<<(unsigned)grid, 32 * kAcWarpsPerCta, 0, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_ac_dense(const AcDev &a, bool noise, cudaStream_t s) {
  if (a.n_freq <= 0 || a.n_dwarps <= 0) return cudaSuccess;
  const long long grid = (a.n_dwarps + kAcWarpsPerCta - 1) / kAcWarpsPerCta;
  if (noise) ac_dense_kernel<true><<<(unsigned)grid, 32 * kAcWarpsPerCta, 0, s>>>(a);
  else ac_dense_kernel<false><<<(unsigned)grid, 32 * kAcWarpsPerCta, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace cedar
