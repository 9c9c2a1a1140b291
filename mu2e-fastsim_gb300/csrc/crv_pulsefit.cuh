// Pulse reconstruction: reco waveforms -> pulses (crv/crvfastsim/reco/pulsefit.py:49-316).
//
// Per waveform: pedestal (DB value, or the first sample when it undershoots the DB value by more than the
// threshold); then rounds: FindNextPeak from `start` (rising edge, optional plateau, falling edge with the plateau
// value above min_adc_difference), a fit window of up to samples_before / samples_after monotonic samples (one dropped
// on each side when more than one was added), a bounded Gumbel least-squares fit in sine-mapped internal coordinates
// (40 Levenberg-Marquardt steps, then 8 Gauss-Newton steps with halving, EDM and Hessian checks), the failed-fit
// fallback, then the rounded fit is subtracted from every sample and the search resumes at the window end.
//
// GPU mapping: one thread per waveform (FP64 throughput is scarce on this GPU, so no lane repeats another's uniform
// work): the waveform's samples sit in a global scratch mirror (L1-resident while the lane works on it), the peak
// search, the fit (sums sequential over the window, as the reference's contractions), the 3x3 solve (LU with partial
// pivoting) and the symmetric eigenvalues (cyclic Jacobi) run in the lane; pulses go to per-waveform record slots
// (rounds are bounded by half the samples).  R = double: every step in FP64; R = float (mixed): parameter mapping,
// residuals, Jacobians and sums in FP32 relative to the window's first sample, solve / acceptance / absolute times in
// FP64.
#pragma once
#include "crv_device.cuh"

namespace crv {

struct PulseRec {            // one reconstructed pulse (shared-memory staging)
  double pe, peph, time, height, beta, chi2, letime, ped, A, mu, b;
  int32_t seq;
  uint8_t failed, zerondf, pedfromdb, pad;
};

struct WaveIn {
  long long nw;              // waveforms
  const long long* off;      // first sample of waveform w in the sample array
  const int32_t* n;          // valid samples
  const long long* start_tdc;
  const double* ped_db;
  const double* area;
  const double* height;
  const int16_t* adc16;      // samples (one of adc16 / adc64)
  const long long* adc64;
};

__device__ __forceinline__ double round_half_away(double x) {
  double a = floor(fabs(x) + 0.5);
  return x < 0.0 ? -a : (x > 0.0 ? a : 0.0 * x);
}

// LU with partial pivoting (largest |a| in the column, first on ties), then substitution.  Returns false on a zero
// pivot (singular).
__device__ __forceinline__ bool solve3(const double M[3][3], const double r[3], double x[3]) {
  double a[3][3], b[3];
  for (int i = 0; i < 3; ++i) {
    b[i] = r[i];
    for (int j = 0; j < 3; ++j) a[i][j] = M[i][j];
  }
  for (int k = 0; k < 3; ++k) {
    int piv = k;
    double mx = fabs(a[k][k]);
    for (int i = k + 1; i < 3; ++i)
      if (fabs(a[i][k]) > mx) { mx = fabs(a[i][k]); piv = i; }
    if (a[piv][k] == 0.0) return false;
    if (piv != k) {
      for (int j = 0; j < 3; ++j) { double tmp = a[k][j]; a[k][j] = a[piv][j]; a[piv][j] = tmp; }
      double tb = b[k]; b[k] = b[piv]; b[piv] = tb;
    }
    double inv = 1.0 / a[k][k];
    for (int i = k + 1; i < 3; ++i) {
      double l = a[i][k] * inv;
      a[i][k] = l;
      for (int j = k + 1; j < 3; ++j) a[i][j] -= l * a[k][j];
      b[i] -= l * b[k];
    }
  }
  for (int i = 2; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < 3; ++j) s -= a[i][j] * x[j];
    x[i] = s / a[i][i];
  }
  return true;
}

// FP64 reciprocal from an FP32 seed and two Newton steps (24 -> 48 -> 96 bits): one FP32 MUFU op and four FP64
// FMAs instead of an FP64 division
__device__ __forceinline__ double rcp64(double d) {
  double r = double(__frcp_rn(float(d)));
  if (!(fabs(r) < 1e300) || r == 0.0) return 1.0 / d;       // outside the FP32 range: plain division
  r = r * (2.0 - d * r);
  r = r * (2.0 - d * r);
  return r;
}

// 3x3 solve by the adjugate (FP32-mixed fits): one reciprocal of the determinant
__device__ __forceinline__ bool solve3_adj(const double M[3][3], const double b[3], double x[3]) {
  double c00 = M[1][1] * M[2][2] - M[1][2] * M[2][1];
  double c01 = M[1][2] * M[2][0] - M[1][0] * M[2][2];
  double c02 = M[1][0] * M[2][1] - M[1][1] * M[2][0];
  double det = M[0][0] * c00 + M[0][1] * c01 + M[0][2] * c02;
  if (det == 0.0 || !isfinite(det)) return false;
  double c10 = M[0][2] * M[2][1] - M[0][1] * M[2][2];
  double c11 = M[0][0] * M[2][2] - M[0][2] * M[2][0];
  double c12 = M[0][1] * M[2][0] - M[0][0] * M[2][1];
  double c20 = M[0][1] * M[1][2] - M[0][2] * M[1][1];
  double c21 = M[0][2] * M[1][0] - M[0][0] * M[1][2];
  double c22 = M[0][0] * M[1][1] - M[0][1] * M[1][0];
  double inv = rcp64(det);
  x[0] = (c00 * b[0] + c10 * b[1] + c20 * b[2]) * inv;
  x[1] = (c01 * b[0] + c11 * b[1] + c21 * b[2]) * inv;
  x[2] = (c02 * b[0] + c12 * b[1] + c22 * b[2]) * inv;
  return true;
}

template <typename R>
__device__ __forceinline__ bool solve3_p(const double M[3][3], const double b[3], double x[3]) {
  return sizeof(R) == 8 ? solve3(M, b, x) : solve3_adj(M, b, x);
}

// eigenvalues of a symmetric 3x3 matrix (cyclic Jacobi), ascending
__device__ __forceinline__ void eig3(const double M[3][3], double e[3]) {
  double a[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) a[i][j] = M[i][j];
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
    double dg = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]);
    if (off == 0.0 || off <= 1e-300 || off < 1e-18 * dg) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        double apq = a[p][q];
        if (apq == 0.0) continue;
        double th = (a[q][q] - a[p][p]) / (2.0 * apq);
        double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) {        // A <- J^T A J
          double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
      }
  }
  e[0] = a[0][0]; e[1] = a[1][1]; e[2] = a[2][2];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2 - i; ++j)
      if (e[j] > e[j + 1]) { double tmp = e[j]; e[j] = e[j + 1]; e[j + 1] = tmp; }
}

struct Fit3 {
  double lo[3], hi[3], half[3];
  double t0;                 // time origin of the FP32 evaluation (first window sample)
};

// One lane's fit: residuals / normal equations at internal parameters u over the window points yw[0..P), times
// (tdc_fs + i) * period.  Sums are sequential over the points (the reference's contractions are sequential).
// R = double: every operation in FP64; R = float: mapping, residuals and sums in FP32 relative to the window start.
template <typename R>
__device__ __forceinline__ void eval_lane(const Fit3& F, const double u[3], const R* yw, long long tdc_fs,
                                          double period, int P, double* chi2, double H[6], double g[3]) {
  R A, mu, b, d0, d1, d2;
  if (sizeof(R) == 8) {
    double p0 = F.lo[0] + (F.hi[0] - F.lo[0]) * (sin(u[0]) + 1.0) * 0.5;
    double p1 = F.lo[1] + (F.hi[1] - F.lo[1]) * (sin(u[1]) + 1.0) * 0.5;
    double p2 = F.lo[2] + (F.hi[2] - F.lo[2]) * (sin(u[2]) + 1.0) * 0.5;
    A = R(p0); mu = R(p1); b = R(p2);
    d0 = R(F.half[0] * cos(u[0])); d1 = R(F.half[1] * cos(u[1])); d2 = R(F.half[2] * cos(u[2]));
  } else {
    float s0, c0, s1, c1, s2, c2;
    sincosf(float(u[0]), &s0, &c0);
    sincosf(float(u[1]), &s1, &c1);
    sincosf(float(u[2]), &s2, &c2);
    A = R(F.lo[0]) + R(F.hi[0] - F.lo[0]) * (s0 + 1.0f) * 0.5f;
    mu = R(F.lo[1] - F.t0) + R(F.hi[1] - F.lo[1]) * (s1 + 1.0f) * 0.5f;
    b = R(F.lo[2]) + R(F.hi[2] - F.lo[2]) * (s2 + 1.0f) * 0.5f;
    d0 = R(F.half[0]) * c0; d1 = R(F.half[1]) * c1; d2 = R(F.half[2]) * c2;
  }
  R c = 0, h00 = 0, h01 = 0, h02 = 0, h11 = 0, h12 = 0, h22 = 0, g0 = 0, g1 = 0, g2 = 0;
  for (int i = 0; i < P; ++i) {
    R t = sizeof(R) == 8 ? R(double(tdc_fs + i) * period) : R(float(i) * float(period));
    R z = (t - mu) / b;
    R ez, gg;
    if (sizeof(R) == 8) { ez = R(exp(double(-z))); gg = R(exp(double(-z - ez))); }
    else { ez = R(__expf(float(-z))); gg = R(__expf(float(-z - ez))); }
    R f = A * gg;
    R r = R(yw[i]) - f;
    R fz = f * (ez - R(1));
    R j0 = gg * d0;
    R j1 = fz * (R(-1) / b) * d1;
    R j2 = fz * (-z / b) * d2;
    c += r * r;
    h00 += j0 * j0; h01 += j0 * j1; h02 += j0 * j2;
    h11 += j1 * j1; h12 += j1 * j2; h22 += j2 * j2;
    g0 += j0 * r; g1 += j1 * r; g2 += j2 * r;
  }
  *chi2 = double(c);
  H[0] = double(h00); H[1] = double(h01); H[2] = double(h02); H[3] = double(h11); H[4] = double(h12);
  H[5] = double(h22);
  g[0] = double(g0); g[1] = double(g1); g[2] = double(g2);
}

__device__ __forceinline__ void sym3(const double H[6], double M[3][3]) {
  M[0][0] = H[0]; M[0][1] = M[1][0] = H[1]; M[0][2] = M[2][0] = H[2];
  M[1][1] = H[3]; M[1][2] = M[2][1] = H[4]; M[2][2] = H[5];
}

// bounded Gumbel fit of one lane (40 LM steps, 8 Gauss-Newton steps with halving, EDM + Hessian checks)
template <typename R>
__device__ void fit_lane(const Fit3& F, const double p0[3], const R* yw, long long tdc_fs, double period, int P,
                         int iters, double par[3], double* chi2_out, bool* conv, bool* hok) {
  double u[3];
  for (int k = 0; k < 3; ++k) {
    double c = 2.0 * (p0[k] - F.lo[k]) / (F.hi[k] - F.lo[k]) - 1.0;
    u[k] = asin(fmin(fmax(c, -1.0), 1.0));
  }
  double chi2, H[6], g[3];
  eval_lane<R>(F, u, yw, tdc_fs, period, P, &chi2, H, g);
  double lam = 1e-3;
  for (int it = 0; it < iters; ++it) {
    double M[3][3];
    sym3(H, M);
    for (int i = 0; i < 3; ++i) M[i][i] = M[i][i] + lam * (M[i][i] + 1e-12);
    double du[3];
    if (!solve3_p<R>(M, g, du)) du[0] = du[1] = du[2] = 0.0;
    double un[3] = {u[0] + du[0], u[1] + du[1], u[2] + du[2]};
    double c2, Hn[6], gn[3];
    eval_lane<R>(F, un, yw, tdc_fs, period, P, &c2, Hn, gn);
    bool better = c2 < chi2;
    if (better) {
      for (int k = 0; k < 3; ++k) { u[k] = un[k]; g[k] = gn[k]; }
      for (int k = 0; k < 6; ++k) H[k] = Hn[k];
      chi2 = c2;
    }
    lam = fmin(fmax(better ? lam * 0.3 : lam * 10.0, 1e-9), 1e9);
  }
  for (int it = 0; it < 8; ++it) {
    double M[3][3];
    sym3(H, M);
    for (int i = 0; i < 3; ++i) M[i][i] += 1e-12;
    double du[3];
    if (!solve3_p<R>(M, g, du)) break;
    for (int k = 0; k < 3; ++k)
      if (!isfinite(du[k])) du[k] = 0.0;
    for (int sc = 0; sc < 4; ++sc) {
      double s = sc == 0 ? 1.0 : (sc == 1 ? 0.5 : (sc == 2 ? 0.25 : 0.125));
      double un[3] = {u[0] + s * du[0], u[1] + s * du[1], u[2] + s * du[2]};
      double c2, Hn[6], gn[3];
      eval_lane<R>(F, un, yw, tdc_fs, period, P, &c2, Hn, gn);
      if (c2 < chi2) {
        for (int k = 0; k < 3; ++k) { u[k] = un[k]; g[k] = gn[k]; }
        for (int k = 0; k < 6; ++k) H[k] = Hn[k];
        chi2 = c2;
        break;                 // the accepted step zeroes du: later scales would re-evaluate the same point
      }
    }
  }
  double M[3][3];
  sym3(H, M);
  for (int i = 0; i < 3; ++i) M[i][i] += 1e-12;
  double st[3];
  double edm;
  bool okh;
  if (solve3_p<R>(M, g, st)) {
    edm = 0.5 * (g[0] * st[0] + g[1] * st[1] + g[2] * st[2]);
    double Hm[3][3], e[3];
    sym3(H, Hm);
    eig3(Hm, e);
    okh = e[0] > 1e-12 * fmax(e[2], 1e-300);
  } else {
    edm = INFINITY;
    okh = false;
  }
  *conv = isfinite(edm) && (edm <= 1e-3 * fmax(chi2, 1.0));
  *hok = okh;
  for (int k = 0; k < 3; ++k) par[k] = F.lo[k] + (F.hi[k] - F.lo[k]) * (sin(u[k]) + 1.0) * 0.5;
  *chi2_out = chi2;
}

// near-threshold local maximum among positions [a, b]
template <typename Y>
__device__ __forceinline__ bool near_lane(const Y* y, int n, int a, int b, Y thr, Y edge) {
  if (a < 0) a = 0;
  if (b > n - 1) b = n - 1;
  for (int i = a; i <= b; ++i) {
    Y left = i > 0 ? y[i - 1] : Y(-1e9);
    Y right = i + 1 < n ? y[i + 1] : Y(-1e9);
    Y d = y[i] - thr;
    if (y[i] >= left && y[i] > right && (d < Y(0) ? -d : d) <= edge) return true;
  }
  return false;
}

// FindNextPeak + fit window of one lane
template <typename Y>
__device__ __forceinline__ bool peak_lane(const CrvParams& p, const Y* y, int n, int start, int* ps_o, int* pe_o,
                                          int* fs_o, int* fe_o) {
  bool rising = false, found = false;
  int ps = 0, pe = 0;
  const Y thr = Y(p.min_adc_difference);
  for (int b = (start + 1 > 1 ? start + 1 : 1); b < n; ++b) {
    Y prev = y[b - 1], cur = y[b];
    if (prev < cur) { rising = true; ps = b; pe = b; }
    else if (prev == cur) { if (rising) pe = b; }
    else if (rising) {
      if (y[pe] > thr) { found = true; break; }
      rising = false;
    }
  }
  if (!found) return false;
  int fs = ps - 1, fe = pe + 1;
  for (int k = 1; k <= p.samples_before; ++k) {
    int i = ps - k;
    if (i < 0 || !(y[i] <= y[i + 1])) break;
    fs = i;
    if (i == 0) break;
  }
  for (int k = 1; k <= p.samples_after; ++k) {
    int i = pe + k;
    if (i >= n || !(y[i - 1] >= y[i])) break;
    fe = i;
  }
  if (ps - fs > 1) fs += 1;
  if (fe - pe > 1) fe -= 1;
  *ps_o = ps; *pe_o = pe; *fs_o = fs; *fe_o = fe;
  return true;
}

struct PulseSlots {
  const long long* off;      // per waveform: first record slot
  const int32_t* cap;        // per waveform: slots (rounds bound)
  int32_t* count;            // per waveform: pulses
  uint8_t* near;             // per waveform: wf_near_threshold
  PulseRec* rec;
};

__device__ __forceinline__ float round_half_away_f(float x) {
  float a = floorf(fabsf(x) + 0.5f);
  return x < 0.0f ? -a : (x > 0.0f ? a : 0.0f * x);
}

// subtract round(fit) from the samples it reaches: walk out from the mode while the rounded value can be non-zero
template <typename R>
__device__ __forceinline__ void subtract_lane(const CrvParams& p, R* y, int n, long long st_tdc, double A,
                                              double mu, double b, int* lo_o, int* hi_o) {
  long long im = (long long)floor(mu / p.period) - st_tdc;
  if (im < 0) im = 0;
  if (im > n - 1) im = n - 1;
  int lo = int(im), hi = int(im);
  // FP32: sample times relative to the mode's sample (exact small multiples of the period)
  const float mu_rel = float(mu - double(st_tdc + im) * p.period);
  const float inv_b = 1.0f / float(b), Af = float(A), Pf = float(p.period);
  for (int dir = -1; dir <= 1; dir += 2) {
    for (int i = int(im) + (dir > 0 ? 1 : 0); i >= 0 && i < n; i += dir) {
      if (sizeof(R) == 8) {
        double t = double(st_tdc + i) * p.period;
        double z = (t - mu) / b;
        double gv = A * exp(-z - exp(-z));
        y[i] -= R(round_half_away(gv));
        if (dir < 0) lo = i; else hi = i;
        // unimodal: past the mode the value only shrinks; stop well below the rounding threshold
        if (fabs(gv) < 0.25 && ((dir < 0 && t < mu) || (dir > 0 && t > mu))) break;
      } else {
        float tr = float(i - int(im)) * Pf;
        float z = (tr - mu_rel) * inv_b;
        float gv = Af * __expf(-z - __expf(-z));
        y[i] -= R(round_half_away_f(gv));
        if (dir < 0) lo = i; else hi = i;
        if (fabsf(gv) < 0.25f && ((dir < 0 && tr < mu_rel) || (dir > 0 && tr > mu_rel))) break;
      }
    }
  }
  *lo_o = lo;
  *hi_o = hi;
}

// one thread per waveform
template <typename R>
__global__ void __launch_bounds__(128) k_pulsefit(CrvParams p, WaveIn W, double* __restrict__ yscr, int max_pulses,
                                                 PulseSlots S, Status* status) {
  const double E = 2.718281828459045;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < W.nw;
       w += (long long)gridDim.x * blockDim.x) {
    int n = W.n[w];
    long long off = W.off[w];
    R* y = reinterpret_cast<R*>(yscr) + off;
    double pdb = W.ped_db[w];
    double x0 = n > 0 ? (W.adc16 ? double(W.adc16[off]) : double(W.adc64[off])) : 0.0;
    bool under = (n > 0) && (pdb - x0 > p.pedestal_undershoot);
    double ped = under ? x0 : pdb;
    if (sizeof(R) == 8) {
      for (int i = 0; i < n; ++i) y[i] = R((W.adc16 ? double(W.adc16[off + i]) : double(W.adc64[off + i])) - ped);
    } else {
      const float pf = float(ped);
      for (int i = 0; i < n; ++i) y[i] = R((W.adc16 ? float(W.adc16[off + i]) : float(W.adc64[off + i])) - pf);
    }
    const R thr = R(p.min_adc_difference), edge = R(p.knife_edge_adc);
    bool near = near_lane<R>(y, n, 0, n - 1, thr, edge);
    long long st_tdc = W.start_tdc[w];
    int start = 0, cnt = 0, cap = S.cap[w];
    long long slot = S.off[w];
    bool failed_before = false;
    for (int seq = 0; seq < max_pulses; ++seq) {
      int ps, pe, fs, fe;
      if (!peak_lane<R>(p, y, n, start, &ps, &pe, &fs, &fe)) break;
      int P = fe - fs + 1;
      double yps = double(y[ps]);
      double t_ps = double(st_tdc + ps) * p.period;
      double t_pe = double(st_tdc + pe) * p.period;
      double t_peak = 0.5 * (t_ps + t_pe);
      Fit3 F;
      F.lo[0] = yps * E * p.min_height_ratio; F.hi[0] = yps * E * p.max_height_ratio;
      F.lo[1] = t_ps - p.max_time_difference; F.hi[1] = t_pe + p.max_time_difference;
      F.lo[2] = p.min_beta; F.hi[2] = p.max_beta;
      for (int k = 0; k < 3; ++k) F.half[k] = (F.hi[k] - F.lo[k]) * 0.5;
      F.t0 = double(st_tdc + fs) * p.period;
      double p0[3] = {yps * E, t_peak, p.default_beta};
      double par[3], chi2;
      bool conv, hok;
      fit_lane<R>(F, p0, y + fs, st_tdc + fs, p.period, P, p.lm_iterations, par, &chi2, &conv, &hok);
      int ndf = P - 3;
      bool nearlim = false;
      for (int k = 0; k < 3; ++k) {
        double span = F.hi[k] - F.lo[k];
        if ((par[k] - F.lo[k]) / span < p.limit_tolerance || (F.hi[k] - par[k]) / span < p.limit_tolerance)
          nearlim = true;
      }
      bool failed = !conv || !hok || nearlim;
      double A = par[0], mu = par[1], b = par[2];
      double height = failed ? yps : A / E;
      double beta = failed ? p.default_beta : b;
      double tp = failed ? t_peak : mu;
      bool fseq = failed || failed_before;
      if (cnt < cap) {
        PulseRec& r = S.rec[slot + cnt];
        r.pe = (failed ? yps * E * p.default_beta : A * b) / W.area[w];
        r.peph = height / W.height[w];
        r.time = tp;
        r.height = height;
        r.beta = beta;
        r.chi2 = (failed || ndf <= 0) ? -1.0 : chi2 / double(ndf > 1 ? ndf : 1);
        r.letime = tp - p.le_time_factor * beta;
        r.ped = ped;
        r.A = A; r.mu = mu; r.b = b;
        r.seq = seq;
        r.failed = fseq; r.zerondf = ndf <= 0; r.pedfromdb = !under; r.pad = 0;
      }
      ++cnt;
      failed_before = fseq;
      int lo, hi;
      subtract_lane<R>(p, y, n, st_tdc, A, mu, b, &lo, &hi);
      near = near || near_lane<R>(y, n, lo - 1, hi + 1, thr, edge);
      start = fe;
    }
    S.count[w] = cnt;
    S.near[w] = near;
    if (cnt > cap) set_flag(status, CRV_ST_LIMIT);
  }
}

}  // namespace crv
