// Pulse reconstruction: reco waveforms -> pulses (crv/crvfastsim/reco/pulsefit.py:49-316).
//
// Per waveform: pedestal (DB value, or the first sample when it undershoots the DB value by more than the
// threshold); then rounds: FindNextPeak from `start` (rising edge, optional plateau, falling edge with the plateau
// value above min_adc_difference), a fit window of up to samples_before / samples_after monotonic samples (one dropped
// on each side when more than one was added), a bounded Gumbel least-squares fit in sine-mapped internal coordinates
// (40 Levenberg-Marquardt steps, then 8 Gauss-Newton steps with halving, EDM and Hessian checks), the failed-fit
// fallback, then the rounded fit is subtracted from every sample and the search resumes at the window end.
//
// GPU mapping: one lane per fit (FP64 throughput is scarce on this GPU, so no lane repeats another's uniform work).
// Pulses are found in rounds over a device task list (one pulse per pending waveform per round, see k_pf_round), so
// the lanes of a warp run the same fit schedule; the waveform's samples sit in a global scratch mirror, the peak
// search, the fit (sums sequential over the window, as the reference's contractions), the 3x3 solve and the symmetric
// eigenvalues (cyclic Jacobi) run in the lane; pulses go to per-waveform record slots (rounds are bounded by half the
// samples).  R = double: every step in FP64, the solve by LU with partial pivoting.  R = float (mixed): parameter
// mapping, residuals, Jacobians, sums and the fit state in FP32 relative to the window's first sample; the
// normal-equation solve in float-float arithmetic on the FP32 pipe (FP64 for values outside FP32's comfortable
// range); absolute pulse times in FP64.
#pragma once
#include "crv_device.cuh"

namespace crv {

struct PulseRec {            // one reconstructed pulse (shared-memory staging)
  double pe, peph, time, height, beta, chi2, letime, ped, A, mu, b;
  int32_t seq;
  uint8_t failed, zerondf, pedfromdb, pad;
};

struct WaveIn {
  long long nw;              // waveforms (an upper bound when nw_dev is set)
  const long long* nw_dev;   // device count of waveforms, or null
  const long long* off;      // first sample of waveform w in the sample array
  const int32_t* n;          // valid samples
  const long long* start_tdc;
  const double* ped_db;
  const double* area;
  const double* height;
  const int16_t* adc16;      // samples (one of adc16 / adc64)
  const long long* adc64;
  long long nsamples;        // rows of the sample array: every waveform must lie inside it
};

__device__ __forceinline__ double round_half_away(double x) {
  double a = floor(fabs(x) + 0.5);
  return x < 0.0 ? -a : (x > 0.0 ? a : 0.0 * x);
}

// LU with partial pivoting (largest |a| in the column, first on ties), then substitution.  Returns false on a zero
// pivot (singular).
static __device__ __noinline__ bool solve3(const double M[3][3], const double r[3], double x[3]) {
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
static __device__ __noinline__ void eig3(const double M[3][3], double e[3]) {
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
static __device__ __noinline__ void eval_lane(const Fit3& F, const double u[3], const R* yw, long long tdc_fs,
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
    bool moved = false;
    for (int sc = 0; sc < 4; ++sc) {
      double s = sc == 0 ? 1.0 : (sc == 1 ? 0.5 : (sc == 2 ? 0.25 : 0.125));
      double un[3] = {u[0] + s * du[0], u[1] + s * du[1], u[2] + s * du[2]};
      double c2, Hn[6], gn[3];
      eval_lane<R>(F, un, yw, tdc_fs, period, P, &c2, Hn, gn);
      if (c2 < chi2) {
        for (int k = 0; k < 3; ++k) { u[k] = un[k]; g[k] = gn[k]; }
        for (int k = 0; k < 6; ++k) H[k] = Hn[k];
        chi2 = c2;
        moved = true;
        break;                 // the accepted step zeroes du: later scales would re-evaluate the same point
      }
    }
    if (!moved) break;         // state unchanged: every remaining Gauss-Newton step would repeat this one exactly
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
  long long rc;              // record slots of the workspace: every waveform's slots must lie inside it
};

// A waveform's samples [off, off + n) lie in the sample array and its record slots in the workspace.  Waveforms that
// break this (inconsistent offsets or lengths from the caller) are not read; the status reports CRV_ST_BOUNDS.
__device__ __forceinline__ bool wave_in_bounds(long long off, int n, long long nsamples) {
  return off >= 0 && n >= 0 && off <= nsamples && (long long)n <= nsamples - off;
}

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

// ---- FP32-mixed fit: evaluation, mapping and state in FP32, the normal-equation solve in float-float ----------------
//
// The evaluation and the solves are called, not inlined: inlined at each call site they made the round kernel large
// enough to stall on instruction fetch (1.7x faster as calls).

struct Fit3f {
  float lo[3], w[3], half[3];   // lower bound (time: relative to the window's first sample), span, half span
};

// residuals / normal equations at internal parameters u; window sample i at time i * period
static __device__ __noinline__ void eval_f32(const Fit3f& F, const float u[3], const float* yw, float period, int P,
                                         float* chi2, float H[6], float g[3]) {
  float s0, c0, s1, c1, s2, c2;
  sincosf(u[0], &s0, &c0);
  sincosf(u[1], &s1, &c1);
  sincosf(u[2], &s2, &c2);
  const float A = F.lo[0] + F.w[0] * (s0 + 1.0f) * 0.5f;
  const float mu = F.lo[1] + F.w[1] * (s1 + 1.0f) * 0.5f;
  const float b = F.lo[2] + F.w[2] * (s2 + 1.0f) * 0.5f;
  const float d0 = F.half[0] * c0, d1 = F.half[1] * c1, d2 = F.half[2] * c2;
  const float ib = 1.0f / b;
  float c = 0, h00 = 0, h01 = 0, h02 = 0, h11 = 0, h12 = 0, h22 = 0, g0 = 0, g1 = 0, g2 = 0;
  for (int i = 0; i < P; ++i) {
    const float z = (float(i) * period - mu) * ib;
    // e^-z overflows FP32 beyond 88; at 80 the Gumbel factor e^(-z - e^-z) is already exactly 0
    const float mz = fminf(-z, 80.0f);
    const float ez = __expf(mz);
    const float gg = __expf(mz - ez);
    const float f = A * gg;
    const float r = yw[i] - f;
    const float fz = f * (ez - 1.0f);
    const float j0 = gg * d0;
    const float j1 = -fz * ib * d1;
    const float j2 = -fz * z * ib * d2;
    c += r * r;
    h00 += j0 * j0; h01 += j0 * j1; h02 += j0 * j2;
    h11 += j1 * j1; h12 += j1 * j2; h22 += j2 * j2;
    g0 += j0 * r; g1 += j1 * r; g2 += j2 * r;
  }
  *chi2 = c;
  H[0] = h00; H[1] = h01; H[2] = h02; H[3] = h11; H[4] = h12; H[5] = h22;
  g[0] = g0; g[1] = g1; g[2] = g2;
}

// symmetric 3x3 solve M x = b (M packed 00 01 02 11 12 22): cofactors, determinant and adjugate product in FP64
// (products of FP32 inputs are exact there), the final division by the determinant in FP32.  The fit calls it only
// for values outside FP32's comfortable range (solve_sym_ff below does the rest).
static __device__ __noinline__ bool solve_sym64(const float M[6], const float b[3], float x[3]) {
  const double m00 = f2d(M[0]), m01 = f2d(M[1]), m02 = f2d(M[2]), m11 = f2d(M[3]), m12 = f2d(M[4]), m22 = f2d(M[5]);
  const double c00 = m11 * m22 - m12 * m12;
  const double c01 = m12 * m02 - m01 * m22;
  const double c02 = m01 * m12 - m11 * m02;
  const double det = m00 * c00 + m01 * c01 + m02 * c02;
  if (!finite_nonzero(det)) return false;
  const double c11 = m00 * m22 - m02 * m02;
  const double c12 = m01 * m02 - m00 * m12;
  const double c22 = m00 * m11 - m01 * m01;
  const double b0 = f2d(b[0]), b1 = f2d(b[1]), b2 = f2d(b[2]);
  const double y0 = c00 * b0 + c01 * b1 + c02 * b2;
  const double y1 = c01 * b0 + c11 * b1 + c12 * b2;
  const double y2 = c02 * b0 + c12 * b1 + c22 * b2;
  const float df = d2f_trunc(det);
  const float r = 1.0f / df;
  if (!(fabsf(r) < 1e30f) || !(fabsf(r) > 1e-30f)) {       // determinant outside the comfortable FP32 range
    const double rd = 1.0 / det;
    x[0] = float(y0 * rd); x[1] = float(y1 * rd); x[2] = float(y2 * rd);
    return true;
  }
  x[0] = d2f_trunc(y0) * r; x[1] = d2f_trunc(y1) * r; x[2] = d2f_trunc(y2) * r;
  return true;
}

// The same solve in float-float arithmetic on the FP32 pipe: every product of two FP32 values split exactly into a
// rounded product and its error (fmaf), sums of such pairs with their rounding errors carried (Dekker's and Knuth's
// error-free transformations), so the cofactors, the determinant and the adjugate product keep ~46 significant bits,
// reduced to the FP32 result's 24 by the final truncation, as the FP64 solve's 53 are.  Values outside FP32's
// comfortable range (or a non-finite or zero determinant) go to the FP64 solve.  Measured on the 9,358,230 pulses of
// 65,536 workload events against the FP64 solve: the same pulses, flags and clusters; the sum of pulse PE moves by
// 3e-14 relative; the fit takes 48 % less time (it was bound by the FP64 pipe: ~24 FP64 operations per solve, at
// 1/64 of the FP32 rate, against ~350 FP32 operations for a whole window evaluation).
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return FF{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return FF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FF ff_norm(float a, float b) {       // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return FF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_mul2m(float a, float b, float c, float d) {   // a*b - c*d
  const FF p = ff_two_prod(a, b), q = ff_two_prod(c, d);
  const FF s = ff_two_sum(p.hi, -q.hi);
  return ff_norm(s.hi, __fadd_rn(s.lo, __fsub_rn(p.lo, q.lo)));
}
__device__ __forceinline__ FF ff_mul(float x, FF y) {
  const FF p = ff_two_prod(x, y.hi);
  return ff_norm(p.hi, fmaf(x, y.lo, p.lo));
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const FF s = ff_two_sum(a.hi, b.hi);
  return ff_norm(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ bool ff_safe(float x) { return fabsf(x) < 1e36f; }   // finite, headroom for the sums

static __device__ __noinline__ bool solve_sym_ff(const float M[6], const float b[3], float x[3]) {
  const float m00 = M[0], m01 = M[1], m02 = M[2], m11 = M[3], m12 = M[4], m22 = M[5];
  const FF c00 = ff_mul2m(m11, m22, m12, m12);
  const FF c01 = ff_mul2m(m12, m02, m01, m22);
  const FF c02 = ff_mul2m(m01, m12, m11, m02);
  const FF det = ff_add(ff_add(ff_mul(m00, c00), ff_mul(m01, c01)), ff_mul(m02, c02));
  const FF c11 = ff_mul2m(m00, m22, m02, m02);
  const FF c12 = ff_mul2m(m01, m02, m00, m12);
  const FF c22 = ff_mul2m(m00, m11, m01, m01);
  const FF y0 = ff_add(ff_add(ff_mul(b[0], c00), ff_mul(b[1], c01)), ff_mul(b[2], c02));
  const FF y1 = ff_add(ff_add(ff_mul(b[0], c01), ff_mul(b[1], c11)), ff_mul(b[2], c12));
  const FF y2 = ff_add(ff_add(ff_mul(b[0], c02), ff_mul(b[1], c12)), ff_mul(b[2], c22));
  const float df = __fadd_rz(det.hi, det.lo);
  const float r = 1.0f / df;
  if (!(ff_safe(c00.hi) && ff_safe(c01.hi) && ff_safe(c02.hi) && ff_safe(c11.hi) && ff_safe(c12.hi) &&
        ff_safe(c22.hi) && ff_safe(det.hi) && ff_safe(y0.hi) && ff_safe(y1.hi) && ff_safe(y2.hi)) ||
      !(fabsf(df) > 1e-30f) || !(fabsf(r) < 1e30f) || !(fabsf(r) > 1e-30f))
    return solve_sym64(M, b, x);
  x[0] = __fadd_rz(y0.hi, y0.lo) * r;
  x[1] = __fadd_rz(y1.hi, y1.lo) * r;
  x[2] = __fadd_rz(y2.hi, y2.lo) * r;
  return true;
}

// Hessian check of the FP32-mixed fit: the smallest eigenvalue above 1e-12 of the matrix's scale, as H - tau I
// positive definite (Sylvester: every leading principal minor positive), tau = 1e-12 max(trace, 1e-300); the trace
// stands in for the largest eigenvalue (within a factor 3 of it for a positive semi-definite H).
__device__ __forceinline__ bool hessian_ok(const float H[6]) {
  const double h00 = f2d(H[0]), h01 = f2d(H[1]), h02 = f2d(H[2]), h11 = f2d(H[3]), h12 = f2d(H[4]), h22 = f2d(H[5]);
  const double tr = h00 + h11 + h22;
  const double tau = 1e-12 * (tr > 1e-300 ? tr : 1e-300);
  const double a = h00 - tau, d = h11 - tau, f = h22 - tau;
  const double m2 = a * d - h01 * h01;
  const double m3 = a * (d * f - h12 * h12) - h01 * (h01 * f - h12 * h02) + h02 * (h01 * h12 - d * h02);
  return a > 0.0 && m2 > 0.0 && m3 > 0.0;
}

__device__ __forceinline__ bool same3(const float a[3], const float b[3]) {
  return a[0] == b[0] && a[1] == b[1] && a[2] == b[2];
}

// the reference's schedule (40 LM steps, 8 Gauss-Newton steps with halving, EDM and Hessian checks) on FP32 state.
// Skipped work is work whose outcome is known: a step that leaves the FP32 parameters unchanged evaluates to the same
// chi2 and is rejected; a rejected step at the clamped damping, or a Gauss-Newton step that no scale improves, leaves
// the state as it was, so every later step would repeat it.  One departure, for the FP32-mixed fits only: the LM phase
// ends at the first solved step that leaves the FP32 parameters unchanged (the schedule would go on raising the
// damping, which makes the step smaller still).  Measured on the 9,358,230 pulses of 65,536 workload events: the same
// pulses, sequence numbers and flags; 10 PE values differ from the full schedule's, by at most 2.5e-7 relative (one
// FP32 rounding), one time by 1e-6 ns; the fit takes 28 % less time.
__device__ inline void fit_f32(const Fit3f& F, const float p0[3], const float* yw, float Pf, int P, int iters,
                               float u_out[3], float* chi2_out, bool* conv, bool* hok) {
  float u[3];
  for (int k = 0; k < 3; ++k) {
    float c = 2.0f * (p0[k] - F.lo[k]) / F.w[k] - 1.0f;
    u[k] = asinf(fminf(fmaxf(c, -1.0f), 1.0f));
  }
  float chi2, H[6], g[3];
  eval_f32(F, u, yw, Pf, P, &chi2, H, g);
  float lam = 1e-3f;
  for (int it = 0; it < iters; ++it) {
    float M[6] = {H[0] + lam * (H[0] + 1e-12f), H[1], H[2], H[3] + lam * (H[3] + 1e-12f), H[4],
                  H[5] + lam * (H[5] + 1e-12f)};
    float du[3];
    const bool solved = solve_sym_ff(M, g, du);
    if (!solved) du[0] = du[1] = du[2] = 0.0f;
    float un[3] = {u[0] + du[0], u[1] + du[1], u[2] + du[2]};
    bool better = false;
    if (!same3(un, u)) {
      float c2, Hn[6], gn[3];
      eval_f32(F, un, yw, Pf, P, &c2, Hn, gn);
      if (c2 < chi2) {
        better = true;
        for (int k = 0; k < 3; ++k) { u[k] = un[k]; g[k] = gn[k]; }
        for (int k = 0; k < 6; ++k) H[k] = Hn[k];
        chi2 = c2;
      }
    } else if (solved) {
      break;
    }
    const float ln = fminf(fmaxf(better ? lam * 0.3f : lam * 10.0f, 1e-9f), 1e9f);
    if (!better && ln == lam) break;
    lam = ln;
  }
  for (int it = 0; it < 8; ++it) {
    float M[6] = {H[0] + 1e-12f, H[1], H[2], H[3] + 1e-12f, H[4], H[5] + 1e-12f};
    float du[3];
    if (!solve_sym_ff(M, g, du)) break;
    for (int k = 0; k < 3; ++k)
      if (!isfinite(du[k])) du[k] = 0.0f;
    bool moved = false;
    for (int sc = 0; sc < 4 && !moved; ++sc) {
      const float s = sc == 0 ? 1.0f : (sc == 1 ? 0.5f : (sc == 2 ? 0.25f : 0.125f));
      float un[3] = {u[0] + s * du[0], u[1] + s * du[1], u[2] + s * du[2]};
      if (same3(un, u)) continue;
      float c2, Hn[6], gn[3];
      eval_f32(F, un, yw, Pf, P, &c2, Hn, gn);
      if (c2 < chi2) {
        for (int k = 0; k < 3; ++k) { u[k] = un[k]; g[k] = gn[k]; }
        for (int k = 0; k < 6; ++k) H[k] = Hn[k];
        chi2 = c2;
        moved = true;
      }
    }
    if (!moved) break;
  }
  float M[6] = {H[0] + 1e-12f, H[1], H[2], H[3] + 1e-12f, H[4], H[5] + 1e-12f};
  float st[3];
  float edm;
  bool okh;
  if (solve_sym_ff(M, g, st)) {
    edm = 0.5f * (g[0] * st[0] + g[1] * st[1] + g[2] * st[2]);
    okh = hessian_ok(H);
  } else {
    edm = INFINITY;
    okh = false;
  }
  *conv = isfinite(edm) && (edm <= 1e-3f * fmaxf(chi2, 1.0f));
  *hok = okh;
  for (int k = 0; k < 3; ++k) u_out[k] = u[k];
  *chi2_out = chi2;
}

// ---- rounds over a device task list -----------------------------------------------------------------------------
//
// A waveform's pulses are found one per round.  Round 0 (k_pf_begin) prepares every waveform and finds its first
// peak; each later launch (k_pf_round) fits one pulse of every waveform still pending, records it, subtracts it and
// searches the next peak, appending the waveform to the next round's list.  Lanes of a warp therefore run the same
// fit schedule on different waveforms instead of one lane per waveform for all its rounds.  After a fixed number of
// rounds a tail launch finishes the few waveforms left, one lane each.  Results depend only on the waveform, so the
// (atomic) order of the lists does not matter.

struct PfState {             // per waveform, carried between rounds
  double ped;
  int32_t start, cnt, ps, pe, fs, fe;
  uint8_t under, fb, near, pad[5];
};

struct PfQueue {
  PfState* st;               // [nw]
  long long* list[2];        // [nw] each: waveforms pending in even / odd rounds
  long long* counts;         // [rounds + 2]: tasks per round (zeroed before round 0)
  int rounds;                // round launches before the tail launch
  int threads;               // launch shape of the round kernels: threads per block
  int blocks_per_sm;         //   and blocks per SM (grid = min(needed, SMs x blocks_per_sm))
};

__device__ __forceinline__ void push_task(long long* list, long long* count, long long w, bool pend) {
  const unsigned m = __ballot_sync(0xffffffffu, pend);
  if (!m) return;
  const int lane = lane_id();
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(reinterpret_cast<unsigned long long*>(count), (unsigned long long)__popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (pend) list[base + __popc(m & ((1u << lane) - 1u))] = w;
}

// pedestal, sample copy, near-threshold scan and the first peak; true when a pulse is pending
template <typename R>
__device__ __forceinline__ bool pf_begin(const CrvParams& p, const WaveIn& W, double* yscr, int max_pulses,
                                         long long w, PfState& st) {
  const int n = W.n[w];
  const long long off = W.off[w];
  R* y = reinterpret_cast<R*>(yscr) + off;
  const double pdb = W.ped_db[w];
  const double x0 = n > 0 ? (W.adc16 ? double(W.adc16[off]) : double(W.adc64[off])) : 0.0;
  const bool under = (n > 0) && (pdb - x0 > p.pedestal_undershoot);
  const double ped = under ? x0 : pdb;
  if (sizeof(R) == 8) {
    for (int i = 0; i < n; ++i) y[i] = R((W.adc16 ? double(W.adc16[off + i]) : double(W.adc64[off + i])) - ped);
  } else {
    const float pf = float(ped);
    for (int i = 0; i < n; ++i) y[i] = R((W.adc16 ? float(W.adc16[off + i]) : float(W.adc64[off + i])) - pf);
  }
  st.ped = ped;
  st.under = under;
  st.start = 0;
  st.cnt = 0;
  st.fb = 0;
  st.near = near_lane<R>(y, n, 0, n - 1, R(p.min_adc_difference), R(p.knife_edge_adc));
  if (max_pulses <= 0) return false;
  return peak_lane<R>(p, y, n, 0, &st.ps, &st.pe, &st.fs, &st.fe);
}

// FP32-mixed pulse step: the fit window, bounds and fitted values relative to the window's first sample in FP32;
// FP64 for the window's absolute time and the absolute pulse times derived from it
__device__ __forceinline__ bool pf_step_f32(const CrvParams& p, const WaveIn& W, double* yscr, int max_pulses,
                                           const PulseSlots& S, long long w, PfState& st) {
  const float E = 2.718281828459045f;
  const int n = W.n[w];
  float* y = reinterpret_cast<float*>(yscr) + W.off[w];
  const long long st_tdc = W.start_tdc[w];
  const int ps = st.ps, pe = st.pe, fs = st.fs, fe = st.fe;
  const int P = fe - fs + 1;
  const float Pf = float(p.period);
  const float yps = y[ps];
  const float mtd = float(p.max_time_difference);
  Fit3f F;
  F.lo[0] = yps * E * float(p.min_height_ratio);
  F.w[0] = yps * E * float(p.max_height_ratio) - F.lo[0];
  F.lo[1] = float(ps - fs) * Pf - mtd;
  F.w[1] = float(pe - ps) * Pf + 2.0f * mtd;
  F.lo[2] = float(p.min_beta);
  F.w[2] = float(p.max_beta) - F.lo[2];
  for (int k = 0; k < 3; ++k) F.half[k] = F.w[k] * 0.5f;
  const float tpk_rel = 0.5f * float(ps + pe - 2 * fs) * Pf;      // peak time relative to the window start
  const float p0[3] = {yps * E, tpk_rel, float(p.default_beta)};
  float u[3], chi2;
  bool conv, hok;
  fit_f32(F, p0, y + fs, Pf, P, p.lm_iterations, u, &chi2, &conv, &hok);
  const int ndf = P - 3;
  bool nearlim = false;
  float par[3];
  const float tol = float(p.limit_tolerance);
  for (int k = 0; k < 3; ++k) {
    const float fr = (sinf(u[k]) + 1.0f) * 0.5f;                   // (par - lo) / span
    par[k] = F.lo[k] + F.w[k] * fr;
    if (fr < tol || 1.0f - fr < tol) nearlim = true;
  }
  const bool failed = !conv || !hok || nearlim;
  const double t0 = double(st_tdc + fs) * p.period;               // absolute time of the window's first sample
  const float A = par[0], b = par[2];
  const double mu = t0 + f2d(par[1]);
  const float height = failed ? yps : A / E;
  const float beta = failed ? float(p.default_beta) : b;
  const double tp = failed ? t0 + f2d(tpk_rel) : mu;
  const bool fseq = failed || st.fb;
  const int seq = st.cnt;
  if (seq < S.cap[w]) {
    PulseRec& r = S.rec[S.off[w] + seq];
    r.pe = f2d((failed ? yps * E * float(p.default_beta) : A * b) / d2f_trunc(W.area[w]));
    r.peph = f2d(height / d2f_trunc(W.height[w]));
    r.time = tp;
    r.height = f2d(height);
    r.beta = f2d(beta);
    r.chi2 = (failed || ndf <= 0) ? -1.0 : f2d(chi2 / float(ndf > 1 ? ndf : 1));
    r.letime = tp - p.le_time_factor * f2d(beta);
    r.ped = st.ped;
    r.A = f2d(A); r.mu = mu; r.b = f2d(b);
    r.seq = seq;
    r.failed = fseq; r.zerondf = ndf <= 0; r.pedfromdb = !st.under; r.pad = 0;
  }
  st.cnt = seq + 1;
  st.fb = fseq;
  // subtract round(fit) walking out from the mode's sample
  int im = fs + int(floorf(par[1] / Pf));
  if (im < 0) im = 0;
  if (im > n - 1) im = n - 1;
  int lo = im, hi = im;
  {
    const float mu_rel = par[1] - float(im - fs) * Pf;             // mode relative to sample im
    const float inv_b = 1.0f / b;
    for (int dir = -1; dir <= 1; dir += 2) {
      for (int i = im + (dir > 0 ? 1 : 0); i >= 0 && i < n; i += dir) {
        const float tr = float(i - im) * Pf;
        const float z = (tr - mu_rel) * inv_b;
        const float gv = A * __expf(-z - __expf(-z));
        y[i] -= round_half_away_f(gv);
        if (dir < 0) lo = i; else hi = i;
        if (fabsf(gv) < 0.25f && ((dir < 0 && tr < mu_rel) || (dir > 0 && tr > mu_rel))) break;
      }
    }
  }
  st.near = st.near || near_lane<float>(y, n, lo - 1, hi + 1, float(p.min_adc_difference), float(p.knife_edge_adc));
  st.start = fe;
  if (st.cnt >= max_pulses) return false;
  return peak_lane<float>(p, y, n, st.start, &st.ps, &st.pe, &st.fs, &st.fe);
}

// fit, record and subtract the pending pulse, then search the next one; true when another pulse is pending
template <typename R>
__device__ __forceinline__ bool pf_step(const CrvParams& p, const WaveIn& W, double* yscr, int max_pulses,
                                        const PulseSlots& S, long long w, PfState& st) {
  if constexpr (sizeof(R) == 4) {
    return pf_step_f32(p, W, yscr, max_pulses, S, w, st);
  } else {
    const double E = 2.718281828459045;
    const int n = W.n[w];
    R* y = reinterpret_cast<R*>(yscr) + W.off[w];
    const long long st_tdc = W.start_tdc[w];
    const int ps = st.ps, pe = st.pe, fs = st.fs, fe = st.fe;
    const int P = fe - fs + 1;
    const double yps = double(y[ps]);
    const double t_ps = double(st_tdc + ps) * p.period;
    const double t_pe = double(st_tdc + pe) * p.period;
    const double t_peak = 0.5 * (t_ps + t_pe);
    Fit3 F;
    F.lo[0] = yps * E * p.min_height_ratio; F.hi[0] = yps * E * p.max_height_ratio;
    F.lo[1] = t_ps - p.max_time_difference; F.hi[1] = t_pe + p.max_time_difference;
    F.lo[2] = p.min_beta; F.hi[2] = p.max_beta;
    for (int k = 0; k < 3; ++k) F.half[k] = (F.hi[k] - F.lo[k]) * 0.5;
    F.t0 = double(st_tdc + fs) * p.period;
    const double p0[3] = {yps * E, t_peak, p.default_beta};
    double par[3], chi2;
    bool conv, hok;
    fit_lane<R>(F, p0, y + fs, st_tdc + fs, p.period, P, p.lm_iterations, par, &chi2, &conv, &hok);
    const int ndf = P - 3;
    bool nearlim = false;
    for (int k = 0; k < 3; ++k) {
      const double span = F.hi[k] - F.lo[k];
      if ((par[k] - F.lo[k]) / span < p.limit_tolerance || (F.hi[k] - par[k]) / span < p.limit_tolerance)
        nearlim = true;
    }
    const bool failed = !conv || !hok || nearlim;
    const double A = par[0], mu = par[1], b = par[2];
    const double height = failed ? yps : A / E;
    const double beta = failed ? p.default_beta : b;
    const double tp = failed ? t_peak : mu;
    const bool fseq = failed || st.fb;
    const int seq = st.cnt;
    if (seq < S.cap[w]) {
      PulseRec& r = S.rec[S.off[w] + seq];
      r.pe = (failed ? yps * E * p.default_beta : A * b) / W.area[w];
      r.peph = height / W.height[w];
      r.time = tp;
      r.height = height;
      r.beta = beta;
      r.chi2 = (failed || ndf <= 0) ? -1.0 : chi2 / double(ndf > 1 ? ndf : 1);
      r.letime = tp - p.le_time_factor * beta;
      r.ped = st.ped;
      r.A = A; r.mu = mu; r.b = b;
      r.seq = seq;
      r.failed = fseq; r.zerondf = ndf <= 0; r.pedfromdb = !st.under; r.pad = 0;
    }
    st.cnt = seq + 1;
    st.fb = fseq;
    int lo, hi;
    subtract_lane<R>(p, y, n, st_tdc, A, mu, b, &lo, &hi);
    st.near = st.near || near_lane<R>(y, n, lo - 1, hi + 1, R(p.min_adc_difference), R(p.knife_edge_adc));
    st.start = fe;
    if (st.cnt >= max_pulses) return false;
    return peak_lane<R>(p, y, n, st.start, &st.ps, &st.pe, &st.fs, &st.fe);
  }
}

__device__ __forceinline__ void pf_finish(const PulseSlots& S, Status* status, long long w, const PfState& st) {
  S.count[w] = st.cnt;
  S.near[w] = st.near;
  if (st.cnt > S.cap[w]) set_flag(status, CRV_ST_LIMIT);
}

template <typename R>
__global__ void __launch_bounds__(128) k_pf_begin(CrvParams p, WaveIn W, double* __restrict__ yscr, int max_pulses,
                                                 PulseSlots S, PfQueue Q, Status* status) {
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  const long long nw = bounded_count(W.nw, W.nw_dev);
  for (long long base = (blockIdx.x * (long long)(blockDim.x >> 5) + warp_in_block()) * 32; base < nw;
       base += nwarps * 32) {
    const long long w = base + lane_id();
    bool pend = false;
    if (w < nw && !(wave_in_bounds(W.off[w], W.n[w], W.nsamples) && S.off[w] >= 0 && S.cap[w] >= 0 &&
                    S.off[w] + S.cap[w] <= S.rc)) {
      set_flag(status, CRV_ST_BOUNDS);
      S.count[w] = 0;
      S.near[w] = 0;
    } else if (w < nw) {
      PfState st;
      pend = pf_begin<R>(p, W, yscr, max_pulses, w, st);
      if (pend) Q.st[w] = st;
      else pf_finish(S, status, w, st);
    }
    push_task(Q.list[0], &Q.counts[0], w, pend);
  }
}

// round r: the tasks of list r & 1 (count counts[r]); tail != 0: finish every task in the lane
template <typename R>
__global__ void __launch_bounds__(128) k_pf_round(CrvParams p, WaveIn W, double* __restrict__ yscr, int max_pulses,
                                                 PulseSlots S, PfQueue Q, int r, int tail, Status* status) {
  const long long* in = Q.list[r & 1];
  const long long n_in = Q.counts[r];
  long long* out = Q.list[(r + 1) & 1];
  long long* n_out = &Q.counts[r + 1];
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long base = (blockIdx.x * (long long)(blockDim.x >> 5) + warp_in_block()) * 32; base < n_in;
       base += nwarps * 32) {
    const long long i = base + lane_id();
    long long w = -1;
    bool pend = false;
    if (i < n_in) {
      w = in[i];
      PfState st = Q.st[w];
      pend = pf_step<R>(p, W, yscr, max_pulses, S, w, st);
      if (tail)
        while (pend) pend = pf_step<R>(p, W, yscr, max_pulses, S, w, st);
      if (pend) Q.st[w] = st;
      else pf_finish(S, status, w, st);
    }
    if (!tail) push_task(out, n_out, w, pend);
  }
}

// One launch for every pulse of a batch.  Each lane holds one waveform and runs its rounds (fit, record, subtract,
// next peak) back to back; a lane whose waveform is finished takes the next unclaimed waveform of the batch (one
// warp-aggregated atomicAdd on a device head per refill), so lanes stay busy until every waveform has been claimed.
// Nothing waits on anything: a warp exits once the waveforms are all claimed and its own lanes are done.  A
// waveform's results depend only on the waveform, so the order of claims does not matter (same outputs as the round
// kernels).  The head is Q.counts[0], zeroed before the launch.
template <typename R>
__global__ void __launch_bounds__(128) k_pf_persist(CrvParams p, WaveIn W, double* __restrict__ yscr, int max_pulses,
                                                    PulseSlots S, PfQueue Q, Status* status) {
  const long long nw = bounded_count(W.nw, W.nw_dev);
  unsigned long long* head = reinterpret_cast<unsigned long long*>(&Q.counts[0]);
  const int lane = lane_id();
  long long w = -1;
  PfState st;
  bool pend = false;
  bool exhausted = nw <= 0;
  while (true) {
    // refill the lanes without a pending pulse (a waveform without any pulse frees its lane again at once)
    while (!exhausted) {
      const unsigned need = __ballot_sync(0xffffffffu, !pend);
      if (!need) break;
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(head, (unsigned long long)__popc(need));
      base = __shfl_sync(0xffffffffu, base, 0);
      exhausted = (long long)(base + __popc(need)) >= nw;
      if (!pend) {
        const long long c = (long long)base + __popc(need & ((1u << lane) - 1u));
        if (c < nw) {
          w = c;
          if (!(wave_in_bounds(W.off[w], W.n[w], W.nsamples) && S.off[w] >= 0 && S.cap[w] >= 0 &&
                S.off[w] + S.cap[w] <= S.rc)) {
            set_flag(status, CRV_ST_BOUNDS);
            S.count[w] = 0;
            S.near[w] = 0;
          } else {
            pend = pf_begin<R>(p, W, yscr, max_pulses, w, st);
            if (!pend) pf_finish(S, status, w, st);
          }
        }
      }
    }
    if (!__any_sync(0xffffffffu, pend)) break;
    if (pend) {
      pend = pf_step<R>(p, W, yscr, max_pulses, S, w, st);
      if (!pend) pf_finish(S, status, w, st);
    }
  }
}

}  // namespace crv
