// Pulse reconstruction: reco waveforms -> pulses (crv/crvfastsim/reco/pulsefit.py:49-316).
//
// Per waveform: pedestal (DB value, or the first sample when it undershoots the DB value by more than the
// threshold); then rounds: FindNextPeak from `start` (rising edge, optional plateau, falling edge with the plateau
// value above min_adc_difference), a fit window of up to samples_before / samples_after monotonic samples (one dropped
// on each side when more than one was added), a bounded Gumbel least-squares fit in sine-mapped internal coordinates
// (40 Levenberg-Marquardt steps, then 8 Gauss-Newton steps with halving, EDM and Hessian checks), the failed-fit
// fallback, then the rounded fit is subtracted from every sample and the search resumes at the window end.
//
// GPU mapping: one warp per waveform; the waveform lives in shared memory; the peak search runs on lane 0; fit points
// are spread over the lanes and the normal equations are warp reductions; the 3x3 solve (LU with partial pivoting)
// and the symmetric eigenvalues (cyclic Jacobi) are FP64 on every lane.  R = double: every step in FP64; R = float
// (mixed): residuals and Jacobians in FP32 relative to the window's first sample time, normal equations accumulated
// in FP32, solve / acceptance / parameters / absolute times in FP64.
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

struct PulseOut {            // per-pulse scratch records + per-waveform counts
  PulseRec* rec;
  long long* base;           // per waveform: first record in rec
  int32_t* count;            // per waveform: pulses
  uint8_t* near;             // per waveform: wf_near_threshold
  long long* cursor;         // device record cursor
  long long cap;             // records available
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
  double t0;                 // time origin of the FP32 evaluation
};

// residuals + normal equations at internal parameters u over the P window points yw[0..P) whose times are
// (tdc_fs + i) * period (lanes split the points)
template <typename R>
__device__ __forceinline__ void evaluate(const Fit3& F, const double u[3], const double* yw, long long tdc_fs,
                                         double period, int P, double* chi2, double H[3][3], double g[3]) {
  double p[3], d[3];
  for (int k = 0; k < 3; ++k) {
    p[k] = F.lo[k] + (F.hi[k] - F.lo[k]) * (sin(u[k]) + 1.0) * 0.5;
    d[k] = F.half[k] * cos(u[k]);
  }
  R A = R(p[0]), b = R(p[2]);
  R mu = sizeof(R) == 8 ? R(p[1]) : R(p[1] - F.t0);
  R s_c = 0, s00 = 0, s01 = 0, s02 = 0, s11 = 0, s12 = 0, s22 = 0, s0 = 0, s1 = 0, s2 = 0;
  for (int i = lane_id(); i < P; i += 32) {
    R t = sizeof(R) == 8 ? R(double(tdc_fs + i) * period) : R(double(i) * period);
    R z = (t - mu) / b;
    R ez = sizeof(R) == 8 ? R(exp(double(-z))) : R(__expf(float(-z)));
    R gg = sizeof(R) == 8 ? R(exp(double(-z - ez))) : R(__expf(float(-z - ez)));
    R f = A * gg;
    R r = R(yw[i]) - f;
    R fz = f * (ez - R(1));
    R j0 = gg * R(d[0]);
    R j1 = fz * (R(-1) / b) * R(d[1]);
    R j2 = fz * (-z / b) * R(d[2]);
    s_c += r * r;
    s00 += j0 * j0; s01 += j0 * j1; s02 += j0 * j2;
    s11 += j1 * j1; s12 += j1 * j2; s22 += j2 * j2;
    s0 += j0 * r; s1 += j1 * r; s2 += j2 * r;
  }
  double v[10] = {double(s_c), double(s00), double(s01), double(s02), double(s11), double(s12), double(s22),
                  double(s0), double(s1), double(s2)};
#pragma unroll
  for (int k = 0; k < 10; ++k) v[k] = warp_sum(v[k]);
  *chi2 = v[0];
  H[0][0] = v[1]; H[0][1] = H[1][0] = v[2]; H[0][2] = H[2][0] = v[3];
  H[1][1] = v[4]; H[1][2] = H[2][1] = v[5]; H[2][2] = v[6];
  g[0] = v[7]; g[1] = v[8]; g[2] = v[9];
}

// bounded Gumbel fit; returns params, chi2, converged, hessian_ok
template <typename R>
__device__ void fit_gumbel(const Fit3& F, const double p0[3], const double* yw, long long tdc_fs, double period, int P,
                           int iters, double par[3], double* chi2_out, bool* conv, bool* hok) {
  double u[3];
  for (int k = 0; k < 3; ++k) {
    double c = 2.0 * (p0[k] - F.lo[k]) / (F.hi[k] - F.lo[k]) - 1.0;
    c = fmin(fmax(c, -1.0), 1.0);
    u[k] = asin(c);
  }
  double chi2, H[3][3], g[3];
  evaluate<R>(F, u, yw, tdc_fs, period, P, &chi2, H, g);
  double lam = 1e-3;
  for (int it = 0; it < iters; ++it) {
    double Aug[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Aug[i][j] = H[i][j];
    for (int i = 0; i < 3; ++i) Aug[i][i] = H[i][i] + lam * (H[i][i] + 1e-12);
    double du[3];
    if (!solve3(Aug, g, du)) du[0] = du[1] = du[2] = 0.0;
    double un[3] = {u[0] + du[0], u[1] + du[1], u[2] + du[2]};
    double c2, Hn[3][3], gn[3];
    evaluate<R>(F, un, yw, tdc_fs, period, P, &c2, Hn, gn);
    bool better = c2 < chi2;
    if (better) {
      for (int k = 0; k < 3; ++k) { u[k] = un[k]; g[k] = gn[k]; }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H[i][j] = Hn[i][j];
      chi2 = c2;
    }
    lam = better ? lam * 0.3 : lam * 10.0;
    lam = fmin(fmax(lam, 1e-9), 1e9);
  }
  for (int it = 0; it < 8; ++it) {
    double M[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) M[i][j] = H[i][j] + (i == j ? 1e-12 : 0.0);
    double du[3];
    if (!solve3(M, g, du)) break;
    for (int k = 0; k < 3; ++k)
      if (!isfinite(du[k])) du[k] = 0.0;
    for (int sc = 0; sc < 4; ++sc) {
      double s = sc == 0 ? 1.0 : (sc == 1 ? 0.5 : (sc == 2 ? 0.25 : 0.125));
      double un[3] = {u[0] + s * du[0], u[1] + s * du[1], u[2] + s * du[2]};
      double c2, Hn[3][3], gn[3];
      evaluate<R>(F, un, yw, tdc_fs, period, P, &c2, Hn, gn);
      if (c2 < chi2) {
        for (int k = 0; k < 3; ++k) { u[k] = un[k]; g[k] = gn[k]; }
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) H[i][j] = Hn[i][j];
        chi2 = c2;
        break;                 // the accepted step zeroes du: later scales re-evaluate the same point
      }
    }
  }
  double M[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M[i][j] = H[i][j] + (i == j ? 1e-12 : 0.0);
  double st[3];
  double edm;
  bool okh;
  if (solve3(M, g, st)) {
    edm = 0.5 * (g[0] * st[0] + g[1] * st[1] + g[2] * st[2]);
    double e[3];
    eig3(H, e);
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

// near-threshold local maximum among samples [a, b] (inclusive range of candidate positions)
__device__ __forceinline__ bool near_threshold_any(const double* y, int n, int a, int b, double thr, double edge) {
  bool any = false;
  if (a < 0) a = 0;
  if (b > n - 1) b = n - 1;
  for (int base = a; base <= b; base += 32) {
    int i = base + lane_id();
    bool hit = false;
    if (i <= b) {
      double left = i > 0 ? y[i - 1] : -1e9;
      double right = i + 1 < n ? y[i + 1] : -1e9;
      hit = (y[i] >= left) && (y[i] > right) && (fabs(y[i] - thr) <= edge);
    }
    any |= __any_sync(0xffffffffu, hit);
  }
  return any;
}

// FindNextPeak (lane 0) + fit window; results broadcast to the warp
__device__ __forceinline__ bool next_peak(const CrvParams& p, const double* y, int n, int start, int* ps_o, int* pe_o,
                                          int* fs_o, int* fe_o) {
  int found = 0, ps = 0, pe = 0, fs = 0, fe = 0;
  if (lane_id() == 0) {
    bool rising = false;
    for (int b = (start + 1 > 1 ? start + 1 : 1); b < n; ++b) {
      double prev = y[b - 1], cur = y[b];
      if (prev < cur) { rising = true; ps = b; pe = b; }
      else if (prev == cur) { if (rising) pe = b; }
      else if (rising) {
        if (y[pe] > p.min_adc_difference) { found = 1; break; }
        rising = false;
      }
    }
    if (found) {
      fs = ps - 1;
      fe = pe + 1;
      for (int k = 1; k <= p.samples_before; ++k) {
        int i = ps - k;
        if (i < 0) break;
        if (!(y[i] <= y[i + 1])) break;
        fs = i;
        if (i == 0) break;
      }
      for (int k = 1; k <= p.samples_after; ++k) {
        int i = pe + k;
        if (i >= n) break;
        if (!(y[i - 1] >= y[i])) break;
        fe = i;
      }
      if (ps - fs > 1) fs += 1;
      if (fe - pe > 1) fe -= 1;
    }
  }
  found = __shfl_sync(0xffffffffu, found, 0);
  *ps_o = __shfl_sync(0xffffffffu, ps, 0);
  *pe_o = __shfl_sync(0xffffffffu, pe, 0);
  *fs_o = __shfl_sync(0xffffffffu, fs, 0);
  *fe_o = __shfl_sync(0xffffffffu, fe, 0);
  return found != 0;
}

constexpr int PF_WARPS = 8;

__host__ __device__ inline size_t pulsefit_smem_per_warp(int cap, int pcap) {
  return size_t(cap) * 8 + size_t(pcap) * sizeof(PulseRec);
}

// second_pass == 0: every waveform with n <= cap whose pulses fit pcap records; others are deferred.
// second_pass == 1: only deferred waveforms; what still does not fit is reported (CRV_ST_CAPACITY).
template <typename R>
__global__ void __launch_bounds__(PF_WARPS * 32) k_pulsefit(CrvParams p, WaveIn W, int cap, int pcap, int second_pass,
                                                          int max_pulses, PulseOut O, int32_t* __restrict__ deferred,
                                                          Status* status) {
  extern __shared__ __align__(16) char smem[];
  char* base = smem + size_t(warp_in_block()) * pulsefit_smem_per_warp(cap, pcap);
  double* y = reinterpret_cast<double*>(base);
  PulseRec* rec = reinterpret_cast<PulseRec*>(base + size_t(cap) * 8);
  const double E = 2.718281828459045;
  long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long w = blockIdx.x * (long long)(blockDim.x >> 5) + warp_in_block(); w < W.nw; w += warps) {
    if (second_pass && !deferred[w]) continue;
    int n = W.n[w];
    if (n > cap) {
      if (lane_id() == 0) {
        if (second_pass) {
          set_flag(status, CRV_ST_CAPACITY);
          need_at_least(status, CRV_NEED_SAMPLES, n);
          O.count[w] = 0;
        } else {
          deferred[w] = 1;
        }
      }
      continue;
    }
    long long off = W.off[w];
    double pdb = W.ped_db[w];
    double x0 = n > 0 ? (W.adc16 ? double(W.adc16[off]) : double(W.adc64[off])) : 0.0;
    bool under = (n > 0) && (pdb - x0 > p.pedestal_undershoot);
    double ped = under ? x0 : pdb;
    for (int i = lane_id(); i < n; i += 32) {
      double a = W.adc16 ? double(W.adc16[off + i]) : double(W.adc64[off + i]);
      y[i] = a - ped;
    }
    __syncwarp();
    bool near = near_threshold_any(y, n, 0, n - 1, p.min_adc_difference, p.knife_edge_adc);
    long long st_tdc = W.start_tdc[w];
    int start = 0, npulse = 0;
    bool failed_before = false;
    for (int seq = 0; seq < max_pulses; ++seq) {
      int ps, pe, fs, fe;
      if (!next_peak(p, y, n, start, &ps, &pe, &fs, &fe)) break;
      int P = fe - fs + 1;
      double yps = y[ps];
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
      fit_gumbel<R>(F, p0, y + fs, st_tdc + fs, p.period, P, p.lm_iterations, par, &chi2, &conv, &hok);
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
      if (lane_id() == 0 && npulse < pcap) {
        PulseRec& r = rec[npulse];
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
      ++npulse;
      failed_before = fseq;
      for (int i = lane_id(); i < n; i += 32) {
        double t = double(st_tdc + i) * p.period;
        double z = (t - mu) / b;
        double gv = A * exp(-z - exp(-z));
        y[i] -= round_half_away(gv);
      }
      __syncwarp();
      near = near_threshold_any(y, n, 0, n - 1, p.min_adc_difference, p.knife_edge_adc) || near;
      start = fe;
    }
    if (npulse > pcap) {
      if (lane_id() == 0) {
        if (second_pass) {
          set_flag(status, CRV_ST_CAPACITY);
          need_at_least(status, CRV_NEED_PULSES, npulse);
          O.count[w] = 0;
        } else {
          deferred[w] = 1;
        }
      }
      __syncwarp();
      continue;
    }
    long long bse = 0;
    if (lane_id() == 0) bse = (long long)atomicAdd(reinterpret_cast<unsigned long long*>(O.cursor),
                                                  (unsigned long long)npulse);
    bse = __shfl_sync(0xffffffffu, bse, 0);
    if (bse + npulse > O.cap) {
      if (lane_id() == 0) {
        set_flag(status, CRV_ST_CAPACITY);
        need_at_least(status, CRV_NEED_PULSES_OUT, bse + npulse);
        O.count[w] = 0;
        O.near[w] = near;
        if (second_pass) deferred[w] = 0;
      }
      continue;
    }
    for (int k = lane_id(); k < npulse; k += 32) O.rec[bse + k] = rec[k];
    if (lane_id() == 0) {
      O.base[w] = bse;
      O.count[w] = npulse;
      O.near[w] = near;
      if (second_pass) deferred[w] = 0;
    }
    __syncwarp();
  }
}

}  // namespace crv
