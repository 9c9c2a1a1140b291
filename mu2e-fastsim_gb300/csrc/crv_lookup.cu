// Lookup-table photon model: the substep kernel of crvfastsim.response.photons._substep_photons
// (crv/crvfastsim/response/photons.py:139-224) over (step, SiPM) rows, with keyed draws.
//
// Built with -fmad=false (FP64 throughout): every operation rounds as written, so the CPU oracle
// (oracle/crv_oracle.c, orc_substep_photons) reproduces the photons bit for bit.
//
// Layout: a warp per row, lanes over its substeps (a 20 mm crossing has 200).  Pass 1 counts the arrivals of every
// row, an exclusive scan turns the counts into output offsets, pass 2 repeats the draws (keyed: the same numbers) and
// writes the photons in (row, substep, table, arrival) order, each lane at its offset from a warp scan.
#include <cstdint>
#include <cuda_runtime.h>

#include "crv_launch.h"
#include "crv_scan.cuh"

namespace crv {

constexpr uint32_t ST_SUBSTEP = 7;
constexpr int SUB_CALL_BINOMIAL = 0, SUB_CALL_PHOTON = 1, SUB_CALL_GAMMA = 2;
constexpr long long SUB_MAX_SUBSTEPS = 1ll << 20;
constexpr int SUB_MAX_ARRIVALS = 4096, SUB_MAX_EMISSIONS = 128;
constexpr int SUB_ROWS_PER_BLOCK = 8;                         // warps per block

// draw block of row (step, chan), table tb, call, substep k, arrival j
__device__ __forceinline__ U4 sub_block(uint32_t seed, long long step, long long chan, int tb, int call, int idx,
                                        long long k, int j) {
  uint32_t w2 = w2_of(ST_SUBSTEP, uint32_t(tb), uint32_t(idx), uint32_t(call), uint32_t(chan));
  uint32_t w3 = (uint32_t(k) << 12) | uint32_t(j);
  return philox(uint32_t(step), uint32_t((unsigned long long)step >> 32), w2, w3, seed, 0u);
}

// Binomial(n, p): inversion (Kachitvichyanukul & Schmeiser's BINV) on min(p, 1 - p) while the mean is at most 256,
// else the normal approximation rint(mean + sqrt(mean (1 - q)) z) clipped to [0, n]
__device__ __forceinline__ long long binomial(long long n, double p, const U4& w) {
  if (n <= 0 || !(p > 0.0)) return 0;
  if (p >= 1.0) return n;
  const bool flip = p > 0.5;
  const double q = flip ? 1.0 - p : p;
  const double mean = double(n) * q;
  long long k;
  if (mean > 256.0) {
    double z0, z1;
    Math<double>::normal_pair(w, &z0, &z1);
    double x = rint(mean + sqrt(mean * (1.0 - q)) * z0);
    k = x < 0.0 ? 0 : (x > double(n) ? n : (long long)x);
  } else {
    double u = u01(w.x, w.y);
    const double s = q / (1.0 - q);
    const double a = double(n + 1) * s;
    double r = dexp(double(n) * dlog(1.0 - q));
    k = 0;
    while (u > r && k < n) {
      u = u - r;
      k += 1;
      r = r * (a / double(k) - s);
    }
  }
  return flip ? n - k : k;
}

// numpy-style findBin: bin i with e[i] <= v <= e[i+1] (the lower bin on an inner edge), -1 outside
__device__ __forceinline__ int find_bin(const double* __restrict__ e, int ne, double v) {
  if (!(v >= e[0]) || !(v <= e[ne - 1])) return -1;
  if (v == e[0]) return 0;
  int lo = 0, hi = ne;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (e[mid] < v) lo = mid + 1; else hi = mid;
  }
  return lo - 1;
}

// the same bins for phi given c = cos phi and ce[j] = cos(phi edge j) (descending): phi > edge j <=> c < ce[j]
__device__ __forceinline__ int find_bin_cos(const double* __restrict__ ce, int ne, double c) {
  if (!(c <= ce[0]) || !(c >= ce[ne - 1])) return -1;
  if (c == ce[0]) return 0;
  int lo = 0, hi = ne;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (ce[mid] > c) lo = mid + 1; else hi = mid;
  }
  return lo - 1;
}

// first index j whose running sum of the uint8 weights reaches thr (the number of running sums below thr)
__device__ __forceinline__ int first_reaching(const uint8_t* __restrict__ wts, int n, double thr) {
  int cum = 0;
  for (int j = 0; j < n; ++j) {
    cum += wts[j];
    if (!(double(cum) < thr)) return j;
  }
  return n;
}

struct SubBins {
  int bin[3];
  double t, z;
};

// geometry and bins of substep k of row r (photons.py:139-196)
__device__ __forceinline__ SubBins substep_bins(const CrvLookup& L, const CrvSubstepRows& R, long long r, long long k,
                                                long long nsub, int bb, int bth) {
  const double frac = (double(k) + 0.5) / double(nsub);
  const double x = R.s[3 * r] + R.d[3 * r] * frac;
  const double y = R.s[3 * r + 1] + R.d[3 * r + 1] * frac;
  const double z = R.s[3 * r + 2] + R.d[3 * r + 2] * frac;
  const double t = R.t0[r] + (R.t1[r] - R.t0[r]) * frac;
  const double half_sep = L.fiber_separation / 2.0;
  // inside the scintillator: box, outside the elliptic fibre hole, not in a rounded corner
  const double ax = fabs(x), ay = fabs(y);
  bool insc = ax < L.half_thickness && ay < L.half_width && fabs(z) < L.half_length;
  const double ex = ax / L.hole_radius_x, ey = (ay - half_sep) / L.hole_radius_y;
  insc = insc && (ex * ex + ey * ey >= 1.0);
  const double cx = L.half_thickness - L.corner_radius, cy = L.half_width - L.corner_radius;
  if (ax > cx && ay > cy) {
    const double qx = ax - cx, qy = ay - cy;
    if (sqrt(qx * qx + qy * qy) > L.corner_radius) insc = false;
  }
  // inside a fibre: radius from the nearer fibre axis and the angle of the step direction to it
  const double y0 = y + half_sep, y1 = y - half_sep;
  const double r0 = sqrt(x * x + y0 * y0), r1 = sqrt(x * x + y1 * y1);
  const bool in0 = r0 <= L.fiber_radius, in1 = r1 <= L.fiber_radius;
  const double ry = in1 ? y1 : y0, rr = in1 ? r1 : r0;
  const double dx = R.d[3 * r], dy = R.d[3 * r + 1];
  const double norm = sqrt(dx * dx + dy * dy) * rr;
  double c = 1.0;
  if (norm > 0.0) {
    c = (dx * x + dy * ry) / norm;
    c = c < -1.0 ? -1.0 : (c > 1.0 ? 1.0 : c);
  }
  const bool infb = fabs(z) < L.half_length && (in0 || in1) && !insc;
  const int nx = L.nedges[0] - 1, ny = L.nedges[1] - 1, nz = L.nedges[2] - 1, nb = L.nedges[3] - 1;
  const int nth = L.nedges[4] - 1, nph = L.nedges[5] - 1, nr = L.nedges[6] - 1;
  (void)nx;
  const int bx = find_bin(L.edges[0], L.nedges[0], ax), by = find_bin(L.edges[1], L.nedges[1], y);
  const int bz = find_bin(L.edges[2], L.nedges[2], z);
  const bool geo = bx >= 0 && by >= 0 && bz >= 0;
  SubBins S;
  S.t = t;
  S.z = z;
  S.bin[0] = (insc && geo) ? bz + by * nz + bx * ny * nz : -1;
  S.bin[1] = (insc && geo && bb >= 0) ? bb + bz * nb + by * nz * nb + bx * ny * nz * nb : -1;
  S.bin[2] = -1;
  if (infb && bb >= 0 && bth >= 0 && bz >= 0) {
    const int bph = find_bin_cos(L.cos_phi_edges, L.nedges[5], c), br = find_bin(L.edges[6], L.nedges[6], rr);
    if (bph >= 0 && br >= 0)
      S.bin[2] = bz + br * nz + bph * nr * nz + bth * nph * nr * nz + bb * nth * nph * nr * nz;
  }
  return S;
}

__device__ __forceinline__ long long photons_per_substep(const CrvSubstepRows& R, int tb, long long r) {
  return tb == 0 ? R.n_scint[r] : (tb == 1 ? R.n_ck_s[r] : R.n_ck_f[r]);
}

// arrivals of table tb at a substep (bin >= 0)
__device__ __forceinline__ long long arrivals(const CrvLookup& L, const CrvSubstepRows& R, uint32_t seed, long long r,
                                              long long step, long long chan, long long k, int tb, int bin, double z) {
  double pr = double(L.table[tb].prob[bin]) * R.dev[r];
  if (R.mu) pr = pr * dexp(-R.mu[r] * z);
  pr = pr < 1.0 ? pr : 1.0;
  return binomial(photons_per_substep(R, tb, r), pr, sub_block(seed, step, chan, tb, SUB_CALL_BINOMIAL, 0, k, 0));
}

// arrival time of arrival j (photons.py:128-137, :214-218)
__device__ __forceinline__ double arrival_time(const CrvLookup& L, uint32_t seed, long long step, long long chan,
                                               long long k, int tb, int bin, int j, double t, Status* status) {
  const CrvLookupTable& T = L.table[tb];
  const U4 w = sub_block(seed, step, chan, tb, SUB_CALL_PHOTON, 0, k, j);
  const double thr = u01(w.x, w.y) * double(T.delay_sum[bin]);
  double tt = t + double(first_reaching(T.delays + (long long)bin * T.ndelay, T.ndelay, thr));
  if (L.fiber_decay_time > 0.0) {
    const double thr2 = u01(w.z, w.w) * double(T.emis_sum[bin]);
    const int ne = first_reaching(T.emis + (long long)bin * T.nemis, T.nemis, thr2);
    if (ne > SUB_MAX_EMISSIONS) {
      set_flag(status, CRV_ST_LIMIT);
    } else if (ne > 0) {
      double g = 0.0;
      for (int i = 0; i < ne; i += 2) {
        const U4 v = sub_block(seed, step, chan, tb, SUB_CALL_GAMMA, i >> 1, k, j);
        g = g - dlog(u01_open(v.x, v.y));
        if (i + 1 < ne) g = g - dlog(u01_open(v.z, v.w));
      }
      tt = tt + g * L.fiber_decay_time;
    }
  }
  return tt;
}

// theta bin of a row: from theta, or from cos theta against the cos of the edges
__device__ __forceinline__ int theta_bin(const CrvLookup& L, const CrvSubstepRows& R, long long r) {
  return R.theta ? find_bin(L.edges[4], L.nedges[4], R.theta[r])
                 : find_bin_cos(L.cos_theta_edges, L.nedges[4], R.cos_theta[r]);
}

__device__ __forceinline__ bool row_ok(const CrvSubstepRows& R, long long r, long long* nsub, Status* status) {
  *nsub = R.nsub[r];
  if (*nsub > SUB_MAX_SUBSTEPS) {
    set_flag(status, CRV_ST_LIMIT);
    return false;
  }
  return *nsub > 0;
}

// Rows a launch takes.  The stage entry point takes every row; the resident chain's dense rows (row 4 step + SiPM,
// every group's rows in one table) take [0, min(nrows, *nrows_dev)) of group gsel, and the seed from *seed_dev (a
// device copy of the chain's parameter-block seed, so that a captured graph of the chain follows a new seed).
struct RowSel {
  const long long* nrows_dev;
  const int8_t* group;
  const uint32_t* seed_dev;
  int gsel;
};

__device__ __forceinline__ long long sel_nrows(const RowSel& q, long long n) {
  if (!q.nrows_dev) return n;
  const long long m = *q.nrows_dev;
  return m < n ? m : n;
}
__device__ __forceinline__ bool sel_row(const RowSel& q, long long r) { return !q.group || q.group[r] == q.gsel; }
__device__ __forceinline__ uint32_t sel_seed(const RowSel& q, uint32_t seed) { return q.seed_dev ? *q.seed_dev : seed; }

__global__ void __launch_bounds__(SUB_ROWS_PER_BLOCK * 32) k_substep_count(CrvLookup L, CrvSubstepRows R,
                                                                           uint32_t seed, long long nrows, RowSel sel,
                                                                           long long* __restrict__ count,
                                                                           Status* status) {
  seed = sel_seed(sel, seed);
  nrows = sel_nrows(sel, nrows);
  const long long warps = (long long)gridDim.x * SUB_ROWS_PER_BLOCK;
  for (long long r = (long long)blockIdx.x * SUB_ROWS_PER_BLOCK + warp_in_block(); r < nrows; r += warps) {
    if (!sel_row(sel, r)) continue;                          // warp-uniform
    long long nsub;
    long long tot = 0;
    if (row_ok(R, r, &nsub, status)) {
      const long long step = R.step[r], chan = R.chan[r];
      const int bb = find_bin(L.edges[3], L.nedges[3], R.beta[r]);
      const int bth = theta_bin(L, R, r);
      for (long long k = lane_id(); k < nsub; k += 32) {
        const SubBins S = substep_bins(L, R, r, k, nsub, bb, bth);
        for (int tb = 0; tb < 3; ++tb)
          if (S.bin[tb] >= 0) {
            long long a = arrivals(L, R, seed, r, step, chan, k, tb, S.bin[tb], S.z);
            if (a >= SUB_MAX_ARRIVALS) { set_flag(status, CRV_ST_LIMIT); a = 0; }
            tot += a;
          }
      }
    }
    tot = warp_sum(tot);
    if (lane_id() == 0) count[r] = tot;
  }
}

// o_chan may be null (not written); a row whose offset is negative has no place in the output and is skipped
__global__ void __launch_bounds__(SUB_ROWS_PER_BLOCK * 32) k_substep_emit(CrvLookup L, CrvSubstepRows R, uint32_t seed,
                                                                          long long nrows, RowSel sel,
                                                                          const long long* __restrict__ offset,
                                                                          const long long* __restrict__ total,
                                                                          long long cap, int64_t* __restrict__ o_step,
                                                                          int64_t* __restrict__ o_chan,
                                                                          double* __restrict__ o_time,
                                                                          Status* status) {
  if (*total > cap) return;                                    // reported by the capacity check
  seed = sel_seed(sel, seed);
  nrows = sel_nrows(sel, nrows);
  const long long warps = (long long)gridDim.x * SUB_ROWS_PER_BLOCK;
  for (long long r = (long long)blockIdx.x * SUB_ROWS_PER_BLOCK + warp_in_block(); r < nrows; r += warps) {
    if (!sel_row(sel, r) || offset[r] < 0) continue;          // warp-uniform
    long long nsub;
    if (!row_ok(R, r, &nsub, status)) continue;               // warp-uniform
    const long long step = R.step[r], chan = R.chan[r];
    const int bb = find_bin(L.edges[3], L.nedges[3], R.beta[r]);
    const int bth = theta_bin(L, R, r);
    long long o = offset[r];
    for (long long k0 = 0; k0 < nsub; k0 += 32) {
      const long long k = k0 + lane_id();
      SubBins S;
      S.bin[0] = S.bin[1] = S.bin[2] = -1;
      S.t = 0.0;
      int a[3] = {0, 0, 0};
      if (k < nsub) {
        S = substep_bins(L, R, r, k, nsub, bb, bth);
        for (int tb = 0; tb < 3; ++tb)
          if (S.bin[tb] >= 0) {
            long long x = arrivals(L, R, seed, r, step, chan, k, tb, S.bin[tb], S.z);
            a[tb] = x >= SUB_MAX_ARRIVALS ? 0 : int(x);
          }
      }
      // arrivals spread over the lanes in (substep, table, arrival) order, as in the FP32-mixed pass
      int sum;
      const int pre = warp_excl(a[0] + a[1] + a[2], &sum);
      for (int base = 0; base < sum; base += 32) {
        const int p = base + lane_id();
        int owner = 0;
#pragma unroll
        for (int step_ = 16; step_ > 0; step_ >>= 1) {
          const int cand = owner + step_;
          const int pc = __shfl_sync(0xffffffffu, pre, cand);
          if (pc <= p) owner = cand;
        }
        const int opre = __shfl_sync(0xffffffffu, pre, owner);
        const int a0 = __shfl_sync(0xffffffffu, a[0], owner), a1 = __shfl_sync(0xffffffffu, a[1], owner);
        const int b0 = __shfl_sync(0xffffffffu, S.bin[0], owner), b1 = __shfl_sync(0xffffffffu, S.bin[1], owner);
        const int b2 = __shfl_sync(0xffffffffu, S.bin[2], owner);
        const double ot = __shfl_sync(0xffffffffu, S.t, owner);
        if (p < sum) {
          int j = p - opre, tb = 0, bn = b0;
          if (j >= a0) { j -= a0; tb = 1; bn = b1; if (j >= a1) { j -= a1; tb = 2; bn = b2; } }
          const long long q = o + p;
          o_step[q] = step;
          if (o_chan) o_chan[q] = chan;
          o_time[q] = arrival_time(L, seed, step, chan, k0 + owner, tb, bn, j, ot, status);
        }
      }
      o += sum;
    }
  }
}

// ---- FP32-mixed variant: geometry, arrival draws and delays in FP32 (24-bit uniforms), edges staged as FP32 in
// shared memory, absolute photon times FP64 (row start time + FP32 offset).  Same keyed counters as the FP64 path,
// different numbers from them; the results agree with the FP64 path statistically.

struct EdgesF {
  const float* e[7];
  const float* cphi;
  const float* cth;
  int n[7];
};

// stage the edges (and cos of the phi / theta edges) of L as FP32 in shared memory; returns the views
__device__ __forceinline__ EdgesF stage_edges_f(const CrvLookup& L, float* sm) {
  EdgesF E;
  int o = 0;
  for (int i = 0; i < 7; ++i) {
    E.n[i] = L.nedges[i];
    for (int j = threadIdx.x; j < L.nedges[i]; j += blockDim.x) sm[o + j] = float(L.edges[i][j]);
    E.e[i] = sm + o;
    o += L.nedges[i];
  }
  for (int j = threadIdx.x; j < L.nedges[5]; j += blockDim.x) sm[o + j] = float(L.cos_phi_edges[j]);
  E.cphi = sm + o;
  o += L.nedges[5];
  for (int j = threadIdx.x; j < L.nedges[4]; j += blockDim.x) sm[o + j] = L.cos_theta_edges ? float(L.cos_theta_edges[j]) : 0.f;
  E.cth = sm + o;
  __syncthreads();
  return E;
}

__device__ __forceinline__ int find_bin_f(const float* e, int ne, float v) {
  if (!(v >= e[0]) || !(v <= e[ne - 1])) return -1;
  if (v == e[0]) return 0;
  int lo = 0, hi = ne;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (e[mid] < v) lo = mid + 1; else hi = mid;
  }
  return lo - 1;
}

__device__ __forceinline__ int find_bin_cos_f(const float* ce, int ne, float c) {
  if (!(c <= ce[0]) || !(c >= ce[ne - 1])) return -1;
  if (c == ce[0]) return 0;
  int lo = 0, hi = ne;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (ce[mid] > c) lo = mid + 1; else hi = mid;
  }
  return lo - 1;
}

// 32-bit counts throughout: conversions between 64-bit integers and floats run on the FP64 pipe
__device__ __forceinline__ int binomial_f(int n, float p, const U4& w) {
  if (n <= 0 || !(p > 0.f)) return 0;
  if (p >= 1.f) return n;
  const bool flip = p > 0.5f;
  const float q = flip ? 1.f - p : p;
  const float mean = float(n) * q;
  int k;
  if (mean > 256.f) {
    float z0, z1;
    Math<float>::normal_pair(w, &z0, &z1);
    const float x = rintf(mean + sqrtf(mean * (1.f - q)) * z0);
    k = x < 0.f ? 0 : (x > float(n) ? n : int(x));
  } else {
    float u = f01(w.x);
    const float s = q / (1.f - q);
    const float a = float(n + 1) * s;
    float r = __expf(float(n) * log1pf(-q));
    k = 0;
    while (u > r && k < n) {
      u = u - r;
      k += 1;
      r = r * (a / float(k) - s);
    }
  }
  return flip ? n - k : k;
}

// a row in FP32: local start, step vector, and per-row constants
struct RowF {
  float s[3], d[3], dev, mu, dt, inv_nsub;
  double t0;
  long long step, chan;
  int nsub, bb, bth, n[3];
};

// double -> float on the integer pipe (truncating; zeros by their bits): every lane of the warp converts the same
// row values, and an FP64-pipe conversion costs a whole warp slot of GB300's FP64 pipe
__device__ __forceinline__ float to_f(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if ((b << 1) == 0ull) return __uint_as_float(uint32_t(b >> 32));
  return d2f_trunc(x);
}

__device__ __forceinline__ RowF load_row_f(const CrvSubstepRows& R, const EdgesF& E, long long r) {
  RowF w;
  for (int x = 0; x < 3; ++x) {
    w.s[x] = to_f(R.s[3 * r + x]);
    w.d[x] = to_f(R.d[3 * r + x]);
  }
  w.dev = to_f(R.dev[r]);
  w.mu = R.mu ? to_f(R.mu[r]) : 0.f;
  w.t0 = R.t0[r];
  w.dt = to_f(R.t1[r] - R.t0[r]);
  w.nsub = int(R.nsub[r]);                                     // at most 2^20 (checked by row_ok)
  w.inv_nsub = 1.f / float(w.nsub);
  w.step = R.step[r];
  w.chan = R.chan[r];
  const long long n3[3] = {R.n_scint[r], R.n_ck_s[r], R.n_ck_f[r]};
  for (int t = 0; t < 3; ++t) w.n[t] = n3[t] < 0 ? 0 : (n3[t] > 0x7FFFFFFFll ? 0x7FFFFFFF : int(n3[t]));
  w.bb = find_bin_f(E.e[3], E.n[3], to_f(R.beta[r]));
  w.bth = R.theta ? find_bin_f(E.e[4], E.n[4], to_f(R.theta[r])) : find_bin_cos_f(E.cth, E.n[4], to_f(R.cos_theta[r]));
  return w;
}

struct GeoF {
  float ht, hw, hl, half_sep, hrx, hry, fr, cr;
};

__device__ __forceinline__ GeoF geo_f(const CrvLookup& L) {
  return {float(L.half_thickness), float(L.half_width), float(L.half_length), float(L.fiber_separation / 2.0),
          float(L.hole_radius_x), float(L.hole_radius_y), float(L.fiber_radius), float(L.corner_radius)};
}

__device__ __forceinline__ void substep_bins_f(const GeoF& g, const EdgesF& E, const RowF& w, int k, int bin[3],
                                               float* z_out, float* frac_out) {
  const float frac = (float(k) + 0.5f) * w.inv_nsub;
  const float x = fmaf(w.d[0], frac, w.s[0]), y = fmaf(w.d[1], frac, w.s[1]), z = fmaf(w.d[2], frac, w.s[2]);
  const float ax = fabsf(x), ay = fabsf(y);
  bool insc = ax < g.ht && ay < g.hw && fabsf(z) < g.hl;
  const float ex = ax / g.hrx, ey = (ay - g.half_sep) / g.hry;
  insc = insc && (ex * ex + ey * ey >= 1.f);
  const float cx = g.ht - g.cr, cy = g.hw - g.cr;
  if (ax > cx && ay > cy) {
    const float qx = ax - cx, qy = ay - cy;
    if (sqrtf(qx * qx + qy * qy) > g.cr) insc = false;
  }
  const float y0 = y + g.half_sep, y1 = y - g.half_sep;
  const float r0 = sqrtf(x * x + y0 * y0), r1 = sqrtf(x * x + y1 * y1);
  const bool in0 = r0 <= g.fr, in1 = r1 <= g.fr;
  const float ry = in1 ? y1 : y0, rr = in1 ? r1 : r0;
  const float norm = sqrtf(w.d[0] * w.d[0] + w.d[1] * w.d[1]) * rr;
  float c = 1.f;
  if (norm > 0.f) c = fminf(1.f, fmaxf(-1.f, (w.d[0] * x + w.d[1] * ry) / norm));
  const bool infb = fabsf(z) < g.hl && (in0 || in1) && !insc;
  const int ny = E.n[1] - 1, nz = E.n[2] - 1, nb = E.n[3] - 1, nth = E.n[4] - 1, nph = E.n[5] - 1, nr = E.n[6] - 1;
  const int bx = find_bin_f(E.e[0], E.n[0], ax), by = find_bin_f(E.e[1], E.n[1], y), bz = find_bin_f(E.e[2], E.n[2], z);
  const bool geo = bx >= 0 && by >= 0 && bz >= 0;
  bin[0] = (insc && geo) ? bz + by * nz + bx * ny * nz : -1;
  bin[1] = (insc && geo && w.bb >= 0) ? w.bb + bz * nb + by * nz * nb + bx * ny * nz * nb : -1;
  bin[2] = -1;
  if (infb && w.bb >= 0 && w.bth >= 0 && bz >= 0) {
    const int bph = find_bin_cos_f(E.cphi, E.n[5], c), br = find_bin_f(E.e[6], E.n[6], rr);
    if (bph >= 0 && br >= 0) bin[2] = bz + br * nz + bph * nr * nz + w.bth * nph * nr * nz + w.bb * nth * nph * nr * nz;
  }
  *z_out = z;
  *frac_out = frac;
}

__device__ __forceinline__ int arrivals_f(const CrvLookup& L, const CrvSubstepRows& R, const RowF& w, uint32_t seed,
                                          int k, int tb, int bin, float z) {
  float pr = L.table[tb].prob[bin] * w.dev;
  if (R.mu) pr = pr * __expf(-w.mu * z);
  pr = fminf(pr, 1.f);
  return binomial_f(w.n[tb], pr, sub_block(seed, w.step, w.chan, tb, SUB_CALL_BINOMIAL, 0, k, 0));
}

__device__ __forceinline__ int first_reaching_f(const uint8_t* __restrict__ wts, int n, float thr) {
  int cum = 0;
  for (int j = 0; j < n; ++j) {
    cum += wts[j];
    if (!(float(cum) < thr)) return j;
  }
  return n;
}

// offset of arrival j from the row start time (FP32: substep time, delay, fibre decay)
__device__ __forceinline__ float arrival_offset_f(const CrvLookup& L, float decay, uint32_t seed, const RowF& w,
                                                  int k, int tb, int bin, int j, float frac, Status* status) {
  const CrvLookupTable& T = L.table[tb];
  const U4 v = sub_block(seed, w.step, w.chan, tb, SUB_CALL_PHOTON, 0, k, j);
  float off = w.dt * frac + float(first_reaching_f(T.delays + (long long)bin * T.ndelay, T.ndelay,
                                                   f01(v.x) * float(T.delay_sum[bin])));
  if (decay > 0.f) {
    const int ne = first_reaching_f(T.emis + (long long)bin * T.nemis, T.nemis, f01(v.z) * float(T.emis_sum[bin]));
    if (ne > SUB_MAX_EMISSIONS) {
      set_flag(status, CRV_ST_LIMIT);
    } else if (ne > 0) {
      float g = 0.f;
      for (int i = 0; i < ne; i += 2) {
        const U4 q = sub_block(seed, w.step, w.chan, tb, SUB_CALL_GAMMA, i >> 1, k, j);
        g -= __logf(f01_open(q.x));
        if (i + 1 < ne) g -= __logf(f01_open(q.z));
      }
      off += g * decay;
    }
  }
  return off;
}

__global__ void __launch_bounds__(SUB_ROWS_PER_BLOCK * 32) k_substep_count_f32(CrvLookup L, CrvSubstepRows R,
                                                                               uint32_t seed, long long nrows,
                                                                               RowSel sel,
                                                                               long long* __restrict__ count,
                                                                               Status* status) {
  extern __shared__ float edges_sm[];
  const EdgesF E = stage_edges_f(L, edges_sm);
  const GeoF g = geo_f(L);
  seed = sel_seed(sel, seed);
  nrows = sel_nrows(sel, nrows);
  const long long warps = (long long)gridDim.x * SUB_ROWS_PER_BLOCK;
  for (long long r = (long long)blockIdx.x * SUB_ROWS_PER_BLOCK + warp_in_block(); r < nrows; r += warps) {
    if (!sel_row(sel, r)) continue;                          // warp-uniform
    long long nsub;
    long long tot = 0;
    if (row_ok(R, r, &nsub, status)) {
      const RowF w = load_row_f(R, E, r);
      int sum = 0;
      for (int k = lane_id(); k < w.nsub; k += 32) {
        int bin[3];
        float z, frac;
        substep_bins_f(g, E, w, k, bin, &z, &frac);
        for (int tb = 0; tb < 3; ++tb)
          if (bin[tb] >= 0) {
            int a = arrivals_f(L, R, w, seed, k, tb, bin[tb], z);
            if (a >= SUB_MAX_ARRIVALS) { set_flag(status, CRV_ST_LIMIT); a = 0; }
            sum += a;
          }
      }
      tot = sum;
    }
    tot = warp_sum(tot);
    if (lane_id() == 0) count[r] = tot;
  }
}

__global__ void __launch_bounds__(SUB_ROWS_PER_BLOCK * 32) k_substep_emit_f32(CrvLookup L, CrvSubstepRows R,
                                                                              uint32_t seed, long long nrows,
                                                                              RowSel sel,
                                                                              const long long* __restrict__ offset,
                                                                              const long long* __restrict__ total,
                                                                              long long cap,
                                                                              int64_t* __restrict__ o_step,
                                                                              int64_t* __restrict__ o_chan,
                                                                              double* __restrict__ o_time,
                                                                              Status* status) {
  extern __shared__ float edges_sm[];
  if (*total > cap) return;                                    // block-uniform, before the staging barrier
  const EdgesF E = stage_edges_f(L, edges_sm);
  const GeoF g = geo_f(L);
  const float decay = float(L.fiber_decay_time);
  seed = sel_seed(sel, seed);
  nrows = sel_nrows(sel, nrows);
  const long long warps = (long long)gridDim.x * SUB_ROWS_PER_BLOCK;
  for (long long r = (long long)blockIdx.x * SUB_ROWS_PER_BLOCK + warp_in_block(); r < nrows; r += warps) {
    if (!sel_row(sel, r) || offset[r] < 0) continue;          // warp-uniform
    long long nsub;
    if (!row_ok(R, r, &nsub, status)) continue;
    const RowF w = load_row_f(R, E, r);
    long long o = offset[r];
    for (int k0 = 0; k0 < w.nsub; k0 += 32) {
      const int k = k0 + lane_id();
      int bin[3] = {-1, -1, -1};
      float z = 0.f, frac = 0.f;
      int a[3] = {0, 0, 0};
      if (k < w.nsub) {
        substep_bins_f(g, E, w, k, bin, &z, &frac);
        for (int tb = 0; tb < 3; ++tb)
          if (bin[tb] >= 0) {
            a[tb] = arrivals_f(L, R, w, seed, k, tb, bin[tb], z);
            if (a[tb] >= SUB_MAX_ARRIVALS) a[tb] = 0;
          }
      }
      // the chunk's arrivals in (substep, table, arrival) order, spread over the lanes: arrival p belongs to the last
      // lane whose prefix is at most p (found by a shuffle binary search), so every lane has work
      int sum;
      const int pre = warp_excl(a[0] + a[1] + a[2], &sum);
      for (int base = 0; base < sum; base += 32) {
        const int p = base + lane_id();
        int owner = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          const int cand = owner + step;
          const int pc = __shfl_sync(0xffffffffu, pre, cand);
          if (pc <= p) owner = cand;
        }
        const int opre = __shfl_sync(0xffffffffu, pre, owner);
        const int a0 = __shfl_sync(0xffffffffu, a[0], owner), a1 = __shfl_sync(0xffffffffu, a[1], owner);
        const int b0 = __shfl_sync(0xffffffffu, bin[0], owner), b1 = __shfl_sync(0xffffffffu, bin[1], owner);
        const int b2 = __shfl_sync(0xffffffffu, bin[2], owner);
        const float ofrac = __shfl_sync(0xffffffffu, frac, owner);
        if (p < sum) {
          int j = p - opre, tb = 0, bn = b0;
          if (j >= a0) { j -= a0; tb = 1; bn = b1; if (j >= a1) { j -= a1; tb = 2; bn = b2; } }
          const long long q = o + p;
          o_step[q] = w.step;
          if (o_chan) o_chan[q] = w.chan;
          o_time[q] = w.t0 + double(arrival_offset_f(L, decay, seed, w, k0 + owner, tb, bn, j, ofrac, status));
        }
      }
      o += sum;
    }
  }
}

__global__ void k_substep_check(const long long* __restrict__ total, long long cap, long long* __restrict__ n_out,
                                Status* status) {
  if (*total > cap) {
    set_flag(status, CRV_ST_CAPACITY);
    need_at_least(status, CRV_NEED_PHOTONS_OUT, *total);
  }
  *n_out = *total;
}

struct SubWs {
  long long *count, *offset, *parts, *total;
};

static SubWs sub_layout(char* base, long long n, size_t* bytes) {
  size_t off = 0;
  auto take = [&](long long cnt) {
    off = (off + 255) & ~size_t(255);
    long long* p = base ? reinterpret_cast<long long*>(base + off) : nullptr;
    off += size_t(cnt > 0 ? cnt : 1) * sizeof(long long);
    return p;
  };
  SubWs w;
  w.count = take(n);
  w.offset = take(n);
  w.parts = take(scan_parts_len(n) + 1);
  w.total = take(1);
  *bytes = off + 256;
  return w;
}

}  // namespace crv

using namespace crv;

extern "C" int64_t crv_substeps_workspace(int64_t nrows) {
  if (nrows < 0) return -1;
  size_t b = 0;
  sub_layout(nullptr, nrows, &b);
  return (int64_t)b;
}

extern "C" int crv_substep_photons(const CrvLookup* L, uint32_t seed, const CrvSubstepRows* rows, int64_t nrows,
                                   int64_t* o_step, int64_t* o_chan, double* o_time, int64_t cap, int64_t* n_out_dev,
                                   void* workspace, int64_t workspace_bytes, void* stream, CrvStatus* status_dev) {
  if (!L || !rows || !n_out_dev || !status_dev || nrows < 0 || cap < 0) return CRV_ERR_ARG;
  for (int i = 0; i < 7; ++i)
    if (!L->edges[i] || L->nedges[i] < 2) return CRV_ERR_ARG;
  if (!L->cos_phi_edges || L->precision < 0 || L->precision > 1) return CRV_ERR_ARG;
  for (int t = 0; t < 3; ++t) {
    const CrvLookupTable& T = L->table[t];
    if (!T.prob || !T.delays || !T.delay_sum || !T.emis || !T.emis_sum || T.ndelay < 1 || T.nemis < 1) return CRV_ERR_ARG;
  }
  const int nb = L->nedges[3] - 1, nx = L->nedges[0] - 1, ny = L->nedges[1] - 1, nz = L->nedges[2] - 1;
  const int nth = L->nedges[4] - 1, nph = L->nedges[5] - 1, nr = L->nedges[6] - 1;
  if ((long long)L->table[0].nbins < (long long)nx * ny * nz || (long long)L->table[1].nbins < (long long)nx * ny * nz * nb ||
      (long long)L->table[2].nbins < (long long)nb * nth * nph * nr * nz)
    return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (nrows == 0) {
    if (cudaMemsetAsync(n_out_dev, 0, sizeof(long long), s) != cudaSuccess) return CRV_ERR_CUDA;
    return CRV_OK;
  }
  if (!rows->s || !rows->d || !rows->t0 || !rows->t1 || !rows->beta || !rows->dev || !rows->nsub || !rows->step ||
      !rows->chan || !rows->n_scint || !rows->n_ck_s || !rows->n_ck_f)
    return CRV_ERR_ARG;
  if (!rows->theta && (!rows->cos_theta || !L->cos_theta_edges)) return CRV_ERR_ARG;
  size_t need = 0;
  sub_layout(nullptr, nrows, &need);
  if (!workspace || (long long)need > workspace_bytes) return CRV_ERR_ARG;
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  size_t dummy;
  SubWs w = sub_layout(base, nrows, &dummy);
  Status* S = reinterpret_cast<Status*>(status_dev);
  const long long blocks = (nrows + SUB_ROWS_PER_BLOCK - 1) / SUB_ROWS_PER_BLOCK;
  const long long maxb = (long long)device_info().sms * 8;
  const unsigned grid = (unsigned)(blocks < maxb ? blocks : maxb);
  const bool f32 = L->precision == 1;
  int nedge = 0;
  for (int i = 0; i < 7; ++i) nedge += L->nedges[i];
  const size_t esm = sizeof(float) * size_t(nedge + L->nedges[5] + L->nedges[4]);
  if (f32 && esm > 48 * 1024) return CRV_ERR_ARG;
  if (f32) {
    crv::Mark mark_("k_substep_count", s);
    k_substep_count_f32<<<grid, SUB_ROWS_PER_BLOCK * 32, esm, s>>>(*L, *rows, seed, nrows, RowSel{}, w.count, S);
  } else {
    crv::Mark mark_("k_substep_count", s);
    k_substep_count<<<grid, SUB_ROWS_PER_BLOCK * 32, 0, s>>>(*L, *rows, seed, nrows, RowSel{}, w.count, S);
  }
  if (cudaGetLastError() != cudaSuccess) return CRV_ERR_CUDA;
  if (exclusive_scan(w.count, nrows, Identity(), w.offset, w.total, w.parts, s) != cudaSuccess) return CRV_ERR_CUDA;
  {
    crv::Mark mark_("k_substep_check", s);
    k_substep_check<<<1, 1, 0, s>>>(w.total, cap, reinterpret_cast<long long*>(n_out_dev), S);
  }
  if (f32) {
    crv::Mark mark_("k_substep_emit", s);
    k_substep_emit_f32<<<grid, SUB_ROWS_PER_BLOCK * 32, esm, s>>>(*L, *rows, seed, nrows, RowSel{}, w.offset,
                                                                 w.total, cap,
                                                                 o_step, o_chan, o_time, S);
  } else {
    crv::Mark mark_("k_substep_emit", s);
    k_substep_emit<<<grid, SUB_ROWS_PER_BLOCK * 32, 0, s>>>(*L, *rows, seed, nrows, RowSel{}, w.offset, w.total,
                                                            cap, o_step,
                                                            o_chan, o_time, S);
  }
  if (cudaGetLastError() != cudaSuccess) return CRV_ERR_CUDA;
  return CRV_OK;
}

// ---- row preparation (photons.iter_rows) -----------------------------------------------------------------------------

namespace crv {

constexpr uint32_t ST_LROWS = 8;
constexpr double LROW_PRECISION_MM = 0.1;
constexpr double AMU_MEV = 931.49410242;       // atomic mass unit (CODATA 2018)

// mass [MeV] and charge [e] of a particle code: table lookup, ions 100ZZZAAAI decoded, unknown (0, 0)
__device__ __forceinline__ void particle(const CrvLookupGroup& G, long long pdg, double* m, double* q) {
  int lo = 0, hi = G.npdg;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (G.pdg_code[mid] < pdg) lo = mid + 1; else hi = mid;
  }
  if (lo < G.npdg && G.pdg_code[lo] == pdg) {
    *m = G.pdg_mass[lo];
    *q = G.pdg_charge[lo];
    return;
  }
  const long long a = pdg < 0 ? -pdg : pdg;
  if (a >= 1000000000ll) {
    *m = double((a / 10) % 1000) * AMU_MEV;
    *q = double((a / 10000) % 1000) * (pdg < 0 ? -1.0 : 1.0);
  } else {
    *m = 0.0;
    *q = 0.0;
  }
}

// Cherenkov photons per mm: linear in beta from (0, 0) through the map, flat beyond its end, times |charge|
__device__ __forceinline__ double cerenkov_per_mm(const double* __restrict__ map, int n, double beta, double q) {
  double x0 = 0.0, y0 = 0.0, v;
  int j = 0;
  while (j < n && map[2 * j] <= beta) { x0 = map[2 * j]; y0 = map[2 * j + 1]; ++j; }
  if (beta < 0.0) v = 0.0;
  else if (j == n) v = n > 0 ? map[2 * (n - 1) + 1] : 0.0;
  else v = (map[2 * j + 1] - y0) / (map[2 * j] - x0) * (beta - x0) + y0;
  return v * fabs(q);
}

// photons per substep: rint(draw / nsub) of Gauss(avg, sqrt avg) for avg > 10, else Poisson(avg) by inversion
__device__ __forceinline__ long long per_substep(double avg, long long nsub, const U4& w) {
  double x;
  if (avg > 10.0) {
    double z0, z1;
    Math<double>::normal_pair(w, &z0, &z1);
    x = avg + sqrt(avg) * z0;
  } else {
    const double lam = avg > 0.0 ? avg : 0.0;
    const double u = u01(w.x, w.y);
    double p = dexp(-lam), F = p;
    int k = 0;
    while (u >= F && k < 200) {
      k += 1;
      p = p * lam / double(k);
      F = F + p;
    }
    x = double(k);
  }
  const double n = rint(x / double(nsub));
  return n > 0.0 ? (long long)n : 0;
}

__device__ __forceinline__ bool in_lgroup(const CrvLookupGroup& G, const CrvLookupSteps& S, long long i) {
  const int b = S.bar[i];
  return b >= 0 && b < G.nbars && G.in_group[b] && isfinite(S.t0[i]) && isfinite(S.t1[i]);
}

__global__ void k_lrows_flag(CrvLookupGroup G, CrvLookupSteps S, long long n, int32_t* __restrict__ flag) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    flag[i] = in_lgroup(G, S, i) ? 1 : 0;
}

// The rows of step i (a step of group G) for each simulated SiPM: row index(si, output channel) of O
template <typename Index>
__device__ __forceinline__ void lrows_of_step(const CrvLookupGroup& G, const CrvLookupSteps& S, uint32_t seed, long long i,
                                              const CrvSubstepRowsOut& O, Index index) {
  const int nsim = G.reflector == 0 ? 4 : 2;
  const int b = S.bar[i];
  const double* c = G.center + 3 * b;
  const double ws[3] = {S.x0[i] - c[0], S.y0[i] - c[1], S.z0[i] - c[2]};
  const double we[3] = {S.x1[i] - c[0], S.y1[i] - c[1], S.z1[i] - c[2]};
  double sl[3], el[3];
  for (int k = 0; k < 3; ++k) {
    const int ax = G.l2w[3 * b + k];
    sl[k] = ws[ax];
    el[k] = we[ax];
  }
  if (G.reflector < 0) { sl[2] = -sl[2]; el[2] = -el[2]; }
  double m, q;
  particle(G, S.pdg[i], &m, &q);
  const double p0 = sqrt(S.px0[i] * S.px0[i] + S.py0[i] * S.py0[i] + S.pz0[i] * S.pz0[i]);
  const double e = 0.5 * (sqrt(p0 * p0 + m * m) + sqrt(S.p1[i] * S.p1[i] + m * m));
  double beta = 1.0;
  if (m > 0.0) {
    const double g = e / m;
    double b2 = 1.0 - 1.0 / (g * g);
    b2 = b2 < 0.0 ? 0.0 : (b2 > 1.0 ? 1.0 : b2);
    beta = sqrt(b2);
  }
  const double avg_s = G.yield[b] * S.edep[i];
  const double avg_cs = cerenkov_per_mm(G.ck_scint, G.nck_scint, beta, q) * S.len[i];
  const double avg_cf = cerenkov_per_mm(G.ck_fiber, G.nck_fiber, beta, q) * S.len[i];
  const double k = G.speed_k[b];
  for (int si = 0; si < nsim; ++si) {
    const int s = G.reflector == 0 ? si : 2 * si;
    double a[3] = {sl[0], sl[1], sl[2]}, bb[3] = {el[0], el[1], el[2]};
    if (s == 1 || s == 3) { a[2] = -a[2]; bb[2] = -bb[2]; }
    if (s == 2 || s == 3) { a[1] = -a[1]; bb[1] = -bb[1]; }
    const double d[3] = {bb[0] - a[0], bb[1] - a[1], bb[2] - a[2]};
    const double dl = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double ct = 1.0;
    if (dl > 0.0) {
      ct = d[2] / dl;
      ct = ct < -1.0 ? -1.0 : (ct > 1.0 ? 1.0 : ct);
    }
    long long nsub = (long long)(dl / LROW_PRECISION_MM);
    nsub = nsub > 1 ? nsub : 1;
    const long long chan_dev = 4ll * b + s;
    const long long chan_out = 4ll * b + (G.reflector < 0 ? s + 1 : s);
    const long long o = index(si, chan_out);
    for (int x = 0; x < 3; ++x) {
      O.s[3 * o + x] = a[x];
      O.d[3 * o + x] = d[x];
    }
    O.t0[o] = S.t0[i] + k * (a[2] + G.half_length);
    O.t1[o] = S.t1[i] + k * (bb[2] + G.half_length);
    O.nsub[o] = nsub;
    O.beta[o] = beta;
    O.cos_theta[o] = ct;
    O.dev[o] = G.dev[chan_dev];
    O.mu[o] = G.mu[b];
    O.step[o] = i;
    O.chan[o] = chan_out;
    const uint32_t lo = uint32_t(i), hi = uint32_t((unsigned long long)i >> 32);
    O.n_scint[o] = per_substep(avg_s, nsub, philox(lo, hi, w2_of(ST_LROWS, 0, 0, 0, uint32_t(chan_dev)), 0u, seed, 0u));
    O.n_ck_s[o] = per_substep(avg_cs, nsub, philox(lo, hi, w2_of(ST_LROWS, 1, 0, 0, uint32_t(chan_dev)), 0u, seed, 0u));
    O.n_ck_f[o] = per_substep(avg_cf, nsub, philox(lo, hi, w2_of(ST_LROWS, 2, 0, 0, uint32_t(chan_dev)), 0u, seed, 0u));
  }
}

__global__ void k_lrows_fill(CrvLookupGroup G, CrvLookupSteps S, uint32_t seed, long long n,
                             const long long* __restrict__ rank, const long long* __restrict__ total,
                             CrvSubstepRowsOut O) {
  const long long ng = *total;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (!in_lgroup(G, S, i)) continue;
    const long long r0 = rank[i];
    lrows_of_step(G, S, seed, i, O, [&](int si, long long) { return (long long)si * ng + r0; });
  }
}

__global__ void k_lrows_count(const long long* __restrict__ total, int nsim, long long* __restrict__ n_rows) {
  *n_rows = *total * nsim;
}

}  // namespace crv

extern "C" int64_t crv_lookup_rows_workspace(int64_t nsteps) {
  if (nsteps < 0) return -1;
  size_t off = 0;
  auto take = [&](size_t bytes) { off = ((off + 255) & ~size_t(255)) + (bytes ? bytes : 1); };
  take(sizeof(int32_t) * nsteps);
  take(sizeof(long long) * nsteps);
  take(sizeof(long long) * (scan_parts_len(nsteps) + 1));
  take(sizeof(long long));
  return (int64_t)(off + 512);
}

extern "C" int crv_lookup_rows(const CrvLookupGroup* G, uint32_t seed, const CrvLookupSteps* st, int64_t nsteps,
                               CrvSubstepRowsOut* out, int64_t cap, int64_t* n_rows_dev, void* workspace,
                               int64_t workspace_bytes, void* stream, CrvStatus* status_dev) {
  if (!G || !st || !out || !n_rows_dev || !status_dev || nsteps < 0) return CRV_ERR_ARG;
  if (G->reflector < -1 || G->reflector > 1 || G->nbars < 1 || G->npdg < 0 || G->nck_scint < 0 || G->nck_fiber < 0)
    return CRV_ERR_ARG;
  if (!G->center || !G->l2w || !G->in_group || !G->yield || !G->speed_k || !G->mu || !G->dev ||
      (G->nck_scint && !G->ck_scint) || (G->nck_fiber && !G->ck_fiber) ||
      (G->npdg && (!G->pdg_code || !G->pdg_mass || !G->pdg_charge)))
    return CRV_ERR_ARG;
  const int nsim = G->reflector == 0 ? 4 : 2;
  if (cap < nsim * nsteps) return CRV_ERR_ARG;                 // every step of the group gives nsim rows
  cudaStream_t s = (cudaStream_t)stream;
  if (nsteps == 0) return cudaMemsetAsync(n_rows_dev, 0, sizeof(long long), s) == cudaSuccess ? CRV_OK : CRV_ERR_CUDA;
  if (!st->x0 || !st->y0 || !st->z0 || !st->x1 || !st->y1 || !st->z1 || !st->px0 || !st->py0 || !st->pz0 ||
      !st->p1 || !st->t0 || !st->t1 || !st->edep || !st->len || !st->bar || !st->pdg)
    return CRV_ERR_ARG;
  if (!out->s || !out->d || !out->t0 || !out->t1 || !out->beta || !out->cos_theta || !out->dev || !out->mu ||
      !out->nsub || !out->step || !out->chan || !out->n_scint || !out->n_ck_s || !out->n_ck_f)
    return CRV_ERR_ARG;
  if (crv_lookup_rows_workspace(nsteps) > workspace_bytes || !workspace) return CRV_ERR_ARG;
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  size_t off = 0;
  auto take = [&](size_t bytes) {
    off = (off + 255) & ~size_t(255);
    char* p = base + off;
    off += bytes ? bytes : 1;
    return p;
  };
  int32_t* flag = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * nsteps));
  long long* rank = reinterpret_cast<long long*>(take(sizeof(long long) * nsteps));
  long long* parts = reinterpret_cast<long long*>(take(sizeof(long long) * (scan_parts_len(nsteps) + 1)));
  long long* total = reinterpret_cast<long long*>(take(sizeof(long long)));
  const long long blocks = (nsteps + 255) / 256, maxb = (long long)device_info().sms * 8;
  const unsigned grid = (unsigned)(blocks < maxb ? blocks : maxb);
  {
    crv::Mark mark_("k_lrows_flag", s);
    k_lrows_flag<<<grid, 256, 0, s>>>(*G, *st, nsteps, flag);
  }
  if (exclusive_scan(flag, nsteps, Identity(), rank, total, parts, s) != cudaSuccess) return CRV_ERR_CUDA;
  {
    crv::Mark mark_("k_lrows_fill", s);
    k_lrows_fill<<<grid, 256, 0, s>>>(*G, *st, seed, nsteps, rank, total, *out);
  }
  {
    crv::Mark mark_("k_lrows_count", s);
    k_lrows_count<<<1, 1, 0, s>>>(total, nsim, reinterpret_cast<long long*>(n_rows_dev));
  }
  (void)status_dev;
  return cudaGetLastError() == cudaSuccess ? CRV_OK : CRV_ERR_CUDA;
}

// ---- the lookup-table model inside the resident chain ------------------------------------------------------------
//
// Rows are dense: row 4 i + c for step i and output channel c = chan & 3, one table of rows for every group; a row of
// no group (a SiPM the group does not simulate, a step of no group or with a non-finite time) has group -1.  The
// counts and the photons then run once per group over the rows of that group (RowSel), with that group's table.

namespace crv {

struct LGroups {
  CrvLookupGroup g[CRV_LOOKUP_CHAIN_GROUPS];
  int n;
};

// rows of every step of the batch; the first thread also writes the row bound and the parameter block's seed
__global__ void k_lrows_chain(CrvParams p, LGroups K, CrvLookupSteps S, const long long* __restrict__ nsteps_dev,
                              long long step_cap, CrvSubstepRowsOut O, int8_t* __restrict__ row_group,
                              long long* __restrict__ nrows, uint32_t* __restrict__ seed_dev) {
  long long n = *nsteps_dev;
  n = n < step_cap ? (n > 0 ? n : 0) : step_cap;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *nrows = 4 * n;
    *seed_dev = p.seed;
  }
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    for (int c = 0; c < 4; ++c) row_group[4 * i + c] = -1;
    int gi = -1;
    for (int k = 0; k < K.n && gi < 0; ++k)
      if (in_lgroup(K.g[k], S, i)) gi = k;
    if (gi < 0) continue;
    lrows_of_step(K.g[gi], S, p.seed, i, O, [&](int, long long chan) {
      const long long o = 4 * i + (chan & 3);
      row_group[o] = int8_t(gi);
      return o;
    });
  }
}

// per-row counts into the chain's int32 per-(step, SiPM) counts (0 for rows of no group; a row beyond the int32
// range is reported and leaves its group, so that no pass writes its photons)
__global__ void k_lcount_narrow(const long long* __restrict__ nrows_dev, long long cap, int8_t* __restrict__ row_group,
                                const long long* __restrict__ c64, int32_t* __restrict__ c32, Status* status) {
  long long n = *nrows_dev;
  n = n < cap ? n : cap;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
    long long v = row_group[r] < 0 ? 0 : c64[r];
    if (v > 0x7FFFFFFFll) {
      set_flag(status, CRV_ST_LIMIT);
      row_group[r] = -1;
      v = 0;
    }
    c32[r] = int32_t(v);
  }
}

static CrvSubstepRows rows_in(const CrvSubstepRowsOut& o) {
  CrvSubstepRows r{};
  r.s = o.s; r.d = o.d; r.t0 = o.t0; r.t1 = o.t1; r.beta = o.beta; r.theta = nullptr; r.dev = o.dev; r.mu = o.mu;
  r.nsub = o.nsub; r.step = o.step; r.chan = o.chan; r.n_scint = o.n_scint; r.n_ck_s = o.n_ck_s; r.n_ck_f = o.n_ck_f;
  r.cos_theta = o.cos_theta;
  return r;
}

static size_t edges_smem(const CrvLookup& L) {
  int nedge = 0;
  for (int i = 0; i < 7; ++i) nedge += L.nedges[i];
  return sizeof(float) * size_t(nedge + L.nedges[5] + L.nedges[4]);
}

static unsigned step_grid(long long n) {
  const long long blocks = (n + 255) / 256;
  const long long maxb = (long long)device_info().sms * 8;
  return (unsigned)(blocks < 1 ? 1 : (blocks < maxb ? blocks : maxb));
}

static unsigned row_grid(long long nrows) {
  const long long blocks = (nrows + SUB_ROWS_PER_BLOCK - 1) / SUB_ROWS_PER_BLOCK;
  const long long maxb = (long long)device_info().sms * 8;
  return (unsigned)(blocks < 1 ? 1 : (blocks < maxb ? blocks : maxb));
}

cudaError_t lookup_chain_rows(const CrvParams& p, const CrvLookupChain& K, const long long* nsteps_dev,
                              long long step_cap, const LookupChainWs& w, cudaStream_t s) {
  LGroups G{};
  G.n = K.ngroups;
  for (int k = 0; k < K.ngroups; ++k) G.g[k] = K.group[k];
  const unsigned grid = step_grid(step_cap);
  crv::Mark mark_("k_lrows_chain", s);
  k_lrows_chain<<<grid, 256, 0, s>>>(p, G, K.steps, nsteps_dev, step_cap, w.rows, w.row_group, w.nrows, w.seed);
  return cudaGetLastError();
}

cudaError_t lookup_chain_count(const CrvLookupChain& K, const LookupChainWs& w, long long row_cap, int32_t* count32,
                               Status* status, cudaStream_t s) {
  const CrvSubstepRows R = rows_in(w.rows);
  const unsigned grid = row_grid(row_cap);
  for (int k = 0; k < K.ngroups; ++k) {
    const CrvLookup& L = K.table[k];
    if (L.precision == 1 && edges_smem(L) > 48 * 1024) return cudaErrorInvalidValue;
    const RowSel sel{w.nrows, w.row_group, w.seed, k};
    crv::Mark mark_("k_substep_count", s);
    if (L.precision == 1)
      k_substep_count_f32<<<grid, SUB_ROWS_PER_BLOCK * 32, edges_smem(L), s>>>(L, R, 0u, row_cap, sel, w.count,
                                                                              status);
    else
      k_substep_count<<<grid, SUB_ROWS_PER_BLOCK * 32, 0, s>>>(L, R, 0u, row_cap, sel, w.count, status);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  crv::Mark mark_("k_lcount_narrow", s);
  k_lcount_narrow<<<step_grid(row_cap), 256, 0, s>>>(w.nrows, row_cap, w.row_group, w.count, count32, status);
  return cudaGetLastError();
}

cudaError_t lookup_chain_emit(const CrvLookupChain& K, const LookupChainWs& w, long long row_cap,
                              const long long* total, long long cap, Status* status, cudaStream_t s) {
  const CrvSubstepRows R = rows_in(w.rows);
  const unsigned grid = row_grid(row_cap);
  for (int k = 0; k < K.ngroups; ++k) {
    const CrvLookup& L = K.table[k];
    const RowSel sel{w.nrows, w.row_group, w.seed, k};
    crv::Mark mark_("k_substep_emit", s);
    if (L.precision == 1)
      k_substep_emit_f32<<<grid, SUB_ROWS_PER_BLOCK * 32, edges_smem(L), s>>>(L, R, 0u, row_cap, sel, w.row_off,
                                                                             total, cap, w.o_step, nullptr,
                                                                             w.o_time, status);
    else
      k_substep_emit<<<grid, SUB_ROWS_PER_BLOCK * 32, 0, s>>>(L, R, 0u, row_cap, sel, w.row_off, total, cap,
                                                              w.o_step, nullptr, w.o_time, status);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace crv
