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

__device__ __forceinline__ bool row_ok(const CrvSubstepRows& R, long long r, long long* nsub, Status* status) {
  *nsub = R.nsub[r];
  if (*nsub > SUB_MAX_SUBSTEPS) {
    set_flag(status, CRV_ST_LIMIT);
    return false;
  }
  return *nsub > 0;
}

__global__ void __launch_bounds__(SUB_ROWS_PER_BLOCK * 32) k_substep_count(CrvLookup L, CrvSubstepRows R,
                                                                           uint32_t seed, long long nrows,
                                                                           long long* __restrict__ count,
                                                                           Status* status) {
  const long long warps = (long long)gridDim.x * SUB_ROWS_PER_BLOCK;
  for (long long r = (long long)blockIdx.x * SUB_ROWS_PER_BLOCK + warp_in_block(); r < nrows; r += warps) {
    long long nsub;
    long long tot = 0;
    if (row_ok(R, r, &nsub, status)) {
      const long long step = R.step[r], chan = R.chan[r];
      const int bb = find_bin(L.edges[3], L.nedges[3], R.beta[r]);
      const int bth = find_bin(L.edges[4], L.nedges[4], R.theta[r]);
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

__global__ void __launch_bounds__(SUB_ROWS_PER_BLOCK * 32) k_substep_emit(CrvLookup L, CrvSubstepRows R, uint32_t seed,
                                                                          long long nrows,
                                                                          const long long* __restrict__ offset,
                                                                          const long long* __restrict__ total,
                                                                          long long cap, int64_t* __restrict__ o_step,
                                                                          int64_t* __restrict__ o_chan,
                                                                          double* __restrict__ o_time,
                                                                          Status* status) {
  if (*total > cap) return;                                    // reported by the capacity check
  const long long warps = (long long)gridDim.x * SUB_ROWS_PER_BLOCK;
  for (long long r = (long long)blockIdx.x * SUB_ROWS_PER_BLOCK + warp_in_block(); r < nrows; r += warps) {
    long long nsub;
    if (!row_ok(R, r, &nsub, status)) continue;               // warp-uniform
    const long long step = R.step[r], chan = R.chan[r];
    const int bb = find_bin(L.edges[3], L.nedges[3], R.beta[r]);
    const int bth = find_bin(L.edges[4], L.nedges[4], R.theta[r]);
    long long o = offset[r];
    for (long long k0 = 0; k0 < nsub; k0 += 32) {
      const long long k = k0 + lane_id();
      SubBins S;
      long long a[3] = {0, 0, 0};
      if (k < nsub) {
        S = substep_bins(L, R, r, k, nsub, bb, bth);
        for (int tb = 0; tb < 3; ++tb)
          if (S.bin[tb] >= 0) {
            a[tb] = arrivals(L, R, seed, r, step, chan, k, tb, S.bin[tb], S.z);
            if (a[tb] >= SUB_MAX_ARRIVALS) a[tb] = 0;
          }
      }
      long long sum;
      long long mine = warp_excl_ll(a[0] + a[1] + a[2], &sum);
      long long q = o + mine;
      if (k < nsub)
        for (int tb = 0; tb < 3; ++tb)
          for (int j = 0; j < int(a[tb]); ++j, ++q) {
            o_step[q] = step;
            o_chan[q] = chan;
            o_time[q] = arrival_time(L, seed, step, chan, k, tb, S.bin[tb], j, S.t, status);
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
  if (!L->cos_phi_edges) return CRV_ERR_ARG;
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
  if (!rows->s || !rows->d || !rows->t0 || !rows->t1 || !rows->beta || !rows->theta || !rows->dev || !rows->nsub ||
      !rows->step || !rows->chan || !rows->n_scint || !rows->n_ck_s || !rows->n_ck_f)
    return CRV_ERR_ARG;
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
  {
    crv::Mark mark_("k_substep_count", s);
    k_substep_count<<<grid, SUB_ROWS_PER_BLOCK * 32, 0, s>>>(*L, *rows, seed, nrows, w.count, S);
  }
  if (cudaGetLastError() != cudaSuccess) return CRV_ERR_CUDA;
  if (exclusive_scan(w.count, nrows, Identity(), w.offset, w.total, w.parts, s) != cudaSuccess) return CRV_ERR_CUDA;
  {
    crv::Mark mark_("k_substep_check", s);
    k_substep_check<<<1, 1, 0, s>>>(w.total, cap, reinterpret_cast<long long*>(n_out_dev), S);
  }
  {
    crv::Mark mark_("k_substep_emit", s);
    k_substep_emit<<<grid, SUB_ROWS_PER_BLOCK * 32, 0, s>>>(*L, *rows, seed, nrows, w.offset, w.total, cap, o_step,
                                                            o_chan, o_time, S);
  }
  if (cudaGetLastError() != cudaSuccess) return CRV_ERR_CUDA;
  return CRV_OK;
}
