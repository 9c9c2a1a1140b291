// Waveform stage: SiPM charges -> zero-suppressed 12-sample digis.
//
// Semantics of the reference synthesis (crv/crvfastsim/reco/waveform.py:65-172, chain.py:219-270):
//   * TDC0 per (event, FEB): one uniform x width (keyed by event and FEB key, so no global order is needed);
//   * charges of a SiPM split into clusters where consecutive times differ by more than max_time + 4 periods; a
//     cluster is kept if n_charges * max(template) >= min_voltage;
//   * the cluster waveform starts at t_start = ceil((t_first - P - TDC0) / P) P + TDC0 and is
//     max(floor((t_last - t_first + max_time) / P), last reached sample + 1) samples long;
//   * every charge adds template[rint((J P + t_start - t) / precision)] * charge / q_ref to samples J >= ceil((t -
//     t_start)/P) within ceil(max_time/P) + 2 samples; electronics noise sigma * z(event, channel, tick) is added to
//     every sample (keyed normals);
//   * zero suppression: a digi starts at sample i if a sample in i-2..i+2 exceeds min_voltage, i >= the end of the
//     previous digi and t_start + i P lies in the window; ADC = clip(int16(V * conv + pedestal + 0.5), min, max);
//     startTDC = rint((start - TDC0) / P).
//
// GPU mapping: one warp per SiPM; the cluster waveform is a shared-memory tile (lanes own samples); each sample sums
// the charges that reach it in charge order (a contiguous range found by binary search), so FP64 sums round exactly
// as the reference's scatter-add; the zero-suppression scan proceeds 32 samples per ballot.
#pragma once
#include "crv_device.cuh"

namespace crv {

struct WfGroups {
  const long long* n;            // device: number of SiPM groups
  const long long* start;        // first charge row of the group
  const int32_t* count;          // charges in the group
  const long long* label;        // SiPM label
  const uint32_t* run;           // run per group (keys), may be null (run 0)
};

struct DigiSlots {
  const long long* off;          // first slot of the group
  const int32_t* cap;            // slots of the group
  int32_t* n;                    // digis written
  long long* chan;
  double* start;
  double* tdc0;
  long long* starttdc;
  double* volt;                  // [slots, 12]; null: volts not kept
  int16_t* adc;                  // [slots, 12]
};

__device__ __forceinline__ int32_t feb_key(const CrvParams& p, const CrvChannels& ch, int c) {
  return p.feb_key_mode == 1 ? ch.feb[c] : ch.roc[c] * 1000 + ch.feb[c];
}

__device__ __forceinline__ double tdc0_of(const CrvParams& p, const CrvChannels& ch, long long label, uint32_t run) {
  long long evk = label / 32768;
  int c = int(label % 32768);
  EvKey ek{uint32_t(evk & 0xFFFFF), uint32_t(evk >> 20), run};
  U4 w = keyed(p.seed, ek, ST_TDC0 << 28, uint32_t(feb_key(p, ch, c)));
  return u01(w.x, w.y) * p.feb_phase_width;
}

__device__ __forceinline__ int reach_samples(const CrvParams& p) { return int(ceil(p.spe_max_time / p.period)) + 2; }

// first sample a charge at time t reaches in a cluster starting at ts
template <typename R>
__device__ __forceinline__ long long first_sample(const CrvParams& p, double t, double ts) {
  if (sizeof(R) == 8) {
    double v = ceil((t - ts) / p.period);
    return v > 0.0 ? (long long)v : 0;
  }
  float v = ceilf(float(t - ts) / float(p.period));
  return v > 0.0f ? (long long)v : 0;
}

// x / d, exactly: a multiplication by 1/d when d is a power of two (the quotient rounds identically), else a division
__device__ __forceinline__ double exact_div(double x, double d) {
  int e;
  double m = frexp(d, &e);
  return m == 0.5 ? x * ldexp(1.0, 1 - e) : x / d;
}

// template index of sample J for a charge at t (returns -1 when the pair does not contribute)
template <typename R>
__device__ __forceinline__ int tmpl_index(const CrvParams& p, long long J, double t, double ts, int tlen) {
  if (sizeof(R) == 8) {
    double st = double(J) * p.period + ts - t;
    if (!(st >= 0.0)) return -1;
    double ti = rint(exact_div(st, p.spe_precision));
    return ti < double(tlen) ? int(ti) : -1;
  }
  float st = float(J) * float(p.period) - float(t - ts);
  if (!(st >= 0.0f)) return -1;
  float ti = rintf(st / float(p.spe_precision));
  return ti < float(tlen) ? int(ti) : -1;
}

// FP32-mixed forms on dt = t - t_start (one FP64 subtraction per charge, then FP32)
__device__ __forceinline__ int first_sample_f(float dt, float P) {
  float v = ceilf(dt / P);
  return v > 0.0f ? int(v) : 0;
}

__device__ __forceinline__ int tmpl_index_f(int J, float dt, float P, float inv_prec, int tlen) {
  float st = float(J) * P - dt;
  if (!(st >= 0.0f)) return -1;
  float ti = rintf(st * inv_prec);
  return ti < float(tlen) ? int(ti) : -1;
}

// A kept cluster, computed once per cluster by the prepass (one thread per SiPM): t_start = k0 P + TDC0, charge rows
// [a, b) relative to the group start, length in samples, and the samples whose start lies in the window [ilo, ihi]
// (valid while the length fits a synthesis pass, at most 16,384 samples).
struct WfCluster {
  double ts;
  long long k0;
  int32_t a, b, L;
  int16_t ilo, ihi;
};

// t_start of a cluster, rounded the same way wherever it is formed (no contraction into an FMA)
__device__ __forceinline__ double cluster_ts(long long k0, double period, double tdc0) {
  return __dadd_rn(__dmul_rn(double(k0), period), tdc0);
}

// samples of a cluster whose start lies in the window: [i_lo, i_hi] (monotone predicates)
__device__ __forceinline__ void window_bounds(const CrvParams& p, double ts, int L, int* lo_o, int* hi_o) {
  if (ts >= p.window_lo && __dadd_rn(ts, __dmul_rn(double(L - 1), p.period)) <= p.window_hi) {
    *lo_o = 0;
    *hi_o = L - 1;
    return;
  }
  double a0 = ceil((p.window_lo - ts) / p.period);
  long long c = (long long)fmax(a0 - 1.0, 0.0);
  while (c < L && !(__dadd_rn(ts, __dmul_rn(double(c), p.period)) >= p.window_lo)) ++c;
  while (c > 0 && __dadd_rn(ts, __dmul_rn(double(c - 1), p.period)) >= p.window_lo) --c;
  double b0 = floor((p.window_hi - ts) / p.period);
  long long d = (long long)fmin(b0 + 1.0, double(L - 1));
  while (d >= 0 && !(__dadd_rn(ts, __dmul_rn(double(d), p.period)) <= p.window_hi)) --d;
  while (d + 1 < L && __dadd_rn(ts, __dmul_rn(double(d + 1), p.period)) <= p.window_hi) ++d;
  *lo_o = int(c);
  *hi_o = int(d);
}

// cluster_length for one thread (charges a..b-1 in turn); nr = reach_samples(p), ip = 1 / template precision
template <typename R>
__device__ __forceinline__ int cluster_length_serial(const CrvParams& p, const double* t, int a, int b, double ts,
                                                     int tlen, int nr, float ip) {
  long long est = (long long)floor((t[b - 1] - t[a] + p.spe_max_time) / p.period);
  long long used = 0;
  const float Pf = float(p.period);
  for (int q = a; q < b; ++q) {
    if (sizeof(R) == 8) {
      long long j0 = first_sample<R>(p, t[q], ts);
      for (int k = nr - 1; k >= 0; --k) {
        if (tmpl_index<R>(p, j0 + k, t[q], ts, tlen) >= 0) {
          if (j0 + k + 1 > used) used = j0 + k + 1;
          break;
        }
      }
    } else {
      float dt = float(t[q] - ts);
      int j0 = first_sample_f(dt, Pf);
      for (int k = nr - 1; k >= 0; --k) {
        if (tmpl_index_f(j0 + k, dt, Pf, ip, tlen) >= 0) {
          if (j0 + k + 1 > used) used = j0 + k + 1;
          break;
        }
      }
    }
  }
  return int(est > used ? est : used);
}

// Per group, one thread each (the per-cluster FP64 scalars are then computed once per cluster, not by a whole
// warp): TDC0, the kept clusters (into cl[group start + k]), the digi bound (sum over kept clusters of
// ceil(length / samples_zs)) and the longest kept cluster.
template <typename R>
__global__ void __launch_bounds__(256) k_wf_prepass(CrvParams p, CrvChannels ch, WfGroups G,
                                                    const double* __restrict__ time, const double* __restrict__ tmpl,
                                                    int tlen, const double* __restrict__ tdc0_rows,
                                                    double* __restrict__ g_tdc0, int32_t* __restrict__ g_bound,
                                                    int32_t* __restrict__ g_maxlen, int32_t* __restrict__ g_nkept,
                                                    WfCluster* __restrict__ cl) {
  __shared__ double vmax_s;
  if (threadIdx.x < 32) {
    double v = -1e300;
    for (int i = threadIdx.x; i < tlen; i += 32) v = fmax(v, tmpl[i]);
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) vmax_s = v;
  }
  __syncthreads();
  const double vmax = vmax_s;
  const double gap = p.spe_max_time + 4.0 * p.period;
  const int nr = reach_samples(p);
  const float ip = float(1.0 / p.spe_precision);
  const int zs = p.samples_zs;
  const long long ng = *G.n;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x) {
    const int n = G.count[g];
    const long long q0 = G.start[g];
    const double* t = time + q0;
    // keyed TDC0 of the group, unless the caller gives one per cluster (then the channel tables are not read)
    const double tdc0 = tdc0_rows ? 0.0 : tdc0_of(p, ch, G.label[g], G.run ? G.run[g] : 0u);
    long long bound = 0;
    int maxlen = 0, nk = 0;
    for (int a = 0; a < n;) {
      int b = a + 1;
      while (b < n && !(t[b] - t[b - 1] > gap)) ++b;
      if (double(b - a) * vmax >= p.min_voltage) {
        const double tdc0c = tdc0_rows ? tdc0_rows[q0 + a] : tdc0;
        const long long k0 = (long long)ceil((t[a] - p.period - tdc0c) / p.period);
        const double ts = cluster_ts(k0, p.period, tdc0c);
        const int L = cluster_length_serial<R>(p, t, a, b, ts, tlen, nr, ip);
        bound += (L + zs - 1) / zs;
        maxlen = L > maxlen ? L : maxlen;
        int ilo = 0, ihi = -1;
        if (L <= 16384) window_bounds(p, ts, L, &ilo, &ihi);
        cl[q0 + nk] = WfCluster{ts, k0, a, b, L, int16_t(ilo), int16_t(ihi)};
        ++nk;
      }
      a = b;
    }
    g_tdc0[g] = tdc0;
    g_bound[g] = int32_t(bound);
    g_maxlen[g] = maxlen;
    g_nkept[g] = nk;
  }
}


constexpr int WF_QSTAGE = 512;    // charges of a cluster staged in shared memory (larger clusters: on the fly)

template <typename R>
__host__ __device__ inline size_t wf_smem_per_warp(int cap) {
  return (size_t(cap) * sizeof(R) + size_t(WF_QSTAGE) * (sizeof(R) + 8) + 15) & ~size_t(15);
}

__device__ __forceinline__ int16_t adc_of(const CrvParams& p, double v) {
  double x = v * p.adc_conversion + double(p.adc_pedestal) + 0.5;
  long long i;
  if (!(x == x)) i = (long long)-2147483648ll;
  else if (x >= 2147483647.0) i = 2147483647ll;
  else if (x <= -2147483648.0) i = -2147483648ll;
  else i = (long long)trunc(x);
  int16_t s = int16_t(uint16_t(uint32_t(int32_t(i)) & 0xFFFFu));
  int r = s;
  if (r < p.min_adc) r = p.min_adc;
  if (r > p.max_adc) r = p.max_adc;
  return int16_t(r);
}

// ADC of an FP32 sample: v * conversion + pedestal + 0.5 is exact in FP64 for an FP32 v (a 24-bit by 12-bit
// product plus a small offset), so one FP32 FMA (one rounding) truncates to the same integer unless it lands on an
// integer itself; only then, or out of range, is the FP64 form evaluated.
__device__ __forceinline__ int16_t adc_of_f(const CrvParams& p, float v, float conv, float off) {
  const float x = fmaf(v, conv, off);
  if (!(fabsf(x) < 1e9f) || x == truncf(x)) return adc_of(p, f2d(v));
  int r = int16_t(uint16_t(uint32_t(int32_t(truncf(x))) & 0xFFFFu));
  if (r < p.min_adc) r = p.min_adc;
  if (r > p.max_adc) r = p.max_adc;
  return int16_t(r);
}

// Synthesis + zero suppression of the groups whose longest kept cluster is in (lo, cap].
template <typename R>
__global__ void __launch_bounds__(256, 3) k_wf_synth(CrvParams p, WfGroups G, const double* __restrict__ time,
                                                  const double* __restrict__ charge, const double* __restrict__ tmpl,
                                                  int tlen, const double* __restrict__ tdc0_rows,
                                                  const double* __restrict__ g_tdc0,
                                                  const int32_t* __restrict__ g_maxlen,
                                                  const int32_t* __restrict__ g_nkept,
                                                  const WfCluster* __restrict__ cl, int lo, int cap, int last_pass,
                                                  DigiSlots D, Status* status) {
  extern __shared__ __align__(16) char smem[];
  char* wbase = smem + size_t(warp_in_block()) * wf_smem_per_warp<R>(cap);
  R* wave = reinterpret_cast<R*>(wbase);
  R* qn_s = reinterpret_cast<R*>(wbase + size_t(cap) * sizeof(R));
  int32_t* j0_s = reinterpret_cast<int32_t*>(wbase + size_t(cap) * sizeof(R) + size_t(WF_QSTAGE) * sizeof(R));
  float* dt_s = reinterpret_cast<float*>(wbase + size_t(cap) * sizeof(R) + size_t(WF_QSTAGE) * (sizeof(R) + 4));
  __shared__ float tmpl_f[1024];
  if (sizeof(R) == 4)
    for (int i = threadIdx.x; i < tlen && i < 1024; i += blockDim.x) tmpl_f[i] = float(tmpl[i]);
  __syncthreads();
  const int nr = reach_samples(p);
  const int zs = p.samples_zs;
  const float Pf = float(p.period), ip = float(1.0 / p.spe_precision);
  const R inv_q = R(1.0 / p.spe_ref_charge);
  const R vthr = R(p.min_voltage);
  const R sigma = R(p.noise_sigma);
  const float conv_f = float(p.adc_conversion), off_f = float(double(p.adc_pedestal) + 0.5);
  long long ng = *G.n;
  long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long g = blockIdx.x * (long long)(blockDim.x >> 5) + warp_in_block(); g < ng; g += warps) {
    int ml = g_maxlen[g];
    if (ml <= lo) continue;
    if (ml > cap) {
      if (last_pass && lane_id() == 0) {
        set_flag(status, CRV_ST_CAPACITY);
        need_at_least(status, CRV_NEED_SAMPLES, ml);
      }
      continue;
    }
    long long q0 = G.start[g];
    const double* t = time + q0;
    const double* qc = charge + q0;
    long long lab = G.label[g];
    uint32_t run = G.run ? G.run[g] : 0u;
    long long evk = lab / 32768;
    EvKey ek{uint32_t(evk & 0xFFFFF), uint32_t(evk >> 20), run};
    uint32_t chan = uint32_t(lab % 32768);
    double tdc0 = g_tdc0[g];
    long long slot = D.off[g];
    int scap = D.cap[g];
    int nd = 0;
    const int nk = g_nkept[g];
    for (int kc = 0; kc < nk; ++kc) {
      const WfCluster C = cl[q0 + kc];
      const int a = C.a, b = C.b, L = C.L;
      const long long k0 = C.k0;
      const double ts = C.ts;
      const double tdc0c = tdc0_rows ? tdc0_rows[q0 + a] : tdc0;
      // stage each charge's first reached sample and normalised charge (once per charge, not per sample)
      const bool staged = (b - a) <= WF_QSTAGE;
      if (staged) {
        for (int q = a + lane_id(); q < b; q += 32) {
          if (sizeof(R) == 8) {
            j0_s[q - a] = int32_t(first_sample<R>(p, t[q], ts));
            qn_s[q - a] = R(qc[q] / p.spe_ref_charge);
          } else {
            float dt = float(t[q] - ts);
            dt_s[q - a] = dt;
            j0_s[q - a] = first_sample_f(dt, Pf);
            qn_s[q - a] = R(d2f_trunc(qc[q])) * inv_q;        // FP32-stage charges: exact FP32 values
          }
        }
        __syncwarp();
      }
      // samples: sum of the charges reaching each sample, in charge order
      for (int j = lane_id(); j < L; j += 32) {
        // charges with first_sample in (j - nr, j]: first_sample is non-decreasing along the cluster.  The staged
        // and the on-the-fly searches are separate loops, so the staged one carries no FP64 work.
        int q1, lo2;
        if (staged) {
          int lo_q = a, hi_q = b;                    // first charge with first_sample > j - nr
          while (lo_q < hi_q) {
            int m = (lo_q + hi_q) >> 1;
            if (j0_s[m - a] > j - nr) hi_q = m; else lo_q = m + 1;
          }
          q1 = lo_q;
          int hi2 = b;                               // first charge with first_sample > j
          lo2 = q1;
          while (lo2 < hi2) {
            int m = (lo2 + hi2) >> 1;
            if (j0_s[m - a] > j) hi2 = m; else lo2 = m + 1;
          }
        } else {
          int lo_q = a, hi_q = b;
          while (lo_q < hi_q) {
            int m = (lo_q + hi_q) >> 1;
            if (first_sample<R>(p, t[m], ts) > (long long)j - nr) hi_q = m; else lo_q = m + 1;
          }
          q1 = lo_q;
          int hi2 = b;
          lo2 = q1;
          while (lo2 < hi2) {
            int m = (lo2 + hi2) >> 1;
            if (first_sample<R>(p, t[m], ts) > (long long)j) hi2 = m; else lo2 = m + 1;
          }
        }
        R acc = R(0);
        if (sizeof(R) == 4 && staged) {
          for (int q = q1; q < lo2; ++q) {
            int ti = tmpl_index_f(j, dt_s[q - a], Pf, ip, tlen);
            if (ti >= 0) acc += R(tmpl_f[ti]) * qn_s[q - a];
          }
        } else {
          for (int q = q1; q < lo2; ++q) {
            int ti = tmpl_index<R>(p, j, t[q], ts, tlen);
            if (ti >= 0) acc += R(tmpl[ti]) * (staged ? qn_s[q - a] : R(qc[q] / p.spe_ref_charge));
          }
        }
        if (p.noise_on) {
          long long tk = k0 + j;
          U4 w = keyed(p.seed, ek, (ST_NOISE << 28) | (chan & 0x7FFFu), uint32_t(tk >> 1));
          R z0, z1;
          Math<R>::normal_pair(w, &z0, &z1);
          acc = acc + sigma * ((tk & 1) ? z1 : z0);
        }
        wave[j] = acc;
      }
      __syncwarp();
      const int i_lo = C.ilo, i_hi = C.ihi;
      // zero suppression over chunks of 32 samples
      int next_i = 0;
      for (int base = 0; base < L; base += 32) {
        int i = base + lane_id();
        bool w = false;
        if (i < L) {
          for (int d = -2; d <= 2 && !w; ++d) {
            int k = i + d;
            if (k >= 0 && k < L && wave[k] > vthr) w = true;
          }
        }
        bool inwin = i >= i_lo && i <= i_hi;
        unsigned cand = __ballot_sync(0xffffffffu, w && inwin);
        while (true) {
          unsigned m = cand;
          if (next_i > base) m &= (next_i - base >= 32) ? 0u : ~((1u << (next_i - base)) - 1u);
          if (!m) break;
          int i0 = base + __ffs(m) - 1;
          // emit digi at i0; its start TDC (start - TDC0) / P is the integer tick k0 + i0
          if (nd < scap) {
            long long o = slot + nd;
            if (lane_id() < zs) {
              int c = i0 + lane_id();
              if constexpr (sizeof(R) == 4) {
                const float v = c < L ? float(wave[c]) : 0.0f;
                if (D.volt) D.volt[o * zs + lane_id()] = f2d(v);
                D.adc[o * zs + lane_id()] = adc_of_f(p, v, conv_f, off_f);
              } else {
                double v = c < L ? double(wave[c]) : 0.0;
                if (D.volt) D.volt[o * zs + lane_id()] = v;
                D.adc[o * zs + lane_id()] = adc_of(p, v);
              }
            }
            if (lane_id() == 0) {
              D.chan[o] = lab;
              D.start[o] = __dadd_rn(ts, __dmul_rn(double(i0), p.period));
              D.tdc0[o] = tdc0c;
              D.starttdc[o] = k0 + i0;
            }
          }
          ++nd;
          next_i = i0 + zs;
        }
      }
      __syncwarp();
    }
    if (lane_id() == 0) {
      D.n[g] = nd;
      if (nd > scap) set_flag(status, CRV_ST_CAPACITY);
    }
  }
}

}  // namespace crv

namespace crv {

struct Digis {
  long long* chan;
  double* start;
  double* tdc0;
  long long* starttdc;
  double* volt;
  int16_t* adc;
};

#ifdef CRV_ENGINE_TU
// Move each group's digis from its slots to the output, ordered by start (stable) within the group.
// O.start, O.tdc0 and O.volt may be null (the resident chain reads channel, start TDC and ADC only): not written
__global__ void k_digi_compact(const long long* __restrict__ ng_dev, DigiSlots D, const long long* __restrict__ out_off,
                               int zs, Digis O, long long out_cap) {
  long long ng = *ng_dev;
  long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long g = blockIdx.x * (long long)(blockDim.x >> 5) + warp_in_block(); g < ng; g += warps) {
    int nd = D.n[g];
    if (nd > D.cap[g]) continue;
    long long s0 = D.off[g], o0 = out_off[g];
    if (o0 + nd > out_cap) continue;
    // digis come out of the synthesis in start order (clusters in time order, digis in sample order): then the stable
    // order by start is the production order and the copy runs over all lanes
    bool sorted = true;
    for (int j = lane_id() + 1; j < nd; j += 32) sorted = sorted && !(D.start[s0 + j] < D.start[s0 + j - 1]);
    if (__all_sync(0xffffffffu, sorted)) {
      for (int i = lane_id(); i < nd; i += 32) {
        O.chan[o0 + i] = D.chan[s0 + i];
        if (O.start) O.start[o0 + i] = D.start[s0 + i];
        if (O.tdc0) O.tdc0[o0 + i] = D.tdc0[s0 + i];
        O.starttdc[o0 + i] = D.starttdc[s0 + i];
      }
      for (long long f = lane_id(); f < (long long)nd * zs; f += 32) {
        if (O.volt) O.volt[o0 * zs + f] = D.volt[s0 * zs + f];
        O.adc[o0 * zs + f] = D.adc[s0 * zs + f];
      }
      continue;
    }
    for (int i = 0; i < nd; ++i) {
      // rank of digi i among the group's digis by start, ties by production order
      double si = D.start[s0 + i];
      int r = 0;
      for (int j = lane_id(); j < nd; j += 32) {
        double sj = D.start[s0 + j];
        r += (sj < si) || (sj == si && j < i);
      }
      r = warp_sum(r);
      long long o = o0 + r, s = s0 + i;
      if (lane_id() == 0) {
        O.chan[o] = D.chan[s];
        if (O.start) O.start[o] = D.start[s];
        if (O.tdc0) O.tdc0[o] = D.tdc0[s];
        O.starttdc[o] = D.starttdc[s];
      }
      if (lane_id() < zs) {
        if (O.volt) O.volt[o * zs + lane_id()] = D.volt[s * zs + lane_id()];
        O.adc[o * zs + lane_id()] = D.adc[s * zs + lane_id()];
      }
    }
  }
}

// Segments of equal labels in a label-sorted array: heads, then group start/label/count.
__global__ void k_label_heads(long long n, const long long* __restrict__ n_dev, const long long* __restrict__ label,
                              int32_t* __restrict__ head) {
  n = bounded_count(n, n_dev);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    head[i] = (i == 0 || label[i] != label[i - 1]) ? 1 : 0;
}

__global__ void k_label_groups(long long n, const long long* __restrict__ n_dev, const long long* __restrict__ label,
                               const int32_t* __restrict__ head, const long long* __restrict__ gidx,
                               long long* __restrict__ gstart, long long* __restrict__ glabel) {
  n = bounded_count(n, n_dev);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    if (head[i]) {
      long long g = gidx[i];
      gstart[g] = i;
      glabel[g] = label[i];
    }
}

// counts from consecutive starts; run per group from a sorted (event key -> run) table (run 0 if absent)
__global__ void k_group_counts(const long long* __restrict__ ng_dev, long long n, const long long* __restrict__ n_dev,
                               const long long* __restrict__ gstart, const long long* __restrict__ glabel,
                               int32_t* __restrict__ gcount, const long long* __restrict__ ev_keys,
                               const uint32_t* __restrict__ ev_runs, long long n_ev, uint32_t* __restrict__ grun,
                               Status* status) {
  long long ng = *ng_dev;
  n = bounded_count(n, n_dev);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x) {
    long long e = (g + 1 < ng ? gstart[g + 1] : n) - gstart[g];
    gcount[g] = int32_t(e);
    uint32_t r = 0;
    if (ev_keys && n_ev > 0) {
      long long k = glabel[g] / 32768;
      long long lo = 0, hi = n_ev;
      while (lo < hi) {
        long long m = (lo + hi) >> 1;
        if (ev_keys[m] < k) lo = m + 1; else hi = m;
      }
      if (lo < n_ev && ev_keys[lo] == k) r = ev_runs[lo];
      else set_flag(status, CRV_ST_ORDER);
    }
    grun[g] = r;
  }
}
#endif

}  // namespace crv
