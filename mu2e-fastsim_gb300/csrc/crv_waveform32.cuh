// FP32-mixed waveform stage: SiPM charges -> zero-suppressed digis with no FP64 instruction on the common path.
//
// Same semantics as crv_waveform.cuh (the reference's synthesis, crv/crvfastsim/reco/waveform.py:65-172), different
// arithmetic: GB300 issues FP64 at ~1/70 of the FP32 rate and a warp-wide FP64 instruction costs the same with one
// active lane as with 32, so the per-cluster scalars that the FP64 path computes in double precision (cluster start
// tick, start time, length, window range, TDC0) are computed here in 64-bit fixed point (times x 2^32, integer
// arithmetic), and every sample sums its charges in FP32 on times relative to the cluster start.
//
//   times        t_fx = trunc(t * 2^32) (|t| < 2^30 ns; larger or non-finite times set CRV_ST_LIMIT / NONFINITE);
//                differences are exact integers, converted to FP32 once (dt of a charge from its cluster start);
//   TDC0         keyed draw as in the FP64 path: the same 53 random bits times the phase width, in fixed point;
//   k0           ceil((t_first - P - TDC0) / P) exactly on the fixed-point values (FP32 estimate, integer fix-up);
//   outputs      start and TDC0 of a digi are the fixed-point values converted exactly to double; volts are the
//                FP32 sums widened exactly; ADC as the FP32 stage rule (adc_of_f).
//
// Two kernels, one warp per SiPM group each:
//   k_wf_prep32   lanes over the group's charges: cluster split by the gap test on consecutive fixed-point times
//                 (ballots), then lanes over the clusters: keep rule, start tick, length, window sample range, digi
//                 bound; kept clusters are written to cl[group start + k] (the record layout of WfCluster, with the
//                 fixed-point start in place of the double).
//   k_wf_synth32  per kept cluster: the charges' FP32 offsets from the cluster start and normalised charges are
//                 staged in shared memory (coalesced loads), then lanes own samples (32 per tile) and sum the
//                 template contributions of the staged charges in charge order (deterministic), keyed noise is
//                 added, and the zero-suppression scan emits digis 32 samples per ballot.
#pragma once
#include "crv_waveform.cuh"

namespace crv {

constexpr int WF_FX = 32;                      // fractional bits of fixed-point times

// trunc(x * 2^32) for |x| < 2^30; false for non-finite or larger values
__device__ __forceinline__ bool d2fx(double x, long long* out) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = int((b >> 52) & 0x7FF);
  if (e == 0x7FF || e >= 1023 + 30) return false;
  if (e < 1023 - WF_FX - 1) {                  // |x| < 2^-33: below the resolution
    *out = 0;
    return true;
  }
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int sh = e - 1075 + WF_FX;             // in [-54, 10]
  const unsigned long long v = sh >= 0 ? (m << sh) : (m >> (-sh));
  *out = (b >> 63) ? -(long long)v : (long long)v;
  return true;
}

// v * 2^-32 as FP32: integer part and fraction converted separately, one final rounding
__device__ __forceinline__ float fx2f(long long v) {
  const int hi = int(v >> 32);                 // floor(v / 2^32): |v| < 2^62
  const unsigned int lo = (unsigned int)(v & 0xFFFFFFFFll);
  return fmaf(__uint2float_rn(lo), 0x1p-32f, __int2float_rn(hi));
}

// v * 2^-32 as double by integer construction of the bits: exact for |v| < 2^53 (times below 2^21 ns), truncated
// beyond
__device__ __forceinline__ double fx2d(long long v) {
  if (v == 0) return 0.0;
  const unsigned long long a = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
  const int lz = __clzll((long long)a);
  const unsigned long long m = lz >= 11 ? a << (lz - 11) : a >> (11 - lz);   // leading bit at 52
  const unsigned long long e = (unsigned long long)(1023 + (63 - lz) - WF_FX);
  return __longlong_as_double((long long)((e << 52) | (m & 0xFFFFFFFFFFFFFull) | (v < 0 ? (1ull << 63) : 0ull)));
}

// ceil(x / d) and floor(x / d) for d > 0 on fixed-point values whose quotient is below 2^30 in magnitude: FP32
// estimate (a 32-bit conversion: the 64-bit one issues at a small fraction of the rate), exact integer correction
__device__ __forceinline__ long long fx_ceil_div(long long x, long long d, float inv_d) {
  long long k = (long long)(int)ceilf(fminf(fmaxf(fx2f(x) * inv_d, -1073741824.0f), 1073741824.0f));
  while (k * d < x) ++k;
  while ((k - 1) * d >= x) --k;
  return k;
}
__device__ __forceinline__ long long fx_floor_div(long long x, long long d, float inv_d) {
  long long k = (long long)(int)floorf(fminf(fmaxf(fx2f(x) * inv_d, -1073741824.0f), 1073741824.0f));
  while (k * d > x) --k;
  while ((k + 1) * d <= x) ++k;
  return k;
}

// keyed TDC0 in fixed point: the FP64 path's 53 random bits times the phase width
__device__ __forceinline__ long long tdc0_fx_of(const CrvParams& p, const CrvChannels& ch, long long label,
                                                uint32_t run, long long width_fx) {
  const long long evk = label / 32768;
  const int c = int(label % 32768);
  EvKey ek{uint32_t(evk & 0xFFFFF), uint32_t(evk >> 20), run};
  U4 w = keyed(p.seed, ek, ST_TDC0 << 28, uint32_t(feb_key(p, ch, c)));
  const unsigned long long u53 = bits53(w.x, w.y);
  return (long long)__umul64hi(u53 << 11, (unsigned long long)width_fx);
}

struct WfFx {                   // per-launch constants of the fixed-point forms
  long long P, gap, maxt, wlo, whi, width;
  float invP;                   // 1 / P in ns (FP32, for the quotient estimates)
  int nmin;                     // smallest charge count of a kept cluster
  bool ok;
};

// order-preserving unsigned key of a double's bits (larger key = larger value), so a maximum over a table is
// integer work: a warp-wide FP64 instruction costs ~60-70 FP32 issue slots on this GPU
__device__ __forceinline__ unsigned long long dkey(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_value(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}

// the template's maximum (NaN entries ignored, as fmax does) by every thread of the block; call from all threads
__device__ __forceinline__ double block_tmpl_max(const double* tmpl, int tlen, unsigned long long* slot) {
  if (threadIdx.x == 0) *slot = dkey(-1e300);
  __syncthreads();
  unsigned long long m = dkey(-1e300);
  for (int i = threadIdx.x; i < tlen; i += blockDim.x) {
    const double v = tmpl[i];
    const unsigned long long k = dkey(v);
    if (v == v && k > m) m = k;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
    if (x > m) m = x;
  }
  if (lane_id() == 0) atomicMax(slot, m);
  __syncthreads();
  return dkey_value(*slot);
}

__device__ __forceinline__ WfFx wf_fx_consts(const CrvParams& p, double vmax) {
  WfFx f;
  f.ok = d2fx(p.period, &f.P) && d2fx(p.spe_max_time + 4.0 * p.period, &f.gap) && d2fx(p.spe_max_time, &f.maxt) &&
         d2fx(fmax(fmin(p.window_lo, 5e8), -5e8), &f.wlo) && d2fx(fmax(fmin(p.window_hi, 5e8), -5e8), &f.whi) &&
         d2fx(p.feb_phase_width, &f.width) && f.P > 0;
  f.invP = float(1.0 / p.period);              // fx_ceil_div / fx_floor_div estimate on times in ns
  // keep rule n * vmax >= min_voltage (n integer, monotone in n): the smallest such n
  int n = vmax > 0.0 ? int(fmin(ceil(p.min_voltage / vmax), 2e9)) : 2000000000;
  if (n < 0) n = 0;
  while (n > 0 && double(n - 1) * vmax >= p.min_voltage) --n;
  while (n < 2000000000 && !(double(n) * vmax >= p.min_voltage)) ++n;
  f.nmin = n;
  return f;
}

// The FP32 path's cluster record: WfCluster's layout with the fixed-point start time in place of the double.
struct WfCluster32 {
  long long ts_fx;
  long long k0;
  int32_t a, b, L;
  int16_t ilo, ihi;
};
static_assert(sizeof(WfCluster32) == sizeof(WfCluster), "FP32 cluster record layout");

__global__ void __launch_bounds__(256) k_wf_prep32(CrvParams p, CrvChannels ch, WfGroups G,
                                                   const double* __restrict__ time, const double* __restrict__ tmpl,
                                                   int tlen, const double* __restrict__ tdc0_rows,
                                                   double* __restrict__ g_tdc0, int32_t* __restrict__ g_bound,
                                                   int32_t* __restrict__ g_maxlen, int32_t* __restrict__ g_nkept,
                                                   int32_t* __restrict__ cstart, WfCluster32* __restrict__ cl,
                                                   Status* status) {
  __shared__ WfFx fx_s;
  __shared__ unsigned long long vmax_s;
  __shared__ float ip_s, pf_s;
  __shared__ int nr_s;
  const double vmax = block_tmpl_max(tmpl, tlen, &vmax_s);
  if (threadIdx.x == 0) {                      // FP64 scalars once per block, in one thread
    fx_s = wf_fx_consts(p, vmax);
    ip_s = float(1.0 / p.spe_precision);
    pf_s = float(p.period);
    nr_s = reach_samples(p);
  }
  __syncthreads();
  const WfFx F = fx_s;
  if (!F.ok || tlen > 1024) {
    if (threadIdx.x == 0 && blockIdx.x == 0) set_flag(status, CRV_ST_LIMIT);
    return;
  }
  const int nr = nr_s;
  const int zs = p.samples_zs;
  const float Pf = pf_s, ip = ip_s;
  const int lane = lane_id();
  const long long ng = *G.n;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long g = blockIdx.x * (long long)(blockDim.x >> 5) + warp_in_block(); g < ng; g += warps) {
    const int n = G.count[g];
    const long long q0 = G.start[g];
    const double* t = time + q0;
    // keyed TDC0 of the group (unless the caller gives one per cluster)
    long long tdc0g = 0;
    if (!tdc0_rows) tdc0g = tdc0_fx_of(p, ch, G.label[g], G.run ? G.run[g] : 0u, F.width);
    // 1) cluster starts: a new cluster where consecutive fixed-point times differ by more than the gap
    int ncl = 0;
    long long prev = 0;
    bool bad = false;
    for (int base = 0; base < n; base += 32) {
      const int q = base + lane;
      long long tf = 0;
      if (q < n) bad |= !d2fx(t[q], &tf);
      long long tp = __shfl_up_sync(0xffffffffu, tf, 1);
      if (lane == 0) tp = prev;
      const bool isnew = q < n && (q == 0 || tf - tp > F.gap);
      const unsigned m = __ballot_sync(0xffffffffu, isnew);
      if (isnew) cstart[q0 + ncl + __popc(m & ((1u << lane) - 1u))] = q;
      ncl += __popc(m);
      prev = __shfl_sync(0xffffffffu, tf, 31);
    }
    if (__any_sync(0xffffffffu, bad)) {
      if (lane == 0) set_flag(status, CRV_ST_LIMIT);
      if (lane == 0) { g_bound[g] = 0; g_maxlen[g] = 0; g_nkept[g] = 0; g_tdc0[g] = 0.0; }
      continue;
    }
    __syncwarp();
    // 2) lanes over clusters: keep rule, start tick, length, window range, digi bound
    long long bound = 0;
    int maxlen = 0, nk = 0;
    for (int cb = 0; cb < ncl; cb += 32) {
      const int c = cb + lane;
      int a = 0, b = 0;
      if (c < ncl) {
        a = cstart[q0 + c];
        b = c + 1 < ncl ? cstart[q0 + c + 1] : n;
      }
      __syncwarp();                              // every lane has read its starts before records are written
      bool keep = c < ncl && (b - a) >= F.nmin;
      WfCluster32 rec{};
      int L = 0;
      if (keep) {
        long long tdc0 = tdc0g;
        if (tdc0_rows && !d2fx(tdc0_rows[q0 + a], &tdc0)) {
          set_flag(status, CRV_ST_LIMIT);
          tdc0 = 0;
        }
        long long tf, tl;
        d2fx(t[a], &tf);
        d2fx(t[b - 1], &tl);
        const long long k0 = fx_ceil_div(tf - F.P - tdc0, F.P, F.invP);
        const long long ts = k0 * F.P + tdc0;
        const long long est = fx_floor_div(tl - tf + F.maxt, F.P, F.invP);
        // the last charge reaches the last sample (the reach only grows with the charge time)
        const float dt = fx2f(tl - ts);
        long long used = 0;
        const int j0 = first_sample_f(dt, Pf);
        for (int k = nr - 1; k >= 0; --k)
          if (tmpl_index_f(j0 + k, dt, Pf, ip, tlen) >= 0) {
            used = j0 + k + 1;
            break;
          }
        L = int(est > used ? est : used);
        int ilo = 0, ihi = -1;
        if (L <= 16384) {
          const long long last = ts + (long long)(L - 1) * F.P;
          ilo = ts >= F.wlo ? 0 : int(min((long long)L, fx_ceil_div(F.wlo - ts, F.P, F.invP)));
          ihi = last <= F.whi ? L - 1 : int(max(-1ll, fx_floor_div(F.whi - ts, F.P, F.invP)));
        }
        rec = WfCluster32{ts, k0, a, b, L, int16_t(ilo), int16_t(ihi)};
      }
      const unsigned km = __ballot_sync(0xffffffffu, keep);
      if (keep) cl[q0 + nk + __popc(km & ((1u << lane) - 1u))] = rec;
      nk += __popc(km);
      long long bnd = keep ? (L + zs - 1) / zs : 0;
      int ml = keep ? L : 0;
      for (int o = 16; o > 0; o >>= 1) {
        bnd += __shfl_xor_sync(0xffffffffu, bnd, o);
        ml = max(ml, __shfl_xor_sync(0xffffffffu, ml, o));
      }
      bound += bnd;
      maxlen = max(maxlen, ml);
    }
    if (lane == 0) {
      g_bound[g] = int32_t(bound);
      g_maxlen[g] = maxlen;
      g_nkept[g] = nk;
      g_tdc0[g] = fx2d(tdc0g);
    }
  }
}

constexpr int WF32_QS = 256;      // charges staged per chunk (per warp)

__host__ __device__ inline size_t wf32_smem_per_warp(int cap) {
  return (size_t(cap) * 4 + size_t(WF32_QS) * 12 + 15) & ~size_t(15);
}

// Synthesis + zero suppression of the groups whose longest kept cluster is in (lo, cap] (FP32-mixed).
__global__ void __launch_bounds__(256, 4) k_wf_synth32(CrvParams p, WfGroups G, const double* __restrict__ time,
                                                    const double* __restrict__ charge, const double* __restrict__ tmpl,
                                                    int tlen, const double* __restrict__ tdc0_rows,
                                                    const double* __restrict__ g_tdc0,
                                                    const int32_t* __restrict__ g_maxlen,
                                                    const int32_t* __restrict__ g_nkept,
                                                    const WfCluster32* __restrict__ cl, int lo, int cap,
                                                    int last_pass, DigiSlots D, Status* status) {
  extern __shared__ __align__(16) char smem[];
  __shared__ float tmpl_f[1024];
  __shared__ long long P_fx_s;
  char* wbase = smem + size_t(warp_in_block()) * wf32_smem_per_warp(cap);
  float* wave = reinterpret_cast<float*>(wbase);
  float2* sq = reinterpret_cast<float2*>(wbase + size_t(cap) * 4);              // (dt, normalised charge)
  int* sj = reinterpret_cast<int*>(wbase + size_t(cap) * 4 + size_t(WF32_QS) * 8);  // first sample reached
  __shared__ float cf_s[7];
  __shared__ int nr_s;
  if (tlen > 1024) return;                     // refused by the host; the table must fit the shared copy
  for (int i = threadIdx.x; i < tlen; i += blockDim.x) tmpl_f[i] = float(tmpl[i]);
  if (threadIdx.x == 0) {                      // FP64 scalars once per block, in one thread
    long long P;
    P_fx_s = d2fx(p.period, &P) ? P : 0;
    cf_s[0] = float(p.period);
    cf_s[1] = float(1.0 / p.spe_precision);
    cf_s[2] = float(1.0 / p.spe_ref_charge);
    cf_s[3] = float(p.min_voltage);
    cf_s[4] = float(p.noise_sigma);
    cf_s[5] = float(p.adc_conversion);
    cf_s[6] = float(double(p.adc_pedestal) + 0.5);
    nr_s = reach_samples(p);
  }
  __syncthreads();
  const long long P_fx = P_fx_s;
  const int nr = nr_s;
  const int zs = p.samples_zs;
  const int lane = lane_id();
  const float Pf = cf_s[0], ip = cf_s[1];
  const float inv_q = cf_s[2];
  const float vthr = cf_s[3];
  const float sigma = cf_s[4];
  const float conv_f = cf_s[5], off_f = cf_s[6];
  const long long ng = *G.n;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  // groups in tiles of 32 per warp: one coalesced load of their longest clusters and a ballot pick this pass's groups
  for (long long g0 = (blockIdx.x * (long long)(blockDim.x >> 5) + warp_in_block()) * 32; g0 < ng; g0 += warps * 32) {
   const long long gl = g0 + lane;
   const int mll = gl < ng ? g_maxlen[gl] : 0;
   unsigned todo = __ballot_sync(0xffffffffu, gl < ng && mll > lo);
   while (todo) {
    const int bsel = __ffs(todo) - 1;
    todo &= todo - 1;
    const long long g = g0 + bsel;
    const int ml = __shfl_sync(0xffffffffu, mll, bsel);
    if (ml > cap) {
      if (last_pass && lane == 0) {
        set_flag(status, CRV_ST_CAPACITY);
        need_at_least(status, CRV_NEED_SAMPLES, ml);
      }
      continue;
    }
    const long long q0 = G.start[g];
    const double* t = time + q0;
    const double* qc = charge + q0;
    const long long lab = G.label[g];
    const uint32_t run = G.run ? G.run[g] : 0u;
    const long long evk = lab / 32768;
    const EvKey ek{uint32_t(evk & 0xFFFFF), uint32_t(evk >> 20), run};
    const uint32_t chan = uint32_t(lab % 32768);
    const double tdc0g = g_tdc0[g];
    const long long slot = D.off[g];
    const int scap = D.cap[g];
    int nd = 0;
    const int nk = g_nkept[g];
    for (int kc = 0; kc < nk; ++kc) {
      const WfCluster32 C = cl[q0 + kc];
      const int a = C.a, b = C.b, L = C.L;
      const long long k0 = C.k0, ts = C.ts_fx;
      const double tdc0c = tdc0_rows ? tdc0_rows[q0 + a] : tdc0g;
      for (int j = lane; j < L; j += 32) wave[j] = 0.0f;
      // charges in chunks: stage (dt, q) and the first sample reached, then every 32-sample tile the chunk reaches
      for (int c0 = a; c0 < b; c0 += WF32_QS) {
        const int nq = min(WF32_QS, b - c0);
        __syncwarp();
        for (int i = lane; i < nq; i += 32) {
          long long tf = 0;
          d2fx(t[c0 + i], &tf);
          const float dt = fx2f(tf - ts);
          sq[i] = make_float2(dt, d2f_trunc(qc[c0 + i]) * inv_q);
          sj[i] = first_sample_f(dt, Pf);
        }
        __syncwarp();
        const int jA = sj[0];
        const int jB = min(sj[nq - 1] + nr - 1, L - 1);
        for (int T = (jA >> 5) << 5; T <= jB; T += 32) {
          // charges of the chunk that can reach the tile: first sample in (T - nr, T + 31]
          int q1 = 0, hi = nq;
          while (q1 < hi) {
            const int m = (q1 + hi) >> 1;
            if (sj[m] > T - nr) hi = m; else q1 = m + 1;
          }
          int q2 = q1;
          hi = nq;
          while (q2 < hi) {
            const int m = (q2 + hi) >> 1;
            if (sj[m] > T + 31) hi = m; else q2 = m + 1;
          }
          // a cluster of at most 16 samples (most of them) takes two lanes per sample, each summing every other
          // charge; the two partial sums are added in a fixed order, so the result is the same on every run
          const int split = L <= 16 ? 1 : 0;
          const int J = T + (split ? (lane & 15) : lane);
          const int part = split ? (lane >> 4) : 0;
          const float JP = float(J) * Pf;
          float acc = 0.0f;
#pragma unroll 4
          for (int q = q1 + part; q < q2; q += 1 + split) {
            const float2 v = sq[q];
            const float st = JP - v.x;
            // nearest integer of st / precision (ties to even) by the 1.5 x 2^23 shift; |st / precision| < 2^22
            const int ti = __float_as_int(fmaf(st, ip, 12582912.0f)) - 0x4B400000;
            if (st >= 0.0f && ti < tlen) acc = fmaf(tmpl_f[ti], v.y, acc);
          }
          const float other = __shfl_down_sync(0xffffffffu, acc, 16);
          if (split) acc = acc + other;
          if (J < L && (split ? lane < 16 : true)) wave[J] = wave[J] + acc;
        }
      }
      __syncwarp();
      // keyed electronics noise on every sample
      if (p.noise_on) {
        for (int j = lane; j < L; j += 32) {
          const long long tk = k0 + j;
          U4 w = keyed(p.seed, ek, (ST_NOISE << 28) | (chan & 0x7FFFu), uint32_t(tk >> 1));
          float z0, z1;
          Math<float>::normal_pair(w, &z0, &z1);
          wave[j] = wave[j] + sigma * ((tk & 1) ? z1 : z0);
        }
        __syncwarp();
      }
      // zero suppression over tiles of 32 samples
      const int i_lo = C.ilo, i_hi = C.ihi;
      int next_i = 0;
      for (int base = 0; base < L; base += 32) {
        const int i = base + lane;
        bool w = false;
        if (i < L) {
          for (int d = -2; d <= 2 && !w; ++d) {
            const int k = i + d;
            if (k >= 0 && k < L && wave[k] > vthr) w = true;
          }
        }
        const bool inwin = i >= i_lo && i <= i_hi;
        const unsigned cand = __ballot_sync(0xffffffffu, w && inwin);
        while (true) {
          unsigned m = cand;
          if (next_i > base) m &= (next_i - base >= 32) ? 0u : ~((1u << (next_i - base)) - 1u);
          if (!m) break;
          const int i0 = base + __ffs(m) - 1;
          if (nd < scap) {
            const long long o = slot + nd;
            if (lane < zs) {
              const int c = i0 + lane;
              const float v = c < L ? wave[c] : 0.0f;
              if (D.volt) D.volt[o * zs + lane] = f2d(v);
              D.adc[o * zs + lane] = adc_of_f(p, v, conv_f, off_f);
            }
            if (lane == 0) {
              D.chan[o] = lab;
              D.start[o] = fx2d(ts + (long long)i0 * P_fx);
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
    if (lane == 0) {
      D.n[g] = nd;
      if (nd > scap) set_flag(status, CRV_ST_CAPACITY);
    }
   }
  }
}

}  // namespace crv
