// Response stage: CrvSteps -> photons at the SiPMs -> SiPM charges.
//
// Photon counts per (step, SiPM) follow the reference rule Gauss(mean, sqrt mean) if mean > 10 else Poisson(mean),
// rint, floor at 0 (crv/crvfastsim/response/photons.py:102-112) with the analytic yield x two-exponential attenuation
// in place of the lookup tables; SiPMs 0/2 read the -length end and 1/3 the +length end (photons.py:333-356).
//
// The SiPM model is the reference's serial one (crv/crvfastsim/response/sipm.py:141-198): per SiPM, photons in time
// order; a pixel fires with p1 (1 - e^(-v/p2)), v = Vov (1 - e^(-(t - t_last)/tau)); each firing draws cross-talk
// on its 4 neighbours, handled breadth first with multiplicity merging 1 - (1 - p)^m before the next photon; trap
// afterpulses are scheduled per firing and fired after all photons in time order.
//
// GPU mapping: one warp per SiPM.  The warp stages the SiPM's photons in shared memory, sorts them by
// (time, draw key) with a bitonic network, and keeps the pixel state (last-discharge time per pixel + a fired
// bitmap) in shared memory.  Photons are evaluated 32 at a time, one per lane, against the state at the start of the
// batch; the batch commits up to the first lane whose result could depend on an earlier lane of the same batch (same
// pixel as an earlier lane) or that starts a cross-talk cascade (then the cascade runs, generation by generation,
// with the frontier spread over the lanes).  Keyed draws make every lane's random numbers independent of the
// processing order, so the result is exactly the serial one.
#pragma once
#include "crv_device.cuh"
#include "crv_scan.cuh"

namespace crv {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename S>
__device__ __forceinline__ double ld_real(const void* p, long long i) {
  return double(static_cast<const S*>(p)[i]);
}

__device__ __forceinline__ double step_real(const CrvSteps& st, const void* p, long long i) {
  return st.real_bytes == 4 ? double(static_cast<const float*>(p)[i]) : static_cast<const double*>(p)[i];
}

// ---------------------------------------------------------------------------------------------------------------------
// event preparation: steps of each event grouped by bar (stable), per-step event index, SiPM count per event

constexpr int PREP_THREADS = 256;

#ifdef CRV_ENGINE_TU
// keys: bar << 16 | step-in-event; sorted ascending in shared memory (bitonic, block-wide)
__device__ void block_bitonic_u32(uint32_t* a, int P) {
  for (int size = 2; size <= P; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int q = threadIdx.x; q < (P >> 1); q += blockDim.x) {
        int lo = 2 * stride * (q / stride) + (q % stride);
        int hi = lo + stride;
        bool up = (lo & size) == 0;
        uint32_t x = a[lo], y = a[hi];
        if ((x > y) == up) { a[lo] = y; a[hi] = x; }
      }
      __syncthreads();
    }
  }
}

// mode 0: count SiPMs per event (sipm_count); mode 1: write the SiPM table at sipm_off
__global__ void k_event_prep(CrvEvents ev, long long nevents, CrvSteps st, CrvChannels ch, int masked,
                             int step_cap, int32_t* __restrict__ step_event, int32_t* __restrict__ step_order,
                             int32_t* __restrict__ sipm_count, const long long* __restrict__ sipm_off,
                             int32_t* __restrict__ s_event, int32_t* __restrict__ s_chan,
                             long long* __restrict__ s_seg, int32_t* __restrict__ s_nseg, Status* status, int mode) {
  extern __shared__ uint32_t keys[];
  __shared__ int wcount[PREP_THREADS / 32];
  for (long long e = blockIdx.x; e < nevents; e += gridDim.x) {
    long long f = ev.first_step[e];
    int n = ev.nsteps[e];
    if (mode == 0 && step_event)
      for (int i = threadIdx.x; i < n; i += blockDim.x) step_event[f + i] = int32_t(e);
    if (n > step_cap || n >= 65536) {
      if (threadIdx.x == 0) {
        if (n >= 65536) set_flag(status, CRV_ST_LIMIT);
        else { set_flag(status, CRV_ST_CAPACITY); need_at_least(status, CRV_NEED_STEPS_PER_EVENT, n); }
        if (mode == 0) sipm_count[e] = 0;
      }
      continue;
    }
    int P = 1;
    while (P < n) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      if (i < n) {
        int b = st.bar[f + i];
        keys[i] = (uint32_t(b) << 16) | uint32_t(i);
      } else {
        keys[i] = 0xFFFFFFFFu;
      }
    }
    __syncthreads();
    block_bitonic_u32(keys, P);
    if (mode == 0 && step_order)
      for (int i = threadIdx.x; i < n; i += blockDim.x) step_order[f + i] = int32_t(f + (keys[i] & 0xFFFFu));
    // segments: thread i starts a segment if bar differs from i-1
    int mine = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      uint32_t b = keys[i] >> 16;
      if (i == 0 || (keys[i - 1] >> 16) != b) {
        for (int s = 0; s < 4; ++s) {
          int c = int(b) * 4 + s;
          bool ok = !masked || (ch.status[c] & 0b101) == 0;
          mine += ok;
        }
      }
    }
    if (mode == 0) {
      int tot = warp_sum(mine);
      if (lane_id() == 0) wcount[warp_in_block()] = tot;
      __syncthreads();
      if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wcount[w];
        sipm_count[e] = t;
      }
      __syncthreads();
    } else {
      // serial write in segment order by thread 0 (events are small; keeps label order)
      if (threadIdx.x == 0) {
        long long o = sipm_off[e];
        for (int i = 0; i < n;) {
          uint32_t b = keys[i] >> 16;
          int j = i;
          while (j < n && (keys[j] >> 16) == b) ++j;
          for (int s = 0; s < 4; ++s) {
            int c = int(b) * 4 + s;
            if (masked && (ch.status[c] & 0b101) != 0) continue;
            s_event[o] = int32_t(e);
            s_chan[o] = c;
            s_seg[o] = f + i;
            s_nseg[o] = j - i;
            ++o;
          }
          i = j;
        }
      }
      __syncthreads();
    }
  }
}

#endif  // CRV_ENGINE_TU

// ---------------------------------------------------------------------------------------------------------------------
// photon counts and arrival times

template <typename R>
__device__ __forceinline__ R readout_distance(R z, R half, int s) {
  R d = (s % 2 == 0) ? (z + half) : (half - z);
  if (d < R(0)) d = R(0);
  if (d > R(2) * half) d = R(2) * half;
  return d;
}

template <typename R>
__device__ __forceinline__ R mean_photons(const CrvParams& p, R edep, R dev, R d) {
  using M = Math<R>;
  R att = R(p.frac_short) * M::exp(-d / R(p.lambda_short)) + R(p.frac_long) * M::exp(-d / R(p.lambda_long));
  return R(p.yield_per_mev) * edep * dev * att;
}

template <typename R>
__device__ __forceinline__ int draw_count(R avg, const U4& w) {
  using M = Math<R>;
  R x;
  if (avg > R(10)) {
    R z0, z1;
    M::normal_pair(w, &z0, &z1);
    x = avg + sqrt(avg) * z0;
  } else {
    R lam = avg > R(0) ? avg : R(0);
    R u = M::uni(w, 0);
    R pk = M::exp(-lam);
    R F = pk;
    int k = 0;
    while (u >= F && k < 200) {
      k += 1;
      pk = pk * lam / R(k);
      F = F + pk;
    }
    x = R(k);
  }
  x = rint(x);
  return x > R(0) ? int(x) : 0;
}


// count[4 * i + s]: photons of step i on SiPM s (masked channels 0 when `masked`)
template <typename R>
__global__ void k_photon_count(CrvParams p, CrvEvents ev, CrvSteps st, CrvBars bars, CrvChannels ch,
                               const int32_t* __restrict__ step_event, long long nsteps,
                               const long long* __restrict__ nsteps_dev, int masked, int32_t* __restrict__ count,
                               Status* status) {
  nsteps = bounded_count(nsteps, nsteps_dev);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nsteps;
       i += (long long)gridDim.x * blockDim.x) {
    int e = step_event[i];
    int sie = int(i - ev.first_step[e]);
    int b = st.bar[i];
    double t = step_real(st, st.t, i);
    if (!isfinite(t)) {
      for (int s = 0; s < 4; ++s) count[4 * i + s] = 0;
      continue;
    }
    int ax = bars.length_axis[b];
    double pos = step_real(st, ax == 0 ? st.x : (ax == 1 ? st.y : st.z), i);
    double z = pos - bars.center_l[b];
    double half = bars.half_l[b];
    R edep = R(step_real(st, st.edep, i));
    EvKey ek{ev.event[e], ev.subrun[e], ev.run[e]};
    for (int s = 0; s < 4; ++s) {
      int c = b * 4 + s;
      int n = 0;
      if (!masked || (ch.status[c] & 0b101) == 0) {
        R d = readout_distance(R(z), R(half), s);
        R avg = mean_photons<R>(p, edep, R(ch.yield_factor[c]), d);
        U4 w = keyed(p.seed, ek, w2_of(ST_COUNT, 0, 0, 0, uint32_t(c)), uint32_t(sie));
        n = draw_count<R>(avg, w);
        if (n > 65536) { set_flag(status, CRV_ST_LIMIT); n = 65536; }
      }
      count[4 * i + s] = n;
    }
  }
}

#ifdef CRV_ENGINE_TU
// per SiPM of the table: photons on it, slot capacity for its charges, photon-id base (event's first step row)
__global__ void k_sipm_sizes(const long long* __restrict__ nsipm_dev, const int32_t* __restrict__ s_event, const int32_t* __restrict__ s_chan,
                             const long long* __restrict__ s_seg, const int32_t* __restrict__ s_nseg,
                             const int32_t* __restrict__ step_order, const int32_t* __restrict__ count,
                             CrvEvents ev, int charge_factor, int32_t* __restrict__ nphot,
                             int32_t* __restrict__ slot_cap, long long* __restrict__ id_base,
                             long long* __restrict__ label, uint32_t* __restrict__ run) {
  long long nsipm = *nsipm_dev;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nsipm;
       g += (long long)gridDim.x * blockDim.x) {
    int s = s_chan[g] & 3;
    long long a = s_seg[g];
    int n = 0;
    for (int k = 0; k < s_nseg[g]; ++k) n += count[4 * (long long)step_order[a + k] + s];
    nphot[g] = n;
    slot_cap[g] = n > 0 ? charge_factor * n + 16 : 0;
    int e = s_event[g];
    id_base[g] = ev.first_step[e];
    long long evkey = ((long long)ev.subrun[e] << 20) | (long long)ev.event[e];
    label[g] = evkey * 32768 + s_chan[g];
    run[g] = ev.run[e];
  }
}

#endif  // CRV_ENGINE_TU

// Emission delays, in decay times, of photons c0 + lane of a row of n photons (c0 a multiple of 32; every lane of the
// warp calls it): the order statistics of n exponential delays by the Renyi representation, S_j = sum_{i <= j} X_i /
// (n - i) with X_i = -log u_i and u_i photon i's keyed uniform.  The delays have the distribution of n independent
// exponential delays; photon j (key j) takes the j-th smallest, so every row's photons come out in time order.  Sums:
// an inclusive Hillis-Steele scan over the chunk's lanes (offsets 1, 2, 4, 8, 16), the earlier chunks' total (*carry,
// updated) in front; the CPU oracle adds in the same order, so FP64 sums are identical.
template <typename R>
__device__ __forceinline__ R row_delay_chunk(uint32_t seed, const EvKey& ek, uint32_t chan, uint32_t sie, int n, int c0,
                                             R* carry) {
  using M = Math<R>;
  const int j = c0 + lane_id();
  R v = R(0);
  if (j < n) {
    U4 w = keyed(seed, ek, w2_of(ST_PHOTON, 0, 0, 0, chan), (sie << 16) | uint32_t(j >> 1));
    v = (-M::log(M::uni_open(w, j & 1))) / R(n - j);
  }
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const R y = __shfl_up_sync(0xffffffffu, v, off);
    if (lane_id() >= off) v = v + y;
  }
  const R S = *carry + v;
  *carry = *carry + __shfl_sync(0xffffffffu, v, 31);
  return S;
}

// photons of each SiPM, contiguous from ph_off[g]: (time, key = step-in-event << 16 | photon)
template <typename R>
__global__ void k_photon_emit(CrvParams p, CrvEvents ev, CrvSteps st, CrvBars bars, long long nsipm,
                              const int32_t* __restrict__ s_event, const int32_t* __restrict__ s_chan,
                              const long long* __restrict__ s_seg, const int32_t* __restrict__ s_nseg,
                              const int32_t* __restrict__ step_order, const int32_t* __restrict__ count,
                              const long long* __restrict__ ph_off, R* __restrict__ ph_t,
                              uint32_t* __restrict__ ph_key) {
  long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long g = blockIdx.x * (long long)(blockDim.x >> 5) + warp_in_block(); g < nsipm; g += warps) {
    int c = s_chan[g], s = c & 3, e = s_event[g];
    EvKey ek{ev.event[e], ev.subrun[e], ev.run[e]};
    long long f = ev.first_step[e];
    long long o = ph_off[g];
    for (int k = 0; k < s_nseg[g]; ++k) {
      long long i = step_order[s_seg[g] + k];
      int n = count[4 * i + s];
      if (n == 0) continue;
      uint32_t sie = uint32_t(i - f);
      int b = st.bar[i];
      int ax = bars.length_axis[b];
      double z = step_real(st, ax == 0 ? st.x : (ax == 1 ? st.y : st.z), i) - bars.center_l[b];
      R d = readout_distance(R(z), R(bars.half_l[b]), s);
      R t = R(step_real(st, st.t, i));
      R dt = d / R(p.signal_speed);
      R carry = R(0);
      for (int c0 = 0; c0 < n; c0 += 32) {
        const R S = row_delay_chunk<R>(p.seed, ek, uint32_t(c), sie, n, c0, &carry);
        const int j = c0 + lane_id();
        if (j < n) {
          ph_t[o + j] = t + dt + R(p.decay_time) * S;
          ph_key[o + j] = (sie << 16) | uint32_t(j);
        }
      }
      o += n;
    }
  }
}

// ---------------------------------------------------------------------------------------------------------------------
// SiPM simulation: one warp per SiPM

// scheduled afterpulses per SiPM: a SiPM of at most 256 photons fires at most a few hundred pixels, with trap-0
// probabilities of a few percent; beyond the queue the SiPM reports CRV_ST_LIMIT
__host__ __device__ constexpr int sipm_tcap(int cap) { return cap <= 256 ? 32 : 128; }
constexpr int SIPM_WARPS = 8;    // warps per block

struct SipmGroups {
  const long long* n;            // device: number of groups
  const long long* guard[2];     // device totals that must not exceed guard_cap (else the pass is skipped)
  long long guard_cap[2];
  const long long* start;        // first photon row of the group
  const int32_t* count;          // photons in the group
  const long long* label;        // SiPM label
  const uint32_t* run;
  const uint32_t* key32;         // draw key per photon (chain) ...
  const long long* key64;        // ... or per photon as int64 (stage API); neither: the photon's index in its SiPM
  const long long* photon_id;    // photon id per photon (stage API), or null: id = id_base[g] + (key >> 16)
  const long long* id_base;
  const long long* slot_off;     // output slot region of the group
  const int32_t* slot_cap;
};

struct SipmOut {
  double* t;
  double* v;
  long long* id;
  int32_t* nmain;                // charges from photons and cascades (time order)
  int32_t* nap;                  // afterpulse charges (time order), stored after the main ones
  int32_t* fired;                // pixels that fired at least once
};

template <typename R>
struct SipmShared {
  R* ph_t;
  uint32_t* ph_key;
  uint32_t* ph_loc;
  R* last;
  uint32_t* bm;
  R* tr_t;
  R* tr_uf;
  long long* tr_id;
  uint16_t* tr_pix;
  uint16_t* fr_pix;
  uint16_t* fr_m;
  uint16_t* cand;
  int* misc;                     // [0] n candidates
  int tcap;                      // afterpulse queue length
};

// loc: the photons' positions in the group are kept (ph_loc), for per-photon ids (photon_id); without them a warp
// needs 4 bytes less per photon and more warps fit an SM
template <typename R>
__host__ __device__ inline size_t sipm_smem_per_warp(int cap, bool loc = true) {
  size_t b = 0;
  b += size_t(cap) * (sizeof(R) + (loc ? 8 : 4));   // ph_t, ph_key, ph_loc
  b += NPS_ALLOC * sizeof(R);                  // last
  b += 64 * 4;                                 // bm (53 used)
  b += size_t(sipm_tcap(cap)) * (2 * sizeof(R) + 8 + 2);   // traps
  b += 64 * 2 + 64 * 2 + 256 * 2 + 16;         // frontier, candidates, misc
  return (b + 15) & ~size_t(15);
}

template <typename R>
__device__ SipmShared<R> carve(char* base, int cap, bool loc) {
  SipmShared<R> S;
  char* q = base;
  S.last = reinterpret_cast<R*>(q); q += NPS_ALLOC * sizeof(R);
  S.ph_t = reinterpret_cast<R*>(q); q += size_t(cap) * sizeof(R);
  const int tcap = sipm_tcap(cap);
  S.tcap = tcap;
  S.tr_t = reinterpret_cast<R*>(q); q += tcap * sizeof(R);
  S.tr_uf = reinterpret_cast<R*>(q); q += tcap * sizeof(R);
  S.tr_id = reinterpret_cast<long long*>(q); q += tcap * 8;
  S.ph_key = reinterpret_cast<uint32_t*>(q); q += size_t(cap) * 4;
  S.ph_loc = loc ? reinterpret_cast<uint32_t*>(q) : nullptr;
  if (loc) q += size_t(cap) * 4;
  S.bm = reinterpret_cast<uint32_t*>(q); q += 64 * 4;
  S.misc = reinterpret_cast<int*>(q); q += 16;
  S.tr_pix = reinterpret_cast<uint16_t*>(q); q += tcap * 2;
  S.fr_pix = reinterpret_cast<uint16_t*>(q); q += 64 * 2;
  S.fr_m = reinterpret_cast<uint16_t*>(q); q += 64 * 2;
  S.cand = reinterpret_cast<uint16_t*>(q); q += 256 * 2;
  return S;
}

__device__ __forceinline__ bool bm_test(const uint32_t* bm, int p) { return (bm[p >> 5] >> (p & 31)) & 1u; }
__device__ __forceinline__ void bm_set(uint32_t* bm, int p) { atomicOr(&bm[p >> 5], 1u << (p & 31)); }

// Photon-map bin by the CDF (GetRandom2), then the pixel id of the point: "truncate" keeps the bin, "lrint" rounds
// the point, i.e. moves to the next pixel in x and in y each with probability 1/2 (crv/crvfastsim/response/sipm.py:
// 80-91).  The two halves are bits 0 and 1 of the draw word whose low bits the bin uniform does not use.
template <typename R>
__device__ __forceinline__ int draw_pixel(const CrvParams& p, const CrvPixels& px, const uint32_t* dead, R u,
                                          uint32_t half) {
  int b;
  if (p.uniform_map) {
    b = int(floor(u * R(NPX)));
  } else {
    double v = double(u) * px.cum[NPX - 1];
    int lo = 0, hi = NPX;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (px.cum[mid] <= v) lo = mid + 1; else hi = mid;
    }
    b = lo;
  }
  if (b > NPX - 1) b = NPX - 1;
  if (b < 0) b = 0;
  int x = b / 40, y = b - 40 * (b / 40);
  if (p.pixel_lrint) { x += int(half & 1u); y += int((half >> 1) & 1u); }
  const int q = x * PXS + y;
  return ((dead[q >> 5] >> (q & 31)) & 1u) ? -1 : q;
}

// SiPM constants in the compute type, converted once per block (held in shared memory: in the FP32 kernels a
// conversion from the FP64 parameters inside the per-photon code would issue on the narrow FP64 pipe every time)
template <typename R>
struct SipmK {
  R vov, tau, p1, p2, q_ct, q_t0, q_t1, life0, life1, t_end;
  float t_end_dn;                // largest float <= t_end: float times compare with it exactly as with t_end
  int ct_on, t0_on, t1_on, npx, npy;
};

template <typename R>
__device__ __forceinline__ SipmK<R> sipm_consts(const CrvParams& p) {
  SipmK<R> K;
  K.vov = R(p.overvoltage); K.tau = R(p.time_constant); K.p1 = R(p.p1); K.p2 = R(p.p2);
  K.q_ct = R(p.q_ct); K.q_t0 = R(p.q_t0); K.q_t1 = R(p.q_t1);
  K.life0 = R(p.trap0_lifetime); K.life1 = R(p.trap1_lifetime); K.t_end = R(p.t_end);
  K.t_end_dn = __double2float_rd(p.t_end);
  K.ct_on = p.q_ct > 0.0; K.t0_on = p.q_t0 > 0.0; K.t1_on = p.q_t1 > 0.0;
  K.npx = p.n_pixels_x; K.npy = p.n_pixels_y;
  return K;
}

// recovered overvoltage of pixel q at time t (Vov if it never fired)
template <typename R>
__device__ __forceinline__ R recovered(const SipmK<R>& K, const SipmShared<R>& S, int q, R t) {
  using M = Math<R>;
  if (!bm_test(S.bm, q)) return K.vov;
  return K.vov * (R(1) - M::exp(-(t - S.last[q]) / K.tau));
}

template <typename R>
__device__ __forceinline__ R pfire(const SipmK<R>& K, R v) {
  using M = Math<R>;
  return K.p1 * (R(1) - M::exp(-v / K.p2));
}

// probability that a node hit m times fires: 1 - (1 - pfire)^m
template <typename R>
__device__ __forceinline__ R pfire_m(const SipmK<R>& K, R v, int m) {
  R q = R(1) - pfire<R>(K, v);
  R qm = q;
  for (int i = 1; i < m; ++i) qm = qm * q;
  return R(1) - qm;
}

// Per SiPM context while simulating.
struct SipmCtx {
  EvKey ek;
  uint32_t chan;
  long long slot;          // first output slot
  int cap;                 // output slots
  int nq;                  // main records so far (may exceed cap: counting only)
  int ntr;                 // scheduled afterpulses
  int limit;               // a key/capacity limit was hit
};

// Schedule the afterpulses of a fired node (trap0: call 1 (u, u_time), call 4 word 0-1 (u_fire);
// trap1: call 4 word 2-3 (u), call 5 (u_time, u_fire)).  Returns how many were scheduled into (t, uf).
template <typename R>
__device__ __forceinline__ int node_traps(const CrvParams& p, const SipmK<R>& K, const SipmCtx& C, uint32_t gen,
                                          uint32_t idx, uint32_t key, R t, R* tt, R* uf) {
  using M = Math<R>;
  if (!K.t0_on && !K.t1_on) return 0;
  U4 a = keyed(p.seed, C.ek, w2_of(ST_SIPM, gen, idx, 1, C.chan), key);
  const bool trap0 = K.t0_on && M::uni(a, 0) < K.q_t0;
  if (!trap0 && !K.t1_on) return 0;              // call 4 is only read by a trap-0 afterpulse or the trap-1 draw
  U4 b = keyed(p.seed, C.ek, w2_of(ST_SIPM, gen, idx, 4, C.chan), key);
  int n = 0;
  if (trap0) {
    tt[n] = t - K.life0 * M::log(M::uni_open(a, 1));
    uf[n] = M::uni(b, 0);
    ++n;
  }
  if (K.t1_on && M::uni(b, 1) < K.q_t1) {
    U4 c = keyed(p.seed, C.ek, w2_of(ST_SIPM, gen, idx, 5, C.chan), key);
    tt[n] = t - K.life1 * M::log(M::uni_open(c, 0));
    uf[n] = M::uni(c, 1);
    ++n;
  }
  return n;
}

// cross-talk candidates of a fired node: bit q set for neighbour q (x-1, x+1, y-1, y+1) when it is drawn
template <typename R>
__device__ __forceinline__ unsigned node_crosstalk(const CrvParams& p, const SipmK<R>& K, const SipmCtx& C,
                                                   uint32_t gen, uint32_t idx, uint32_t key, int pix) {
  using M = Math<R>;
  if (!K.ct_on) return 0;
  U4 a = keyed(p.seed, C.ek, w2_of(ST_SIPM, gen, idx, 2, C.chan), key);
  U4 b = keyed(p.seed, C.ek, w2_of(ST_SIPM, gen, idx, 3, C.chan), key);
  int x = pix / PXS, y = pix - PXS * (pix / PXS);
  const R q = K.q_ct;
  unsigned m = 0;
  if (x > 0 && M::uni(a, 0) < q) m |= 1u;
  if (x + 1 < K.npx && M::uni(a, 1) < q) m |= 2u;
  if (y > 0 && M::uni(b, 0) < q) m |= 4u;
  if (y + 1 < K.npy && M::uni(b, 1) < q) m |= 8u;
  return m;
}

__device__ __forceinline__ int neighbour(int pix, int q) {
  return q == 0 ? pix - PXS : (q == 1 ? pix + PXS : (q == 2 ? pix - 1 : pix + 1));
}

// Append a charge record (lane-ordered position pos relative to C.nq) if it fits.
// widening to the FP64 output columns (FP32: by integer bit arithmetic, off the FP64 pipe)
__device__ __forceinline__ double widen(double x) { return x; }
__device__ __forceinline__ double widen(float x) { return f2d(x); }

template <typename R>
__device__ __forceinline__ void put_charge(const SipmOut& O, const SipmCtx& C, int pos, R t, R v, long long id) {
  int k = C.nq + pos;
  if (k < C.cap) {
    long long o = C.slot + k;
    O.t[o] = widen(t);
    O.v[o] = widen(v);
    O.id[o] = id;
  }
}

// Build the next frontier from the candidate list (lane 0): sort, unique with multiplicity, drop dead.
template <typename R>
__device__ __forceinline__ int make_frontier(const SipmShared<R>& S, int nc, const uint32_t* dead, int* limit) {
  int nf = 0;
  if (lane_id() == 0) {
    for (int a = 1; a < nc; ++a) {           // insertion sort (tiny lists)
      uint16_t x = S.cand[a];
      int b = a - 1;
      while (b >= 0 && S.cand[b] > x) { S.cand[b + 1] = S.cand[b]; --b; }
      S.cand[b + 1] = x;
    }
    for (int a = 0; a < nc;) {
      int b = a;
      while (b < nc && S.cand[b] == S.cand[a]) ++b;
      int q = S.cand[a];
      if (!((dead[q >> 5] >> (q & 31)) & 1u)) {
        if (nf > MAX_IDX) { *limit = 1; break; }
        S.fr_pix[nf] = uint16_t(q);
        S.fr_m[nf] = uint16_t(b - a);
        ++nf;
      }
      a = b;
    }
    S.misc[1] = nf;
  }
  __syncwarp();
  nf = S.misc[1];
  __syncwarp();
  return nf;
}

// Cross-talk cascade of one fired primary (generation 1 onwards), frontier spread over the lanes.
template <typename R>
__device__ void run_cascade(const CrvParams& p, const SipmK<R>& K, const SipmShared<R>& S, const uint32_t* dead,
                            SipmCtx& C, const SipmOut& O, unsigned cand0, int pix0, R t, uint32_t key, long long id) {
  // generation-1 candidates from the primary
  int nc = 0;
  if (lane_id() == 0) {
    for (int q = 0; q < 4; ++q)
      if (cand0 & (1u << q)) S.cand[nc++] = uint16_t(neighbour(pix0, q));
  }
  nc = __shfl_sync(FULL, nc, 0);
  __syncwarp();
  int lim = 0;
  int nf = make_frontier<R>(S, nc, dead, &lim);
  lim = __shfl_sync(FULL, lim, 0);
  if (lim) nf = 0;
  uint32_t gen = 1;
  while (nf > 0) {
    if (gen > MAX_GEN) { lim = 1; break; }
    int ncand = 0;
    for (int base = 0; base < nf; base += 32) {
      int i = base + lane_id();
      bool act = i < nf;
      int q = act ? S.fr_pix[i] : 0;
      R v = R(0);
      bool fire = false;
      if (act) {
        v = recovered<R>(K, S, q, t);
        R pm = pfire_m<R>(K, v, S.fr_m[i]);
        U4 w = keyed(p.seed, C.ek, w2_of(ST_SIPM, gen, uint32_t(i), 0, C.chan), key);
        fire = Math<R>::uni(w, 1) < pm;
      }
      unsigned fm = __ballot_sync(FULL, fire);
      int pos = __popc(fm & lanemask_lt());
      R tt[2], uf[2];
      int ntr = 0;
      unsigned ct = 0;
      if (fire) {
        put_charge<R>(O, C, pos, t, v, id);
        S.last[q] = t;
        bm_set(S.bm, q);
        ntr = node_traps<R>(p, K, C, gen, uint32_t(i), key, t, tt, uf);
        ct = node_crosstalk<R>(p, K, C, gen, uint32_t(i), key, q);
      }
      C.nq += __popc(fm);
      // traps in node order
      int tot;
      int tpos = warp_excl(ntr, &tot);
      for (int a = 0; a < ntr; ++a) {
        int k = C.ntr + tpos + a;
        if (k < S.tcap) { S.tr_t[k] = tt[a]; S.tr_uf[k] = uf[a]; S.tr_pix[k] = uint16_t(q); S.tr_id[k] = id; }
      }
      C.ntr += tot;
      // candidates
      int nct = __popc(ct);
      int cpos = warp_excl(nct, &tot);
      int a = 0;
      for (int qq = 0; qq < 4; ++qq)
        if (ct & (1u << qq)) {
          int k = ncand + cpos + a++;
          if (k < 256) S.cand[k] = uint16_t(neighbour(q, qq));
        }
      ncand += tot;
      __syncwarp();
    }
    if (ncand > 256) { lim = 1; break; }
    ++gen;
    nf = make_frontier<R>(S, ncand, dead, &lim);
    lim = __shfl_sync(FULL, lim, 0);
    if (lim) break;
  }
  if (__any_sync(FULL, lim)) C.limit = 1;
}

// Serial-semantics simulation of one SiPM whose sorted photons (n <= cap) sit in S.ph_*.
template <typename R>
__device__ void simulate_sipm(const CrvParams& p, const SipmK<R>& K, const CrvPixels& px, const SipmShared<R>& S,
                              const uint32_t* dead, SipmCtx& C, const SipmOut& O, int n, const long long* photon_id,
                              long long gstart, long long id_base) {
  using M = Math<R>;
  for (int w = lane_id(); w < 64; w += 32) S.bm[w] = 0u;
  __syncwarp();
  int k = 0;
  while (k < n) {
    int i = k + lane_id();
    bool has = i < n;
    R t = has ? S.ph_t[i] : R(0);
    uint32_t key = has ? S.ph_key[i] : 0u;
    int pix = -1;
    U4 w0{0, 0, 0, 0};
    if (has) {
      w0 = keyed(p.seed, C.ek, w2_of(ST_SIPM, 0, 0, 0, C.chan), key);
      pix = draw_pixel<R>(p, px, dead, M::uni(w0, 0), w0.y);
    }
    bool live = pix >= 0;
    unsigned same = __match_any_sync(FULL, live ? pix : -1 - lane_id());
    bool collide = live && (same & lanemask_lt()) != 0u;
    bool fire = false;
    unsigned ct = 0;
    R v = R(0);
    if (live && !collide) {
      v = recovered<R>(K, S, pix, t);
      R pm = pfire_m<R>(K, v, 1);
      fire = M::uni(w0, 1) < pm;
      if (fire) ct = node_crosstalk<R>(p, K, C, 0, 0, key, pix);
    }
    int nv = min(n - k, 32);
    unsigned cm = __ballot_sync(FULL, collide);
    unsigned sm = __ballot_sync(FULL, ct != 0u);
    int f = cm ? __ffs(cm) - 1 : 32;
    int g = sm ? __ffs(sm) - 1 : 32;
    int ncommit = (g < f) ? g + 1 : min(f, nv);
    bool commit = lane_id() < ncommit && fire;
    long long id = 0;
    if (commit) id = photon_id ? photon_id[gstart + S.ph_loc[i]] : id_base + (long long)(key >> 16);
    unsigned fm = __ballot_sync(FULL, commit);
    R tt[2], uf[2];
    int ntr = 0;
    if (commit) {
      put_charge<R>(O, C, __popc(fm & lanemask_lt()), t, v, id);
      S.last[pix] = t;
      bm_set(S.bm, pix);
      ntr = node_traps<R>(p, K, C, 0, 0, key, t, tt, uf);
    }
    C.nq += __popc(fm);
    int tot;
    int tpos = warp_excl(ntr, &tot);
    for (int a = 0; a < ntr; ++a) {
      int kk = C.ntr + tpos + a;
      if (kk < S.tcap) { S.tr_t[kk] = tt[a]; S.tr_uf[kk] = uf[a]; S.tr_pix[kk] = uint16_t(pix); S.tr_id[kk] = id; }
    }
    C.ntr += tot;
    __syncwarp();
    if (g < f) {
      unsigned c0 = __shfl_sync(FULL, ct, g);
      int p0 = __shfl_sync(FULL, pix, g);
      R tg = __shfl_sync(FULL, t, g);
      uint32_t kg = __shfl_sync(FULL, key, g);
      long long idg = __shfl_sync(FULL, id, g);
      run_cascade<R>(p, K, S, dead, C, O, c0, p0, tg, kg, idg);
    }
    k += ncommit;
  }
  if (C.ntr > S.tcap) C.limit = 1;
}

// Afterpulses after all photons, in (time, schedule order); stored after the main records.  Returns the count.
template <typename R>
__device__ int run_afterpulses(const SipmK<R>& K, const SipmShared<R>& S, SipmCtx& C, const SipmOut& O) {
  int ntr = min(C.ntr, S.tcap);
  int nap = 0;
  if (lane_id() == 0 && ntr > 0) {
    // insertion sort by time (stable: equal times keep schedule order)
    for (int a = 1; a < ntr; ++a) {
      R x = S.tr_t[a], xu = S.tr_uf[a];
      uint16_t xp = S.tr_pix[a];
      long long xi = S.tr_id[a];
      int b = a - 1;
      while (b >= 0 && S.tr_t[b] > x) {
        S.tr_t[b + 1] = S.tr_t[b]; S.tr_uf[b + 1] = S.tr_uf[b]; S.tr_pix[b + 1] = S.tr_pix[b];
        S.tr_id[b + 1] = S.tr_id[b];
        --b;
      }
      S.tr_t[b + 1] = x; S.tr_uf[b + 1] = xu; S.tr_pix[b + 1] = xp; S.tr_id[b + 1] = xi;
    }
    for (int a = 0; a < ntr; ++a) {
      R t1 = S.tr_t[a];
      if (t1 > K.t_end) continue;
      int q = S.tr_pix[a];
      R v = recovered<R>(K, S, q, t1);
      if (S.tr_uf[a] < pfire<R>(K, v)) {
        S.last[q] = t1;
        S.bm[q >> 5] |= 1u << (q & 31);
        long long id = S.tr_id[a];
        int kk = C.nq + nap;
        if (kk < C.cap) {
          long long o = C.slot + kk;
          O.t[o] = widen(t1);
          O.v[o] = widen(v);
          O.id[o] = id;
        }
        ++nap;
      }
    }
  }
  nap = __shfl_sync(FULL, nap, 0);
  __syncwarp();
  return nap;
}

// Order-preserving integer image of an FP64 time, -0 taken as +0 (as the numeric comparison does): FP64 sort
// comparisons on the integer pipe instead of the FP64 pipe.
__device__ __forceinline__ unsigned long long ord_time(double t) {
  unsigned long long u = (unsigned long long)__double_as_longlong(t);
  if (u == 0x8000000000000000ull) u = 0ull;
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// (ta, ka) > (tb, kb) in (time, key) order
__device__ __forceinline__ bool after(float ta, uint32_t ka, float tb, uint32_t kb) {
  return (ta > tb) || (ta == tb && ka > kb);
}
__device__ __forceinline__ bool after(double ta, uint32_t ka, double tb, uint32_t kb) {
  const unsigned long long a = ord_time(ta), b = ord_time(tb);
  return (a > b) || (a == b && ka > kb);
}

// sort the staged photons by (time, key) (warp bitonic over the next power of two)
template <typename R>
__device__ void sort_photons(const SipmShared<R>& S, int n) {
  int P = 1;
  while (P < n) P <<= 1;
  for (int i = n + lane_id(); i < P; i += 32) {
    S.ph_t[i] = R(INFINITY);
    S.ph_key[i] = 0xFFFFFFFFu;
    if (S.ph_loc) S.ph_loc[i] = 0xFFFFFFFFu;
  }
  __syncwarp();
  for (int size = 2; size <= P; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int q = lane_id(); q < (P >> 1); q += 32) {
        const int lo = ((q & ~(stride - 1)) << 1) | (q & (stride - 1));   // stride is a power of two
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const R ta = S.ph_t[lo], tb = S.ph_t[hi];
        const uint32_t ka = S.ph_key[lo], kb = S.ph_key[hi];
        if (after(ta, ka, tb, kb) == up) {
          S.ph_t[lo] = tb; S.ph_t[hi] = ta;
          S.ph_key[lo] = kb; S.ph_key[hi] = ka;
          if (S.ph_loc) {
            uint32_t la = S.ph_loc[lo];
            S.ph_loc[lo] = S.ph_loc[hi]; S.ph_loc[hi] = la;
          }
        }
      }
      __syncwarp();
    }
  }
}

// SiPM stage over photon groups (PT: storage type of the photon times)
template <typename R, typename PT>
__global__ void __launch_bounds__(512) k_sipm_sim(CrvParams p, CrvPixels px, SipmGroups G,
                                                 const PT* __restrict__ ph_time, int lo, int cap, int last_pass,
                                                 SipmOut O, Status* status) {
  extern __shared__ __align__(16) char smem[];
  __shared__ uint32_t dead[64];
  __shared__ SipmK<R> K;
  for (int i = threadIdx.x; i < 64; i += blockDim.x) dead[i] = i < DEAD_WORDS ? px.dead_bits[i] : 0u;
  if (threadIdx.x == 0) K = sipm_consts<R>(p);
  __syncthreads();
  const bool loc = G.photon_id != nullptr;
  SipmShared<R> S = carve<R>(smem + size_t(warp_in_block()) * sipm_smem_per_warp<R>(cap, loc), cap, loc);
  for (int q = 0; q < 2; ++q)
    if (G.guard[q] && *G.guard[q] > G.guard_cap[q]) return;
  const long long ngroups = *G.n;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  // groups in tiles of 32 per warp: one coalesced load of their counts and a ballot pick the groups of this pass (a
  // later pass, which holds few groups, does not walk every group with a dependent load)
  for (long long g0 = (blockIdx.x * (long long)(blockDim.x >> 5) + warp_in_block()) * 32; g0 < ngroups;
       g0 += warps * 32) {
   const long long gl = g0 + lane_id();
   const int cl = gl < ngroups ? G.count[gl] : 0;
   unsigned todo = __ballot_sync(FULL, gl < ngroups && cl > lo);
   while (todo) {
    const int bsel = __ffs(todo) - 1;
    todo &= todo - 1;
    const long long g = g0 + bsel;
    const int cnt = __shfl_sync(FULL, cl, bsel);
    long long a = G.start[g];
    long long lab = G.label[g];
    SipmCtx C;
    long long evk = lab / 32768;
    C.ek = EvKey{uint32_t(evk & 0xFFFFF), uint32_t(evk >> 20), G.run[g]};
    C.chan = uint32_t(lab % 32768);
    C.slot = G.slot_off[g];
    C.cap = G.slot_cap[g];
    C.nq = 0;
    C.ntr = 0;
    C.limit = 0;
    if (cnt > cap) {
      if (lane_id() == 0 && last_pass) {
        set_flag(status, CRV_ST_CAPACITY);
        need_at_least(status, CRV_NEED_PHOTONS_PER_SIPM, cnt);
        O.nmain[g] = 0; O.nap[g] = 0; O.fired[g] = 0;
      }
      continue;
    }
    // stage photons with t <= t_end, four chunks of 32 per step (their loads in flight together)
    int n = 0;
    for (int base = 0; base < cnt; base += 128) {
      PT tv[4];
      uint32_t kv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = base + 32 * u + lane_id();
        tv[u] = i < cnt ? ph_time[a + i] : PT(0);
        kv[u] = i < cnt ? (G.key32 ? G.key32[a + i] : G.key64 ? uint32_t(G.key64[a + i]) : uint32_t(i)) : 0u;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = base + 32 * u + lane_id();
        bool keep;
        if constexpr (sizeof(PT) == 4) keep = i < cnt && (float(tv[u]) <= K.t_end_dn);
        else keep = i < cnt && (double(tv[u]) <= p.t_end);
        const unsigned km = __ballot_sync(FULL, keep);
        if (keep) {
          const int o = n + __popc(km & lanemask_lt());
          S.ph_t[o] = R(tv[u]);
          S.ph_key[o] = kv[u];
          if (loc) S.ph_loc[o] = uint32_t(i);
        }
        n += __popc(km);
      }
    }
    __syncwarp();
    // the photons of one (step, SiPM) row come out of the photon stage in (time, key) order, so a SiPM hit by one
    // step needs no sort: check the order, sort only when it is broken
    bool ordered = true;
    for (int i = lane_id(); i + 1 < n; i += 32)
      ordered = ordered && !after(S.ph_t[i], S.ph_key[i], S.ph_t[i + 1], S.ph_key[i + 1]);
    if (!__all_sync(FULL, ordered)) sort_photons<R>(S, n);
    const long long idb = G.id_base ? G.id_base[g] : 0;
    simulate_sipm<R>(p, K, px, S, dead, C, O, n, G.photon_id, a, idb);
    int nap = run_afterpulses<R>(K, S, C, O);
    int fired = 0;
    for (int w = lane_id(); w < DEAD_WORDS; w += 32) fired += __popc(S.bm[w]);
    fired = warp_sum(fired);
    if (lane_id() == 0) {
      O.nmain[g] = C.nq;
      O.nap[g] = nap;
      O.fired[g] = fired;
      if (C.nq + nap > C.cap) {
        set_flag(status, CRV_ST_CAPACITY);
        long long per = cnt > 0 ? (C.nq + nap - 16 + cnt - 1) / cnt : 1;
        need_at_least(status, CRV_NEED_CHARGE_FACTOR, per < 1 ? 1 : per);
      }
      if (C.limit) set_flag(status, CRV_ST_LIMIT);
    }
    __syncwarp();
   }
  }
}

#ifdef CRV_ENGINE_TU
// compaction: merge each group's main and afterpulse runs by time into the output at out_off[g]
__global__ void k_charge_compact(const long long* __restrict__ ngroups_dev, const long long* __restrict__ glabel,
                                 const long long* __restrict__ slot_off, const int32_t* __restrict__ slot_cap,
                                 const int32_t* __restrict__ nmain, const int32_t* __restrict__ nap,
                                 const long long* __restrict__ out_off, const double* __restrict__ st,
                                 const double* __restrict__ sv, const long long* __restrict__ sid, double capacitance,
                                 double overvoltage, int fp32, CrvCharges out, long long out_cap) {
  // out.pe and out.photon may be null (the resident chain reads label, time and charge only): not written
  // FP32-mixed: voltages are FP32 values; charge and PE in FP32 (no FP64 multiply and division per charge)
  const float cap_f = float(capacitance), inv_vov_f = 1.0f / float(overvoltage);
  long long ngroups = *ngroups_dev;
  long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  // groups in tiles of 32 per warp: one coalesced load of their sizes and offsets, then the non-empty ones in order
  for (long long g0 = (blockIdx.x * (long long)(blockDim.x >> 5) + warp_in_block()) * 32; g0 < ngroups;
       g0 += warps * 32) {
   const long long gl = g0 + lane_id();
   int nm_l = 0, na_l = 0;
   long long s0_l = 0, o0_l = 0, lab_l = 0;
   bool ok = false;
   if (gl < ngroups) {
     nm_l = nmain[gl];
     na_l = nap[gl];
     s0_l = slot_off[gl];
     o0_l = out_off[gl];
     lab_l = glabel[gl];
     // an overflowed group (reported through the status) or one beyond the output is not written
     ok = nm_l + na_l > 0 && nm_l + na_l <= slot_cap[gl] && o0_l + nm_l + na_l <= out_cap;
   }
   unsigned todo = __ballot_sync(0xffffffffu, ok);
   while (todo) {
    const int bsel = __ffs(todo) - 1;
    todo &= todo - 1;
    const int nm = __shfl_sync(0xffffffffu, nm_l, bsel), na = __shfl_sync(0xffffffffu, na_l, bsel);
    const long long s0 = __shfl_sync(0xffffffffu, s0_l, bsel), o0 = __shfl_sync(0xffffffffu, o0_l, bsel);
    const long long lab = __shfl_sync(0xffffffffu, lab_l, bsel);
    // rank of each record in the merged order: main i -> i + #(ap with t < t_main_i);
    // ap j -> j + #(main with t <= t_ap_j)
    for (int i = lane_id(); i < nm + na; i += 32) {
      long long src = s0 + i;
      double t = st[src];
      int r;
      if (i < nm) {
        int c = 0;
        for (int j = 0; j < na; ++j) c += st[s0 + nm + j] < t;
        r = i + c;
      } else {
        int lo = 0, hi = nm;       // main records are time ordered: count main with t_main <= t
        while (lo < hi) {
          int mid = (lo + hi) >> 1;
          if (st[s0 + mid] <= t) lo = mid + 1; else hi = mid;
        }
        r = (i - nm) + lo;
      }
      long long o = o0 + r;
      double v = sv[src];
      out.label[o] = lab;
      out.time[o] = t;
      if (fp32) {
        const float vf = d2f_trunc(v);
        out.charge[o] = f2d(cap_f * vf);
        if (out.pe) out.pe[o] = f2d(vf * inv_vov_f);
      } else {
        out.charge[o] = capacitance * v;
        if (out.pe) out.pe[o] = v / overvoltage;
      }
      if (out.photon) out.photon[o] = sid[src];
    }
   }
  }
}

__global__ void k_counts_total(const long long* __restrict__ n_dev, const int32_t* __restrict__ a,
                               const int32_t* __restrict__ b, int32_t* __restrict__ out) {
  long long n = *n_dev;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = a[i] + b[i];
}

#endif  // CRV_ENGINE_TU

}  // namespace crv
