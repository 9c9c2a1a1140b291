// Coincidence finder: reco pulses of each event -> coincidence clusters (crv/crvfastsim/reco/coinc.py:112-392,
// crv/crvfastsim/reco/coinc_cpu.py:11-51; per-event loop of crv/crvfastsim/chain.py:325-362).
//
// Per event and sector type (ascending): hits = first pulses (secondary pulses dropped) with the fibre-length time
// correction to the type's outermost readout end and PE doubled when the same-end partner SiPM has a compensated
// status bit; per readout side: filterHits (same + one adjacent counter in the layer, |dt| <= max_dt_adjacent, PE sum
// >= threshold, sums in list order), greedy single-linkage clustering in list order (|dx| <= max(maxd), |dt| < max_dt),
// the 2/3/4-layer combination check (time window, slope window and pairwise slope differences; passing combinations
// widen maxd to the gaps to their x-neighbours); then clustering of the coincidence hits of both sides (opposite sides
// get + 2 half-length / v), attachment of filtered first pulses on missing opposite counter ends, PE-weighted
// properties.
//
// GPU mapping: one warp per event; hits and work lists in shared memory; the O(H^2) filter, the link tests and the
// combination enumeration are spread over the lanes; list-order decisions (greedy joins, attachment order) are taken
// in order with ballots.  All arithmetic is FP64.
#pragma once
#include "crv_device.cuh"

namespace crv {

struct CoincGeom {
  const int32_t *bar_sector, *bar_layer, *bar_counter;
  const double *bar_x, *bar_y, *bar_pos;           // pos: [nbars][3]
  const int32_t *sec_type, *sec_cut, *sec_length_dir;
  const double *sec_pos0, *sec_pos1;
  const double* cuts;                              // [ncuts][10]
  const int32_t* type_id;                          // [ntypes], ascending
  const double *type_p0, *type_p1, *type_half, *type_maxdt;
  const int32_t *type_side0, *type_side1;
  int32_t ntypes;
  int32_t pad;
};

struct CoincIn {
  long long nev;                                   // events (an upper bound when nev_dev is set)
  const long long* nev_dev;                        // device count of events, or null
  const long long* ev_start;                       // first pulse row of event e
  const int32_t* ev_count;                         // pulses of event e
  const int32_t *bar, *sipm, *seq;
  const double *time, *pe;
  const int32_t* status;                           // per channel
};

struct ClusterRec {
  double pe, start, end, slope, avgtime, pos[3], sidepe[2], sidetime[2];
  int32_t type, sidehits[2], nlayers, poscalc, mem_begin, mem_count, pad;
};

struct CoincOut {
  ClusterRec* rec;                                 // slots: event e uses rows [ev_start[e], ev_start[e] + ev_count[e])
  int32_t* mem_idx;                                // member slots, same rows
  int32_t* ncl;                                    // clusters per event
  int32_t* nmem;                                   // members per event
};

enum { CUT_PE = 0, CUT_DTADJ, CUT_DT, CUT_SMIN, CUT_SMAX, CUT_SDIFF, CUT_LAYERS, CUT_MINPE, CUT_D0, CUT_D1 };

// Per-warp shared memory, per hit of the event (narrow types; y, sector and the initial maxd are read from the bar and
// cut tables when needed).
struct CoincShared {
  // hits of the event (all types)
  double *x, *t, *pe;
  unsigned long long* wid;                         // widened maxd (non-negative doubles as ordered integers)
  int32_t* idx;                                    // pulse row within the event
  uint16_t *bar, *counter;
  uint8_t *cut, *layer, *side, *sipm, *seq0, *type, *kept;   // seq0: first pulse of its waveform
  // work lists (indices into hits or into the coincidence list)
  int32_t *list, *clus, *filt, *coinc, *cl_of, *order, *tmp;
};

__host__ __device__ inline size_t coinc_smem_per_warp(int hcap) {
  return (size_t(hcap) * (4 * 8 + 8 * 4 + 2 * 2 + 7) + 64 + 15) & ~size_t(15);
}

__device__ inline CoincShared coinc_carve(char* b, int hcap) {
  CoincShared S;
  double* d = reinterpret_cast<double*>(b);
  S.x = d; S.t = d + hcap; S.pe = d + 2 * hcap;
  S.wid = reinterpret_cast<unsigned long long*>(d + 3 * hcap);
  int32_t* q = reinterpret_cast<int32_t*>(d + 4 * hcap);
  int32_t** f[] = {&S.idx, &S.list, &S.clus, &S.filt, &S.coinc, &S.cl_of, &S.order, &S.tmp};
  for (int k = 0; k < 8; ++k) *f[k] = q + k * hcap;
  uint16_t* h = reinterpret_cast<uint16_t*>(q + 8 * hcap);
  S.bar = h; S.counter = h + hcap;
  uint8_t* c = reinterpret_cast<uint8_t*>(h + 2 * hcap);
  uint8_t** g[] = {&S.cut, &S.layer, &S.side, &S.sipm, &S.seq0, &S.type, &S.kept};
  for (int k = 0; k < 7; ++k) *g[k] = c + k * hcap;
  return S;
}

__device__ __forceinline__ double cutv(const CoincGeom& G, int c, int k) { return G.cuts[c * 10 + k]; }

// int(v) (truncation) for |v| < 2^31, from the bits: integer instructions instead of an FP64 conversion
__device__ __forceinline__ int trunc_int(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int e = int((b >> 52) & 0x7FF) - 1023;
  if (e < 0) return 0;
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int r = int(m >> (52 - e));
  return (b >> 63) ? -r : r;
}

// link test of hit/copy a and b (maxd taken from ma, mb)
__device__ __forceinline__ bool linked(const CoincShared& S, int a, int b, double ma, double mb, double max_dt,
                                       bool opposite, double dt_opp) {
  double md = ma > mb ? ma : mb;
  double mt = max_dt + ((opposite && S.side[a] != S.side[b]) ? dt_opp : 0.0);
  return fabs(S.x[a] - S.x[b]) <= md && fabs(S.t[a] - S.t[b]) < mt;
}

// The same decision, with an FP32 rejection first: most pairs lie far apart in time, and a time difference that the
// FP32 copies (truncated: within 2^-23 relative of the FP64 times) put beyond the window by more than four times their
// rounding bound is beyond it in FP64 too, so only the pairs left go through the FP64 test.  tc: the FP32 copy of item
// a's time; mt_hi: an FP32 value at least the largest window the pair can have, less 2^-23 relative.
__device__ __forceinline__ bool linked_fast(const CoincShared& S, int a, float tc, int b, float tb, double ma,
                                            double mb, double max_dt, float mt_hi, bool opposite, double dt_opp) {
  const float d = fabsf(tc - tb);
  if (d > mt_hi + 4.8e-7f * (fabsf(tc) + fabsf(tb) + mt_hi)) return false;
  return linked(S, a, b, ma, mb, max_dt, opposite, dt_opp);
}

// Greedy clustering of items 0..n-1 in list order: item k is hit ids[k] with maxd mds[k].  Writes the cluster of
// every item into cl_of[k], the items grouped by cluster in join order into out[], and cluster starts into
// clstart[0..ncl].  Returns the number of clusters.
//
// The reference seeds a cluster with the first item left, then scans the remaining items in order, adding every
// item linked to a member (including members added earlier in the same scan), and repeats the scan until it adds
// nothing.  Here the scan goes over 32 items at a time, one per lane: each lane tests its item against the members;
// the lowest linked lane joins first, the lanes after it re-test against that new member, and so on, which is the
// sequential scan's order exactly.
//
// tfs (n floats of scratch): the items' FP32 times.  The cluster's FP32 time range [lo, hi] rejects, with one test, a
// candidate that linked_fast would reject against every member: its distance to the range exceeds linked_fast's bound
// for the largest member time magnitude in the range (the FP32 operations are monotone, so every member's own test
// would reject it too).
__device__ int greedy(const CoincShared& S, const int32_t* ids, const double* mds, int n, double max_dt, bool opposite,
                      double dt_opp, int32_t* cl_of, int32_t* out, int32_t* clstart, float* tfs) {
  const int lane = lane_id();
  for (int k = lane; k < n; k += 32) {
    cl_of[k] = -1;
    tfs[k] = d2f_trunc(S.t[ids[k]]);
  }
  __syncwarp();
  const float mt_hi = d2f_trunc(max_dt + (opposite ? fabs(dt_opp) : 0.0));
  int nout = 0, ncl = 0, first = 0;
  while (true) {
    int seed = -1;
    for (int base = first; base < n && seed < 0; base += 32) {
      const int k = base + lane;
      const unsigned m = __ballot_sync(0xffffffffu, k < n && cl_of[k] < 0);
      if (m) seed = base + __ffs(m) - 1;
    }
    if (seed < 0) break;
    first = seed + 1;
    __syncwarp();
    if (lane == 0) { out[nout] = seed; cl_of[seed] = ncl; clstart[ncl] = nout; }
    __syncwarp();
    const int c0 = nout;
    ++nout;
    float lo = tfs[seed], hi = lo;
    bool grew = true;
    while (grew) {
      grew = false;
      for (int base = first; base < n; base += 32) {
        const int k = base + lane;
        const bool cand = k < n && cl_of[k] < 0;
        int hc = 0;
        double mc = 0.0;
        float tc = 0.0f;
        bool link = false;
        if (cand) {
          hc = ids[k];
          mc = mds[k];
          tc = tfs[k];
          const float mg = mt_hi + 4.8e-7f * (fabsf(tc) + fmaxf(fabsf(lo), fabsf(hi)) + mt_hi);
          if (!(tc - hi > mg) && !(lo - tc > mg))
            for (int m = c0; m < nout && !link; ++m) {
              const int it = out[m];
              link = linked_fast(S, hc, tc, ids[it], tfs[it], mc, mds[it], max_dt, mt_hi, opposite, dt_opp);
            }
        }
        unsigned L = __ballot_sync(0xffffffffu, link);
        while (L) {
          const int b = __ffs(L) - 1;
          const int nk = base + b;
          __syncwarp();
          if (lane == 0) { out[nout] = nk; cl_of[nk] = ncl; }
          ++nout;
          grew = true;
          L &= L - 1u;
          const float tn = tfs[nk];
          lo = fminf(lo, tn);
          hi = fmaxf(hi, tn);
          bool t = false;
          if (cand && !link && lane > b) {
            t = linked_fast(S, hc, tc, ids[nk], tn, mc, mds[nk], max_dt, mt_hi, opposite, dt_opp);
            link = t;
          }
          L |= __ballot_sync(0xffffffffu, t);
        }
        __syncwarp();
      }
    }
    ++ncl;
  }
  __syncwarp();
  if (lane == 0) clstart[ncl] = nout;
  __syncwarp();
  return ncl;
}

// combination check of one cluster (members: hit ids in mem[0..m)); kept hits get kept=1 and wid widened.
__device__ void check_coincidence(const CoincGeom& G, const CoincShared& S, const int32_t* mem, int m,
                                  int big_threshold) {
  int cnt[4] = {0, 0, 0, 0};
  int nmin = 1 << 30, nmax = -1;
  for (int k = 0; k < m; ++k) {
    int h = mem[k];
    cnt[S.layer[h]]++;
    int cl = trunc_int(cutv(G, S.cut[h], CUT_LAYERS));
    nmin = cl < nmin ? cl : nmin;
    nmax = cl > nmax ? cl : nmax;
  }
  for (int k = lane_id(); k < m; k += 32) {
    int h = mem[k];
    S.wid[h] = (unsigned long long)__double_as_longlong(cutv(G, S.cut[h], CUT_D1));
    S.kept[h] = 0;
  }
  __syncwarp();
  int nonempty = (cnt[0] > 0) + (cnt[1] > 0) + (cnt[2] > 0) + (cnt[3] > 0);
  if (m > big_threshold && nonempty >= nmin) {
    for (int k = lane_id(); k < m; k += 32) S.kept[mem[k]] = 1;
    __syncwarp();
    return;
  }
  // a combination of nl layers needs nl non-empty layers, and is skipped unless one of its hits asks for at most nl
  // layers (nmin or more): with fewer non-empty layers than nmin no combination can keep a hit
  if (nonempty < nmin) return;
  // bucket lists: offsets
  int off[5] = {0, cnt[0], cnt[0] + cnt[1], cnt[0] + cnt[1] + cnt[2], m};
  if (lane_id() == 0) {
    int fill[4] = {off[0], off[1], off[2], off[3]};
    for (int k = 0; k < m; ++k) { int h = mem[k]; S.tmp[fill[S.layer[h]]++] = h; }
  }
  __syncwarp();
  for (int nl = 2; nl <= 4; ++nl) {
    bool need = (nl == 2 && nmin == 2) || (nl == 3 && nmin <= 3 && 3 <= nmax) || (nl == 4 && nmax == 4);
    if (!need) continue;
    for (int mask = 0; mask < 16; ++mask) {
      if (__popc(mask) != nl) continue;
      int ls[4], sz[4], k = 0;
      long long total = 1;
      for (int l = 0; l < 4; ++l)
        if (mask & (1 << l)) { ls[k] = l; sz[k] = cnt[l]; total *= cnt[l]; ++k; }
      if (total == 0) continue;
      for (long long c = lane_id(); c < total; c += 32) {
        int hs[4];
        long long r = c;
        for (int q = nl - 1; q >= 0; --q) {         // mixed radix, first layer slowest
          hs[q] = S.tmp[off[ls[q]] + int(r % sz[q])];
          r /= sz[q];
        }
        bool skip = true;
        for (int q = 0; q < nl; ++q) skip = skip && (cutv(G, S.cut[hs[q]], CUT_LAYERS) > nl);
        if (skip) continue;
        double mdt = -1e300, lo = 1e300, hi = -1e300, msd = -1e300, tmin = 1e300, tmax = -1e300;
        for (int q = 0; q < nl; ++q) {
          int c_ = S.cut[hs[q]];
          mdt = fmax(mdt, cutv(G, c_, CUT_DT));
          lo = fmin(lo, cutv(G, c_, CUT_SMIN));
          hi = fmax(hi, cutv(G, c_, CUT_SMAX));
          msd = fmax(msd, cutv(G, c_, CUT_SDIFF));
          tmin = fmin(tmin, S.t[hs[q]]);
          tmax = fmax(tmax, S.t[hs[q]]);
        }
        if (tmax - tmin > mdt) continue;
        double sl[3];
        bool ok = true;
        for (int q = 0; q + 1 < nl; ++q) {
          double s = (S.x[hs[q + 1]] - S.x[hs[q]]) / (G.bar_y[S.bar[hs[q + 1]]] - G.bar_y[S.bar[hs[q]]]);
          if (s < lo || s > hi) { ok = false; break; }
          sl[q] = s;
        }
        if (!ok) continue;
        if (nl > 2 && fabs(sl[0] - sl[1]) > msd) continue;
        if (nl > 3 && (fabs(sl[0] - sl[2]) > msd || fabs(sl[1] - sl[2]) > msd)) continue;
        // widen: x-sorted neighbours (stable)
        int srt[4];
        for (int q = 0; q < nl; ++q) srt[q] = hs[q];
        for (int a = 1; a < nl; ++a) {
          int v = srt[a];
          int b = a - 1;
          while (b >= 0 && S.x[srt[b]] > S.x[v]) { srt[b + 1] = srt[b]; --b; }
          srt[b + 1] = v;
        }
        for (int q = 0; q < nl; ++q) {
          double w = -1e300;
          if (q > 0) w = fmax(w, S.x[srt[q]] - S.x[srt[q - 1]]);
          if (q + 1 < nl) w = fmax(w, S.x[srt[q + 1]] - S.x[srt[q]]);
          // gaps are >= 0; maxd starts at final_max_distance: order non-negative doubles as integers
          if (w >= 0.0) atomicMax(&S.wid[srt[q]], (unsigned long long)__double_as_longlong(w));
          S.kept[srt[q]] = 1;
        }
      }
      __syncwarp();
    }
  }
  __syncwarp();
}

// scratch of the per-type lists beyond CoincShared (carved after it)
// scratch of the per-type lists beyond CoincShared; the attachment lists reuse lists that are dead by then (the
// type's hit list, the combination buckets, the first clustering's starts, cluster ids and maxd)
struct CoincWork {
  int32_t *clstart, *ccl, *cstart, *att_c, *att_cl, *att_bar, *att_sipm;
  double *cmd, *att_dt, *fmd;
};

__host__ __device__ inline size_t coinc_work_per_warp(int hcap) {
  return (size_t(hcap + 1) * 4 * 3 + size_t(hcap) * 8 * 2 + 64 + 15) & ~size_t(15);
}

__device__ inline CoincWork work_carve(char* b, int hcap, const CoincShared& S) {
  CoincWork W;
  double* d = reinterpret_cast<double*>(b);
  W.cmd = d; W.fmd = d + hcap;
  int32_t* q = reinterpret_cast<int32_t*>(d + 2 * hcap);
  W.clstart = q; W.ccl = q + (hcap + 1); W.cstart = q + 2 * (hcap + 1);
  W.att_c = S.list; W.att_cl = S.tmp; W.att_bar = W.clstart; W.att_sipm = S.cl_of; W.att_dt = W.fmd;
  return W;
}

// properties of one cluster (members: hit ids mem[0..m)); returns false when the cluster is below min_cluster_pes
__device__ bool cluster_props(const CoincGeom& G, const CoincShared& S, const CrvParams& p, int ti, int type,
                              const int32_t* mem, int m, ClusterRec& R) {
  double tot = 0.0, minpe = 1e300;
  for (int k = 0; k < m; ++k) {
    tot += S.pe[mem[k]];
    minpe = fmin(minpe, cutv(G, S.cut[mem[k]], CUT_MINPE));
  }
  if (tot < minpe) return false;
  double pos[3] = {0, 0, 0}, sx = 0, sy = 0, sxy = 0, syy = 0;
  for (int c = 0; c < 3; ++c) {
    double a = 0.0;
    for (int k = 0; k < m; ++k) a += G.bar_pos[S.bar[mem[k]] * 3 + c] * S.pe[mem[k]];
    pos[c] = a / tot;
  }
  for (int k = 0; k < m; ++k) {
    int h = mem[k];
    double pe = S.pe[h], x = S.x[h], y = G.bar_y[S.bar[h]];
    sxy += pe * x * y; sx += pe * x; sy += pe * y; syy += pe * y * y;
  }
  double slope = (tot * sxy - sx * sy) / (tot * syy - sy * sy);
  int nh[2] = {0, 0};
  double spe[2] = {0, 0}, stp[2] = {0, 0}, st[2], tmin[2] = {1e300, 1e300}, tmax[2] = {-1e300, -1e300};
  double t0 = 1e300, t1 = -1e300;
  unsigned layers = 0;
  for (int k = 0; k < m; ++k) {
    int h = mem[k];
    double t = S.t[h];
    t0 = fmin(t0, t); t1 = fmax(t1, t);
    layers |= 1u << S.layer[h];
    if (S.pe[h] > 0.0) {
      int sd = S.side[h];
      nh[sd] += 1; spe[sd] += S.pe[h]; stp[sd] += t * S.pe[h];
      tmin[sd] = fmin(tmin[sd], t); tmax[sd] = fmax(tmax[sd], t);
    }
  }
  for (int sd = 0; sd < 2; ++sd) {
    st[sd] = spe[sd] > 0.0 ? stp[sd] / spe[sd] : 0.0;
    if (!nh[sd]) { tmin[sd] = 0.0; tmax[sd] = 0.0; }
  }
  int ld = G.sec_length_dir[G.bar_sector[S.bar[mem[0]]]];
  double v = p.fiber_signal_speed, P0 = G.type_p0[ti], P1 = G.type_p1[ti];
  bool calc = false;
  double avg;
  if (nh[0] && nh[1]) {
    double org = 0.5 * (v * (st[0] - st[1]) + (P0 + P1));
    if (P0 < org && org < P1 && tmax[0] - tmin[0] < p.max_time_interval && tmax[1] - tmin[1] < p.max_time_interval) {
      calc = true;
      pos[ld] = org;
      avg = st[0] - (org - P0) / v;
    } else {
      org = pos[ld];
      avg = 0.5 * ((st[0] - (org - P0) / v) + (st[1] - (P1 - org) / v));
    }
  } else {
    double org = pos[ld];
    avg = nh[0] ? (st[0] - (org - P0) / v) : (st[1] - (P1 - org) / v);
  }
  R.pe = tot; R.start = t0; R.end = t1; R.slope = slope; R.avgtime = avg - p.time_offset;
  for (int c = 0; c < 3; ++c) R.pos[c] = pos[c];
  R.sidepe[0] = spe[0]; R.sidepe[1] = spe[1]; R.sidetime[0] = st[0]; R.sidetime[1] = st[1];
  R.type = type; R.sidehits[0] = nh[0]; R.sidehits[1] = nh[1]; R.nlayers = __popc(layers); R.poscalc = calc;
  return true;
}

constexpr int CO_WARPS_MAX = 8;

// Per-event scratch of the global-memory pass: event e's lists start at byte (ev_start[e] + 16 e) * COINC_GBYTES, room
// for the per-warp layout of its pulse count rounded up to 16 (coinc_smem_per_warp + coinc_work_per_warp), so the
// regions of different events are disjoint.
constexpr size_t COINC_GBYTES = 128;

// warp bitonic sort of a[0..n) ascending over the next power of two (a has room for it; padding with ~0)
__device__ inline void warp_sort_u64(unsigned long long* a, int n) {
  int P = 1;
  while (P < n) P <<= 1;
  for (int i = n + lane_id(); i < P; i += 32) a[i] = ~0ull;
  __syncwarp();
  for (int size = 2; size <= P; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int q = lane_id(); q < (P >> 1); q += 32) {
        const int lo = ((q & ~(stride - 1)) << 1) | (q & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const unsigned long long x = a[lo], y = a[hi];
        if ((x > y) == up) { a[lo] = y; a[hi] = x; }
      }
      __syncwarp();
    }
}

// pass 0: events with at most hcap hits (others deferred); pass 1: deferred events with at most hcap hits (others stay
// deferred); pass 2 (GLOBAL): the remaining deferred events, lists in global memory (gscratch) sized by the event.
// The global pass is its own instantiation, so the shared-memory passes do not carry its code and registers.
template <bool GLOBAL>
__global__ void __launch_bounds__(CO_WARPS_MAX * 32) k_coinc(CrvParams p, CoincGeom G, CoincIn I, int hcap,
                                                           int pass, CoincOut O, int32_t* __restrict__ deferred,
                                                           char* __restrict__ gscratch, Status* status) {
  extern __shared__ __align__(16) char smem[];
  CoincShared S;
  CoincWork W;
  unsigned long long* sk = nullptr;                // global pass: (layer, counter, order) sort words
  if (!GLOBAL) {
    size_t per = coinc_smem_per_warp(hcap) + coinc_work_per_warp(hcap);
    char* wb = smem + size_t(warp_in_block()) * per;
    S = coinc_carve(wb, hcap);
    W = work_carve(wb + coinc_smem_per_warp(hcap), hcap, S);
  }
  long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const long long nev = bounded_count(I.nev, I.nev_dev);
  for (long long e = blockIdx.x * (long long)(blockDim.x >> 5) + warp_in_block(); e < nev; e += warps) {
    if (pass > 0 && !deferred[e]) continue;
    long long r0 = I.ev_start[e];
    int np_ = I.ev_count[e];
    if (GLOBAL) {
      hcap = (np_ + 15) & ~15;
      char* wb = gscratch + size_t(r0 + 16 * e) * COINC_GBYTES;
      S = coinc_carve(wb, hcap);
      W = work_carve(wb + coinc_smem_per_warp(hcap), hcap, S);
      sk = reinterpret_cast<unsigned long long*>(wb + coinc_smem_per_warp(hcap) + coinc_work_per_warp(hcap));
    }
    // hits in pulse order
    int H = 0;
    for (int base = 0; base < np_; base += 32) {
      int i = base + lane_id();
      bool ok = false;
      int bar = 0, sec = 0, cut = -1, ti = -1;
      if (i < np_) {
        long long r = r0 + i;
        bar = I.bar[r];
        sec = G.bar_sector[bar];
        cut = G.sec_cut[sec];
        ok = cut >= 0 && !(p.ignore_secondary && I.seq[r] > 0);
        if (ok) {
          int ty = G.sec_type[sec];
          for (int k = 0; k < G.ntypes; ++k) if (G.type_id[k] == ty) ti = k;
          ok = ti >= 0;
        }
      }
      unsigned m = __ballot_sync(0xffffffffu, ok);
      int pos = H + __popc(m & ((1u << lane_id()) - 1u));
      if (ok && pos < hcap) {
        long long r = r0 + i;
        int sipm = I.sipm[r];
        int side = sipm % 2;
        double t = I.time[r];
        t += (side == 0 ? (G.sec_pos0[sec] - G.type_p0[ti]) : (G.type_p1[ti] - G.sec_pos1[sec])) / p.fiber_signal_speed;
        double pe = I.pe[r];
        int partner = bar * 4 + sipm + (sipm < 2 ? 2 : -2);
        if (I.status[partner] & p.compensate_mask) pe *= 2.0;
        S.idx[pos] = i; S.bar[pos] = uint16_t(bar); S.layer[pos] = uint8_t(G.bar_layer[bar]);
        S.counter[pos] = uint16_t(G.bar_counter[bar]); S.side[pos] = uint8_t(side); S.sipm[pos] = uint8_t(sipm);
        S.seq0[pos] = I.seq[r] == 0; S.cut[pos] = uint8_t(cut); S.type[pos] = uint8_t(ti);
        S.x[pos] = G.bar_x[bar]; S.t[pos] = t; S.pe[pos] = pe;
      }
      H += __popc(m);
    }
    if (H > hcap) {
      if (lane_id() == 0) {
        if (GLOBAL) {                                // cannot happen: the global lists hold every pulse of the event
          set_flag(status, CRV_ST_CAPACITY);
          need_at_least(status, CRV_NEED_HITS_PER_EVENT, H);
          O.ncl[e] = 0; O.nmem[e] = 0;
        } else {
          deferred[e] = 1;
        }
      }
      continue;
    }
    __syncwarp();
    int ncl_ev = 0, nmem_ev = 0;
    for (int ti = 0; ti < G.ntypes; ++ti) {
      // hits of this type, in order
      int nt = 0;
      for (int base = 0; base < H; base += 32) {
        int h = base + lane_id();
        bool in = h < H && S.type[h] == ti;
        unsigned m = __ballot_sync(0xffffffffu, in);
        if (in) S.list[nt + __popc(m & ((1u << lane_id()) - 1u))] = h;
        nt += __popc(m);
      }
      __syncwarp();
      if (nt == 0) continue;
      int nf = 0, nc = 0;
      for (int side = 0; side < 2; ++side) {
        // filterHits over the side's hits (list order sums)
        int f0 = nf;
        if constexpr (GLOBAL) {
          // large events: the side's hits sorted by (layer, counter, list order); each hit sums the entries of its own
          // and the two adjacent counters, which are contiguous there and, per counter, in list order
          int ns = 0;
          for (int base = 0; base < nt; base += 32) {
            const int k = base + lane_id();
            const bool on = k < nt && S.side[S.list[k]] == side;
            const unsigned m = __ballot_sync(0xffffffffu, on);
            if (on) {
              const int j = ns + __popc(m & ((1u << lane_id()) - 1u));
              const int h = S.list[k];
              const uint32_t key = uint32_t(S.layer[h]) * 65536u + S.counter[h];
              sk[j] = ((unsigned long long)key << 32) | uint32_t(j);
              S.tmp[j] = h;
            }
            ns += __popc(m);
          }
          __syncwarp();
          warp_sort_u64(sk, ns);
          for (int base = 0; base < ns; base += 32) {
            const int j = base + lane_id();
            bool pass_ = false;
            int h = -1;
            if (j < ns) {
              h = S.tmp[j];
              const uint32_t K = uint32_t(S.layer[h]) * 65536u + S.counter[h];
              const unsigned long long first = K > 0 ? (unsigned long long)(K - 1) << 32 : 0ull;
              int lo = 0, hi = ns;
              while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (sk[mid] < first) lo = mid + 1; else hi = mid;
              }
              double same = 0.0, a1 = 0.0, a2 = 0.0;
              const double dadj = cutv(G, S.cut[h], CUT_DTADJ);
              for (int q = lo; q < ns; ++q) {
                const unsigned long long w = sk[q];
                const uint32_t kq = uint32_t(w >> 32);
                if (kq > K + 1) break;
                const int a = S.tmp[uint32_t(w)];
                if (fabs(S.t[a] - S.t[h]) > dadj) continue;
                // each entry goes to the one sum its counter offset names (the other two would add +0.0, which
                // leaves a sum that starts at +0.0 unchanged: FP64 work saved, the same sums)
                const int d = int(kq) - int(K);
                if (d == 0) same += S.pe[a];
                else if (d == -1) a1 += S.pe[a];
                else a2 += S.pe[a];
              }
              const double thr = cutv(G, S.cut[h], CUT_PE);
              pass_ = (same + a1 >= thr) || (same + a2 >= thr);
            }
            const unsigned m = __ballot_sync(0xffffffffu, pass_);
            if (pass_) S.filt[nf + __popc(m & ((1u << lane_id()) - 1u))] = h;
            nf += __popc(m);
          }
        } else {
          // the side's hits bucketed by layer in list order (S.tmp: the previous side's combination buckets are used
          // up): a hit then scans the hits of its own side and layer only, in list order.  Only those, on this or an
          // adjacent counter, enter a sum (a hit elsewhere would add +0.0 to every sum, which changes none of them),
          // so the sums add the same terms in the same order as a scan of the whole list.
          int lb0 = 0, lb1 = 0, lb2 = 0, lb3 = 0, ns = 0;
          for (int l = 0; l < 4; ++l) {
            if (l == 1) lb1 = ns;
            if (l == 2) lb2 = ns;
            if (l == 3) lb3 = ns;
            for (int base = 0; base < nt; base += 32) {
              const int k = base + lane_id();
              const int h = k < nt ? S.list[k] : 0;
              const bool on = k < nt && S.side[h] == side && S.layer[h] == l;
              const unsigned m = __ballot_sync(0xffffffffu, on);
              if (on) S.tmp[ns + __popc(m & ((1u << lane_id()) - 1u))] = h;
              ns += __popc(m);
            }
          }
          __syncwarp();
        for (int base = 0; base < nt; base += 32) {
          int k = base + lane_id();
          bool pass = false;
          if (k < nt) {
            int h = S.list[k];
            if (S.side[h] == side) {
              double same = 0.0, a1 = 0.0, a2 = 0.0;
              double dadj = cutv(G, S.cut[h], CUT_DTADJ);
              const int l = S.layer[h];
              const int qa = l == 0 ? lb0 : l == 1 ? lb1 : l == 2 ? lb2 : lb3;
              const int qb = l == 0 ? lb1 : l == 1 ? lb2 : l == 2 ? lb3 : ns;
              for (int q = qa; q < qb; ++q) {
                int a = S.tmp[q];
                const int d = int(S.counter[a]) - int(S.counter[h]);
                if (d < -1 || d > 1 || fabs(S.t[a] - S.t[h]) > dadj) continue;
                if (d == 0) same += S.pe[a];
                else if (d == -1) a1 += S.pe[a];
                else a2 += S.pe[a];
              }
              double thr = cutv(G, S.cut[h], CUT_PE);
              pass = (same + a1 >= thr) || (same + a2 >= thr);
            }
          }
          unsigned m = __ballot_sync(0xffffffffu, pass);
          if (pass) S.filt[nf + __popc(m & ((1u << lane_id()) - 1u))] = S.list[k];
          nf += __popc(m);
        }
        }
        __syncwarp();
        int nfs = nf - f0;
        if (nfs == 0) continue;
        for (int k = lane_id(); k < nfs; k += 32) W.fmd[k] = cutv(G, S.cut[S.filt[f0 + k]], CUT_D0);
        __syncwarp();
        int ncl1 = greedy(S, S.filt + f0, W.fmd, nfs, G.type_maxdt[ti], false, 0.0, S.cl_of, S.clus, W.clstart,
                          reinterpret_cast<float*>(S.order));
        // clusters one per lane first: one with fewer non-empty layers than its smallest layer cut keeps no hit (as
        // check_coincidence finds), so only the others go through the check, in cluster order
        for (int cb = 0; cb < ncl1; cb += 32) {
         bool live = false;
         if (cb + lane_id() < ncl1) {
           const int c = cb + lane_id();
           unsigned lmask = 0;
           int nmin = 1 << 30;
           for (int z = W.clstart[c]; z < W.clstart[c + 1]; ++z) {
             const int h = S.filt[f0 + S.clus[z]];
             lmask |= 1u << S.layer[h];
             const int cl = trunc_int(cutv(G, S.cut[h], CUT_LAYERS));
             nmin = cl < nmin ? cl : nmin;
           }
           live = __popc(lmask) >= nmin;
         }
         unsigned lm = __ballot_sync(0xffffffffu, live);
         while (lm) {
          const int c = cb + __ffs(lm) - 1;
          lm &= lm - 1u;
          int a = W.clstart[c], b = W.clstart[c + 1];
          for (int k = lane_id(); k < b - a; k += 32) S.order[k] = S.filt[f0 + S.clus[a + k]];
          __syncwarp();
          check_coincidence(G, S, S.order, b - a, p.big_cluster_threshold);
          // kept members sorted by pulse idx -> coincidence list
          int mk = b - a;
          for (int k = lane_id(); k < mk; k += 32) {
            int h = S.order[k];
            if (!S.kept[h]) continue;
            int r = 0;
            for (int q = 0; q < mk; ++q) {
              int o = S.order[q];
              r += S.kept[o] && S.idx[o] < S.idx[h];
            }
            S.coinc[nc + r] = h;
            double w = __longlong_as_double((long long)S.wid[h]);
            double f = cutv(G, S.cut[h], CUT_D1);
            W.cmd[nc + r] = w > f ? w : f;
          }
          int nk = 0;
          for (int k = lane_id(); k < mk; k += 32) nk += S.kept[S.order[k]];
          nk = warp_sum(nk);
          __syncwarp();
          nc += nk;
         }
        }
      }
      if (nc == 0) continue;
      bool both = G.type_side0[ti] && G.type_side1[ti];
      double dt_opp = 2.0 * G.type_half[ti] / p.fiber_signal_speed;
      int ncl2 = greedy(S, S.coinc, W.cmd, nc, G.type_maxdt[ti], both, dt_opp, W.ccl, S.clus, W.cstart,
                        reinterpret_cast<float*>(S.order));
      // attachment of filtered first pulses on missing opposite counter ends
      int natt = 0;
      if (both && p.add_opposite) {
        double mdt = G.type_maxdt[ti] + dt_opp;
        for (int base = 0; base < nf; base += 32) {
          int k = base + lane_id();
          bool got = false;
          int bestc = 0;
          double bestdt = 0.0;
          int h = -1;
          if (k < nf) {
            h = S.filt[k];
            bool member = false;
            for (int q = 0; q < nc && !member; ++q) member = S.coinc[q] == h;
            if (S.seq0[h] && !member) {
              for (int q = 0; q < nc; ++q) {
                int a = S.coinc[q];
                if (!S.seq0[a] || S.bar[a] != S.bar[h] || S.side[h] != 1 - S.side[a]) continue;
                double dt = fabs(S.t[h] - S.t[a]);
                if (!(dt < mdt)) continue;
                int cl = W.ccl[q];
                bool occ = false;
                for (int z = W.cstart[cl]; z < W.cstart[cl + 1] && !occ; ++z) {
                  int o = S.coinc[S.clus[z]];
                  occ = S.bar[o] == S.bar[h] && S.side[o] == S.side[h];
                }
                if (occ) continue;
                if (!got || dt < bestdt || (dt == bestdt && cl < bestc)) { got = true; bestdt = dt; bestc = cl; }
              }
            }
          }
          unsigned m = __ballot_sync(0xffffffffu, got);
          if (got) {
            int o = natt + __popc(m & ((1u << lane_id()) - 1u));
            W.att_c[o] = k; W.att_cl[o] = bestc; W.att_dt[o] = bestdt;
            W.att_bar[o] = S.bar[h]; W.att_sipm[o] = S.sipm[h];
          }
          natt += __popc(m);
        }
        __syncwarp();
        if (lane_id() == 0 && natt > 1) {     // sort by (cluster, bar, sipm, dt, candidate)
          for (int a = 1; a < natt; ++a) {
            int c = W.att_c[a], cl = W.att_cl[a], br = W.att_bar[a], sp = W.att_sipm[a];
            double dt = W.att_dt[a];
            int b = a - 1;
            while (b >= 0) {
              bool gt = W.att_cl[b] != cl ? W.att_cl[b] > cl : W.att_bar[b] != br ? W.att_bar[b] > br
                      : W.att_sipm[b] != sp ? W.att_sipm[b] > sp : W.att_dt[b] != dt ? W.att_dt[b] > dt
                      : W.att_c[b] > c;
              if (!gt) break;
              W.att_c[b + 1] = W.att_c[b]; W.att_cl[b + 1] = W.att_cl[b]; W.att_bar[b + 1] = W.att_bar[b];
              W.att_sipm[b + 1] = W.att_sipm[b]; W.att_dt[b + 1] = W.att_dt[b];
              --b;
            }
            W.att_c[b + 1] = c; W.att_cl[b + 1] = cl; W.att_bar[b + 1] = br; W.att_sipm[b + 1] = sp;
            W.att_dt[b + 1] = dt;
          }
          // keep the first per (cluster, bar, sipm): mark duplicates with cluster -1
          for (int a = 1; a < natt; ++a) {
            int b = a - 1;
            while (b >= 0 && W.att_cl[b] < 0) --b;
            if (b >= 0 && W.att_cl[b] == W.att_cl[a] && W.att_bar[b] == W.att_bar[a] && W.att_sipm[b] == W.att_sipm[a])
              W.att_cl[a] = -1 - W.att_cl[a];
          }
        }
        __syncwarp();
      }
      // clusters -> records (lane 0), members into the event's member slots
      if (lane_id() == 0) {
        for (int c = 0; c < ncl2; ++c) {
          int m = 0;
          int a = W.cstart[c], b = W.cstart[c + 1];
          for (int z = a; z < b; ++z) S.order[m++] = S.coinc[S.clus[z]];
          for (int z = 0; z < natt; ++z)
            if (W.att_cl[z] == c) S.order[m++] = S.filt[W.att_c[z]];
          ClusterRec R;
          if (!cluster_props(G, S, p, ti, G.type_id[ti], S.order, m, R)) continue;
          R.mem_begin = nmem_ev;
          R.mem_count = m;
          R.pad = 0;
          if (ncl_ev < np_ && nmem_ev + m <= np_) {
            O.rec[r0 + ncl_ev] = R;
            for (int z = 0; z < m; ++z) O.mem_idx[r0 + nmem_ev + z] = S.idx[S.order[z]];
          }
          ++ncl_ev;
          nmem_ev += m;
        }
      }
      ncl_ev = __shfl_sync(0xffffffffu, ncl_ev, 0);
      nmem_ev = __shfl_sync(0xffffffffu, nmem_ev, 0);
      __syncwarp();
    }
    if (lane_id() == 0) {
      O.ncl[e] = ncl_ev;
      O.nmem[e] = nmem_ev;
      if (pass > 0) deferred[e] = 0;
      if (ncl_ev > np_ || nmem_ev > np_) set_flag(status, CRV_ST_LIMIT);
    }
    __syncwarp();
  }
}

}  // namespace crv
