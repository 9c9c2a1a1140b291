// C ABI of the CRV response engine: argument checks, workspace layout, launch orchestration.
// The kernels of each precision live in crv_kernels_f64.cu / crv_kernels_f32.cu; this unit holds the precision-free
// kernels (event preparation, SiPM sizing, compaction, scans).
#define CRV_ENGINE_TU 1
#include <cuda.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "crv_launch.h"
#include "crv_response.cuh"
#include "crv_waveform.cuh"
#include "crv_pulsefit.cuh"
#include "crv_coinc.cuh"

namespace crv {

const DeviceInfo& device_info() {
  static DeviceInfo di{0, 0};
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 0, optin = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    di.sms = sms > 0 ? sms : 1;
    di.smem_optin = size_t(optin > 0 ? optin : 48 * 1024);
  });
  return di;
}

// ---- launch accounting / profiling ---------------------------------------------------------------------------------

namespace {
struct ProfRec {
  const char* name;
  cudaEvent_t a, b;
};
std::mutex g_prof_mu;
bool g_prof_on = false;
std::vector<ProfRec> g_prof;
std::vector<cudaEvent_t> g_pool;
size_t g_pool_used = 0;
std::atomic<long long> g_launches{0};

cudaEvent_t pool_event() {
  if (g_pool_used == g_pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    g_pool.push_back(e);
  }
  return g_pool[g_pool_used++];
}
}  // namespace

Mark::Mark(const char* name, cudaStream_t s) : slot(-1), stream(s) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  if (!g_prof_on) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  ProfRec r{name, pool_event(), pool_event()};
  cudaEventRecord(r.a, s);
  slot = int(g_prof.size());
  g_prof.push_back(r);
}

Mark::~Mark() {
  if (slot < 0) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  cudaEventRecord(g_prof[slot].b, stream);
}

__global__ void k_scan_parts(long long* __restrict__ part, long long nb, long long* __restrict__ total) {
  // single block: running exclusive scan over chunks of blockDim.x
  __shared__ long long carry;
  __shared__ long long wsum[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (long long base = 0; base < nb; base += blockDim.x) {
    long long i = base + threadIdx.x;
    long long v = i < nb ? part[i] : 0;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      long long q = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
      long long qq = q;
      for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, qq, o);
        if (lane >= o) qq += y;
      }
      if (lane < (int)(blockDim.x >> 5)) wsum[lane] = qq - q;
    }
    __syncthreads();
    long long ex = carry + wsum[w] + x - v;
    if (i < nb) part[i] = ex;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = ex + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_check_caps(const long long* __restrict__ total, long long cap, int need_slot, Status* status) {
  if (threadIdx.x == 0 && blockIdx.x == 0 && *total > cap) {
    set_flag(status, CRV_ST_CAPACITY);
    need_at_least(status, need_slot, *total);
  }
}

__global__ void k_copy_i64(const long long* __restrict__ src, long long* __restrict__ dst) { *dst = *src; }

__global__ void k_sipm_diag(const long long* __restrict__ nsipm_dev, long long cap, const long long* __restrict__ label,
                            const int32_t* __restrict__ nphot, const int32_t* __restrict__ fired,
                            int64_t* __restrict__ o_label, int32_t* __restrict__ o_phot, int32_t* __restrict__ o_fired,
                            Status* status) {
  long long n = *nsipm_dev;
  if (n > cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) { set_flag(status, CRV_ST_CAPACITY); }
    return;
  }
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
    if (o_label) o_label[g] = label[g];
    if (o_phot) o_phot[g] = nphot[g];
    if (o_fired) o_fired[g] = fired[g];
  }
}

__global__ void k_slot_caps(long long ng, const int32_t* __restrict__ gcount, int factor, int32_t* __restrict__ cap) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x)
    cap[g] = gcount[g] > 0 ? factor * gcount[g] + 16 : 0;
}

__global__ void k_fill_step_event(CrvEvents ev, long long nevents, int32_t* __restrict__ step_event) {
  long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long e = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); e < nevents; e += warps) {
    long long f = ev.first_step[e];
    for (int i = threadIdx.x & 31; i < ev.nsteps[e]; i += 32) step_event[f + i] = int32_t(e);
  }
}

__global__ void k_set_i64(long long* __restrict__ dst, long long v) { *dst = v; }

// *out = (*total <= cap) ? *n : 0  (downstream kernels then see no groups)
__global__ void k_guard_groups(const long long* __restrict__ total, long long cap, const long long* __restrict__ n,
                               long long* __restrict__ out) {
  *out = (*total <= cap) ? *n : 0;
}

// ---------------------------------------------------------------------------------------------------------------------
// workspace carving

struct Carve {
  char* base;
  size_t off = 0;
  template <typename T>
  T* take(long long n) {
    off = (off + 255) & ~size_t(255);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += size_t(n > 0 ? n : 1) * sizeof(T);
    return p;
  }
};

struct RespWs {
  int32_t *step_event, *step_order, *count, *sipm_count;
  long long* sipm_off;
  int32_t *s_event, *s_chan, *s_nseg, *nphot, *slot_cap, *nmain, *nap, *fired, *ntot;
  long long *s_seg, *id_base, *label, *ph_off, *slot_off, *out_off, *parts, *totals;
  uint32_t* run;
  void* ph_t;
  uint32_t* ph_key;
  double *slot_t, *slot_v;
  long long* slot_id;
  long long nb, pc, sc;
  LookupChainWs lk;              // lookup-table model (resident chain): rows, counts, offsets, photon ids
};

// lookup: the lookup-table model's arrays too (photon times in FP64 in ph_t, whatever the precision)
static RespWs resp_layout(char* base, const CrvParams& p, long long ne, long long ns, long long photon_cap, size_t* bytes,
                          bool lookup = false) {
  Carve c{base};
  RespWs w;
  w.nb = 4 * ns;
  w.pc = photon_cap;
  w.sc = (long long)(p.charge_factor > 0 ? p.charge_factor : 1) * photon_cap + 16 * w.nb;
  size_t rb = p.precision == 1 && !lookup ? 4 : 8;
  w.step_event = c.take<int32_t>(ns);
  w.step_order = c.take<int32_t>(ns);
  w.count = c.take<int32_t>(4 * ns);
  w.sipm_count = c.take<int32_t>(ne);
  w.sipm_off = c.take<long long>(ne);
  w.s_event = c.take<int32_t>(w.nb);
  w.s_chan = c.take<int32_t>(w.nb);
  w.s_nseg = c.take<int32_t>(w.nb);
  w.nphot = c.take<int32_t>(w.nb);
  w.slot_cap = c.take<int32_t>(w.nb);
  w.nmain = c.take<int32_t>(w.nb);
  w.nap = c.take<int32_t>(w.nb);
  w.fired = c.take<int32_t>(w.nb);
  w.ntot = c.take<int32_t>(w.nb);
  w.s_seg = c.take<long long>(w.nb);
  w.id_base = c.take<long long>(w.nb);
  w.label = c.take<long long>(w.nb);
  w.ph_off = c.take<long long>(w.nb);
  w.slot_off = c.take<long long>(w.nb);
  w.out_off = c.take<long long>(w.nb);
  w.run = c.take<uint32_t>(w.nb);
  long long mx = ne > w.nb ? ne : w.nb;
  w.parts = c.take<long long>(scan_parts_len(mx) + 1);
  w.totals = c.take<long long>(8);
  w.ph_t = c.take<char>(photon_cap * (long long)rb);
  w.ph_key = c.take<uint32_t>(photon_cap);
  w.slot_t = c.take<double>(w.sc);
  w.slot_v = c.take<double>(w.sc);
  w.slot_id = c.take<long long>(w.sc);
  w.lk = LookupChainWs{};
  if (lookup) {
    const long long nr = w.nb;
    CrvSubstepRowsOut& o = w.lk.rows;
    o.s = c.take<double>(3 * nr);
    o.d = c.take<double>(3 * nr);
    double** dcols[6] = {&o.t0, &o.t1, &o.beta, &o.cos_theta, &o.dev, &o.mu};
    for (auto q : dcols) *q = c.take<double>(nr);
    int64_t** icols[6] = {&o.nsub, &o.step, &o.chan, &o.n_scint, &o.n_ck_s, &o.n_ck_f};
    for (auto q : icols) *q = c.take<int64_t>(nr);
    w.lk.row_group = c.take<int8_t>(nr);
    w.lk.count = c.take<long long>(nr);
    w.lk.row_off = c.take<long long>(nr);
    w.lk.nrows = c.take<long long>(1);
    w.lk.seed = c.take<uint32_t>(1);
    w.lk.o_step = c.take<int64_t>(photon_cap);
    w.lk.o_time = reinterpret_cast<double*>(w.ph_t);
  }
  *bytes = c.off + 256;
  return w;
}

}  // namespace crv

using namespace crv;

#define CK(x)                                   \
  do {                                          \
    cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) return CRV_ERR_CUDA; \
  } while (0)

static unsigned grid_for(long long n, int per_block, int mult) {
  long long b = (n + per_block - 1) / per_block;
  long long mx = (long long)device_info().sms * mult;
  if (b < 1) b = 1;
  return (unsigned)(b < mx ? b : mx);
}

extern "C" {

int crv_version(void) { return CRVGPU_VERSION; }

long long crv_launch_count(void) { return g_launches.load(); }

void crv_profile(int on) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof.clear();
  g_pool_used = 0;
  g_prof_on = on != 0;
}

int crv_profile_read(int cap, char* names, float* ms) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  int n = int(g_prof.size());
  for (int i = 0; i < n && i < cap; ++i) {
    cudaEventSynchronize(g_prof[i].b);
    float t = 0.f;
    cudaEventElapsedTime(&t, g_prof[i].a, g_prof[i].b);
    ms[i] = t;
    strncpy(names + size_t(i) * 64, g_prof[i].name, 63);
    names[size_t(i) * 64 + 63] = 0;
  }
  return n;
}

const char* crv_status_string(int32_t flags) {
  static thread_local char buf[256];
  if (flags == 0) return "ok";
  buf[0] = 0;
  const char* names[] = {"capacity", "limit", "nonfinite", "order", "bounds"};
  for (int i = 0; i < 5; ++i)
    if (flags & (1 << i)) {
      if (buf[0]) strncat(buf, "|", sizeof(buf) - strlen(buf) - 1);
      strncat(buf, names[i], sizeof(buf) - strlen(buf) - 1);
    }
  return buf;
}

int64_t crv_response_workspace(const CrvParams* p, int64_t nevents, int64_t nsteps, int64_t photon_cap,
                               int32_t max_steps_per_event) {
  if (!p || nevents < 0 || nsteps < 0 || photon_cap < 0) return -1;
  (void)max_steps_per_event;
  size_t bytes = 0;
  resp_layout(nullptr, *p, nevents, nsteps, photon_cap, &bytes);
  return (int64_t)bytes;
}

int crv_photon_counts(const CrvParams* p, const CrvEvents* ev, int64_t nevents, const CrvSteps* st, int64_t nsteps,
                      const CrvBars* bars, const CrvChannels* ch, int32_t* step_event, int32_t* count, void* stream,
                      CrvStatus* status_dev) {
  if (!p || !ev || !st || !bars || !ch || !step_event || !count || !status_dev) return CRV_ERR_ARG;
  if (st->real_bytes != 4 && st->real_bytes != 8) return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Status* S = reinterpret_cast<Status*>(status_dev);
  if (nevents == 0 || nsteps == 0) return CRV_OK;
  {
    crv::Mark mark_("k_fill_step_event", s);
    k_fill_step_event<<<grid_for(nevents, 8, 32), 256, 0, s>>>(*ev, nevents, step_event);
  }
  CK(cudaGetLastError());
  if (p->precision == 1)
    CK(launch_photon_count<float>(*p, *ev, *st, *bars, *ch, step_event, nsteps, nullptr, 0, count, S, s));
  else
    CK(launch_photon_count<double>(*p, *ev, *st, *bars, *ch, step_event, nsteps, nullptr, 0, count, S, s));
  return CRV_OK;
}

int crv_photons(const CrvParams* p, const CrvEvents* ev, int64_t nevents, const CrvSteps* st, int64_t nsteps,
                const CrvBars* bars, const int32_t* step_event, const int32_t* count, const int64_t* row_offset,
                int64_t* o_step, int64_t* o_chan, double* o_time, int64_t* o_key, void* stream,
                CrvStatus* status_dev) {
  if (!p || !ev || !st || !bars || !step_event || !count || !row_offset || !status_dev) return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (nevents == 0 || nsteps == 0) return CRV_OK;
  const long long* ro = reinterpret_cast<const long long*>(row_offset);
  if (p->precision == 1)
    CK(launch_photon_rows<float>(*p, *ev, *st, *bars, step_event, nsteps, count, ro, o_step, o_chan, o_time, o_key, s));
  else
    CK(launch_photon_rows<double>(*p, *ev, *st, *bars, step_event, nsteps, count, ro, o_step, o_chan, o_time, o_key,
                                  s));
  return CRV_OK;
}

// Stage bodies take an optional device count beside each host count (the host count is then a capacity), so that a
// whole chain can run without reading sizes back: the public entry points pass null.
// Lookup-table model in the resident chain: the output offset of every row of every SiPM, its steps in order (rows of
// SiPMs without an entry keep -1 and are not written)
__global__ void k_lrow_offsets(const long long* __restrict__ nsipm_dev, const int32_t* __restrict__ s_chan,
                               const long long* __restrict__ s_seg, const int32_t* __restrict__ s_nseg,
                               const int32_t* __restrict__ step_order, const int32_t* __restrict__ count,
                               const long long* __restrict__ ph_off, long long* __restrict__ row_off) {
  const long long nsipm = *nsipm_dev;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nsipm;
       g += (long long)gridDim.x * blockDim.x) {
    const int sp = s_chan[g] & 3;
    const long long a = s_seg[g];
    long long o = ph_off[g];
    for (int k = 0; k < s_nseg[g]; ++k) {
      const long long r = 4 * (long long)step_order[a + k] + sp;
      row_off[r] = o;
      o += count[r];
    }
  }
}

static int response_run(const CrvParams* p, const CrvEvents* ev, int64_t nevents, const CrvSteps* st, int64_t nsteps,
                        const long long* nsteps_dev, int32_t max_steps_per_event, const CrvBars* bars,
                        const CrvChannels* ch, const CrvPixels* px, int64_t photon_cap, CrvCharges* out,
                        int64_t out_cap, int64_t* n_out_dev, int64_t* sipm_label, int32_t* sipm_photons,
                        int32_t* sipm_fired, int64_t sipm_cap, int64_t* n_sipm_dev, void* workspace,
                        int64_t workspace_bytes, void* stream, CrvStatus* status_dev,
                        const CrvLookupChain* lk = nullptr) {
  if (!p || !ev || !st || !bars || !ch || !px || !out || !n_out_dev || !status_dev) return CRV_ERR_ARG;
  if (st->real_bytes != 4 && st->real_bytes != 8) return CRV_ERR_ARG;
  if (nevents < 0 || nsteps < 0 || photon_cap < 0 || out_cap < 0 || max_steps_per_event < 0) return CRV_ERR_ARG;
  if (lk && (lk->ngroups < 0 || lk->ngroups > CRV_LOOKUP_CHAIN_GROUPS || !nsteps_dev)) return CRV_ERR_ARG;
  size_t need = 0;
  resp_layout(nullptr, *p, nevents, nsteps, photon_cap, &need, lk != nullptr);
  if (!workspace || (size_t)workspace_bytes < need) return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  Status* S = reinterpret_cast<Status*>(status_dev);
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  size_t dummy;
  RespWs w = resp_layout(base, *p, nevents, nsteps, photon_cap, &dummy, lk != nullptr);
  CK(cudaMemsetAsync(w.totals, 0, 8 * sizeof(long long), s));
  if (nevents == 0 || nsteps == 0) {
    CK(cudaMemsetAsync(n_out_dev, 0, sizeof(long long), s));
    if (n_sipm_dev) CK(cudaMemsetAsync(n_sipm_dev, 0, sizeof(long long), s));
    return CRV_OK;
  }
  CK(cudaMemsetAsync(w.nphot, 0, sizeof(int32_t) * w.nb, s));
  CK(cudaMemsetAsync(w.slot_cap, 0, sizeof(int32_t) * w.nb, s));
  CK(cudaMemsetAsync(w.nmain, 0, sizeof(int32_t) * w.nb, s));
  CK(cudaMemsetAsync(w.nap, 0, sizeof(int32_t) * w.nb, s));
  CK(cudaMemsetAsync(w.fired, 0, sizeof(int32_t) * w.nb, s));
  CK(cudaMemsetAsync(w.ntot, 0, sizeof(int32_t) * w.nb, s));
  // 1. events: steps grouped by bar, SiPM counts; 2. scan; 3. SiPM table
  int stepcap = 1;
  while (stepcap < max_steps_per_event) stepcap <<= 1;
  if (stepcap > 65536) stepcap = 65536;
  size_t psmem = size_t(stepcap) * 4;
  if (psmem > device_info().smem_optin) return CRV_ERR_ARG;
  CK(allow_dynamic_smem(k_event_prep));
  unsigned gp = grid_for(nevents, 1, 8);
  {
    crv::Mark mark_("k_event_prep", s);
    k_event_prep<<<gp, PREP_THREADS, psmem, s>>>(*ev, nevents, *st, *ch, 1, stepcap, w.step_event, w.step_order,
                                                  w.sipm_count, nullptr, nullptr, nullptr, nullptr, nullptr, S, 0);
  }
  CK(cudaGetLastError());
  CK(exclusive_scan(w.sipm_count, nevents, Identity(), w.sipm_off, &w.totals[0], w.parts, s));
  {
    crv::Mark mark_("k_event_prep", s);
    k_event_prep<<<gp, PREP_THREADS, psmem, s>>>(*ev, nevents, *st, *ch, 1, stepcap, nullptr, nullptr, nullptr,
                                                  w.sipm_off, w.s_event, w.s_chan, w.s_seg, w.s_nseg, S, 1);
  }
  CK(cudaGetLastError());
  // 4. photon counts per (step, SiPM): the lookup-table model's rows and arrival counts, or the analytic model's
  if (lk) {
    CK(lookup_chain_rows(*p, *lk, nsteps_dev, nsteps, w.lk, s));
    CK(lookup_chain_count(*lk, w.lk, w.nb, w.count, S, s));
  } else if (p->precision == 1)
    CK(launch_photon_count<float>(*p, *ev, *st, *bars, *ch, w.step_event, nsteps, nsteps_dev, 1, w.count, S, s));
  else
    CK(launch_photon_count<double>(*p, *ev, *st, *bars, *ch, w.step_event, nsteps, nsteps_dev, 1, w.count, S, s));
  // 5. per-SiPM photons and charge slots; scans
  int factor = p->charge_factor > 0 ? p->charge_factor : 1;
  {
    crv::Mark mark_("k_sipm_sizes", s);
    k_sipm_sizes<<<grid_for(w.nb, 256, 8), 256, 0, s>>>(&w.totals[0], w.s_event, w.s_chan, w.s_seg, w.s_nseg,
                                                        w.step_order, w.count, *ev, factor, w.nphot, w.slot_cap,
                                                        w.id_base, w.label, w.run);
  }
  CK(cudaGetLastError());
  CK(exclusive_scan(w.nphot, w.nb, Identity(), w.ph_off, &w.totals[1], w.parts, s, &w.totals[0]));
  CK(exclusive_scan(w.slot_cap, w.nb, Identity(), w.slot_off, &w.totals[2], w.parts, s, &w.totals[0]));
  {
    crv::Mark mark_("k_check_caps", s);
    k_check_caps<<<1, 32, 0, s>>>(&w.totals[1], w.pc, CRV_NEED_PHOTONS_TOTAL, S);
  }
  {
    crv::Mark mark_("k_check_caps", s);
    k_check_caps<<<1, 32, 0, s>>>(&w.totals[2], w.sc, CRV_NEED_SLOTS_TOTAL, S);
  }
  CK(cudaGetLastError());
  // 6. photons of every SiPM (lookup model: each row's photons at the offset of its step in its SiPM)
  if (lk) {
    CK(cudaMemsetAsync(w.lk.row_off, 0xFF, sizeof(long long) * size_t(w.nb), s));
    {
      crv::Mark mark_("k_lrow_offsets", s);
      k_lrow_offsets<<<grid_for(w.nb, 256, 8), 256, 0, s>>>(&w.totals[0], w.s_chan, w.s_seg, w.s_nseg, w.step_order,
                                                            w.count, w.ph_off, w.lk.row_off);
    }
    CK(cudaGetLastError());
    CK(lookup_chain_emit(*lk, w.lk, w.nb, &w.totals[1], w.pc, S, s));
  } else if (p->precision == 1)
    CK(launch_photon_emit<float>(*p, *ev, *st, *bars, w.nb, &w.totals[0], w.s_event, w.s_chan, w.s_seg, w.s_nseg,
                                 w.step_order, w.count, w.ph_off, (float*)w.ph_t, w.ph_key, &w.totals[1], w.pc, s));
  else
    CK(launch_photon_emit<double>(*p, *ev, *st, *bars, w.nb, &w.totals[0], w.s_event, w.s_chan, w.s_seg, w.s_nseg,
                                  w.step_order, w.count, w.ph_off, (double*)w.ph_t, w.ph_key, &w.totals[1], w.pc, s));
  // 7. SiPM simulation
  SipmGroups G{};
  G.n = &w.totals[0];
  G.guard[0] = &w.totals[1];
  G.guard_cap[0] = w.pc;
  G.guard[1] = &w.totals[2];
  G.guard_cap[1] = w.sc;
  G.start = w.ph_off;
  G.count = w.nphot;
  G.label = w.label;
  G.run = w.run;
  G.key32 = lk ? nullptr : w.ph_key;          // lookup model: draw key = index of the photon in its SiPM
  G.key64 = nullptr;
  G.photon_id = lk ? reinterpret_cast<const long long*>(w.lk.o_step) : nullptr;
  G.id_base = w.id_base;
  G.slot_off = w.slot_off;
  G.slot_cap = w.slot_cap;
  SipmOut O{w.slot_t, w.slot_v, w.slot_id, w.nmain, w.nap, w.fired};
  if (p->precision == 1 && lk)
    CK((launch_sipm<float, double>(*p, *px, G, &w.totals[0], (const double*)w.ph_t, O, S, s)));
  else if (p->precision == 1)
    CK((launch_sipm<float, float>(*p, *px, G, &w.totals[0], (const float*)w.ph_t, O, S, s)));
  else
    CK((launch_sipm<double, double>(*p, *px, G, &w.totals[0], (const double*)w.ph_t, O, S, s)));
  // 8. compaction into label/time order
  {
    crv::Mark mark_("k_counts_total", s);
    k_counts_total<<<grid_for(w.nb, 256, 8), 256, 0, s>>>(&w.totals[0], w.nmain, w.nap, w.ntot);
  }
  CK(cudaGetLastError());
  CK(exclusive_scan(w.ntot, w.nb, Identity(), w.out_off, &w.totals[3], w.parts, s, &w.totals[0]));
  {
    crv::Mark mark_("k_check_caps", s);
    k_check_caps<<<1, 32, 0, s>>>(&w.totals[3], out_cap, CRV_NEED_CHARGES_OUT, S);
  }
  {
    crv::Mark mark_("k_charge_compact", s);
    k_charge_compact<<<grid_for(w.nb, 8, 16), 256, 0, s>>>(&w.totals[0], w.label, w.slot_off, w.slot_cap, w.nmain,
                                                            w.nap, w.out_off, w.slot_t, w.slot_v, w.slot_id,
                                                            p->capacitance, p->overvoltage, p->precision == 1,
                                                            *out, out_cap);
  }
  CK(cudaGetLastError());
  {
    crv::Mark mark_("k_copy_i64", s);
    k_copy_i64<<<1, 1, 0, s>>>(&w.totals[3], reinterpret_cast<long long*>(n_out_dev));
  }
  if (n_sipm_dev) {
    crv::Mark mark_("k_copy_i64", s);
    k_copy_i64<<<1, 1, 0, s>>>(&w.totals[0], reinterpret_cast<long long*>(n_sipm_dev));
  }
  if (sipm_label || sipm_photons || sipm_fired)
    {
      crv::Mark mark_("k_sipm_diag", s);
      k_sipm_diag<<<grid_for(w.nb, 256, 8), 256, 0, s>>>(&w.totals[0], sipm_cap, w.label, w.nphot, w.fired,
                                                         sipm_label, sipm_photons, sipm_fired, S);
    }
  CK(cudaGetLastError());
  return CRV_OK;
}

int crv_response(const CrvParams* p, const CrvEvents* ev, int64_t nevents, const CrvSteps* st, int64_t nsteps,
                 int32_t max_steps_per_event, const CrvBars* bars, const CrvChannels* ch, const CrvPixels* px,
                 int64_t photon_cap, CrvCharges* out, int64_t out_cap, int64_t* n_out_dev, int64_t* sipm_label,
                 int32_t* sipm_photons, int32_t* sipm_fired, int64_t sipm_cap, int64_t* n_sipm_dev, void* workspace,
                 int64_t workspace_bytes, void* stream, CrvStatus* status_dev) {
  return response_run(p, ev, nevents, st, nsteps, nullptr, max_steps_per_event, bars, ch, px, photon_cap, out, out_cap,
                      n_out_dev, sipm_label, sipm_photons, sipm_fired, sipm_cap, n_sipm_dev, workspace,
                      workspace_bytes, stream, status_dev);
}

// ---- sipm.simulate over caller-grouped photons -------------------------------------------------------------------

struct SipmWs {
  long long *slot_off, *out_off, *parts, *totals, *label_dummy;
  int32_t *slot_cap, *nmain, *nap, *ntot;
  double *slot_t, *slot_v;
  long long* slot_id;
  long long sc;
};

static SipmWs sipm_layout(char* base, const CrvParams& p, long long ng, long long nph, size_t* bytes) {
  Carve c{base};
  SipmWs w;
  w.sc = (long long)(p.charge_factor > 0 ? p.charge_factor : 1) * nph + 16 * ng;
  w.slot_off = c.take<long long>(ng);
  w.out_off = c.take<long long>(ng);
  w.parts = c.take<long long>(scan_parts_len(ng) + 1);
  w.totals = c.take<long long>(8);
  w.label_dummy = nullptr;
  w.slot_cap = c.take<int32_t>(ng);
  w.nmain = c.take<int32_t>(ng);
  w.nap = c.take<int32_t>(ng);
  w.ntot = c.take<int32_t>(ng);
  w.slot_t = c.take<double>(w.sc);
  w.slot_v = c.take<double>(w.sc);
  w.slot_id = c.take<long long>(w.sc);
  *bytes = c.off + 256;
  return w;
}

int64_t crv_sipm_workspace(const CrvParams* p, int64_t ngroups, int64_t nphotons) {
  if (!p || ngroups < 0 || nphotons < 0) return -1;
  size_t b = 0;
  sipm_layout(nullptr, *p, ngroups, nphotons, &b);
  return (int64_t)b;
}

}  // extern "C"

extern "C" int crv_sipm(const CrvParams* p, const CrvPixels* px, int64_t ngroups, int64_t nphotons, const int64_t* gstart,
                        const int32_t* gcount, const int64_t* glabel, const uint32_t* grun, const double* time,
                        const int64_t* key, const int64_t* photon, CrvCharges* out, int64_t out_cap,
                        int64_t* n_out_dev, int32_t* g_charges, int32_t* g_fired, void* workspace,
                        int64_t workspace_bytes, void* stream, CrvStatus* status_dev) {
  if (!p || !px || !out || !n_out_dev || !status_dev || ngroups < 0) return CRV_ERR_ARG;
  if (ngroups > 0 && (!gstart || !gcount || !glabel || !grun || !time || !key || !photon || !g_fired)) return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (ngroups == 0) {
    CK(cudaMemsetAsync(n_out_dev, 0, sizeof(long long), s));
    return CRV_OK;
  }
  long long nph_bound = nphotons;
  size_t need = 0;
  sipm_layout(nullptr, *p, ngroups, nph_bound, &need);
  if (!workspace || (long long)need > workspace_bytes) return CRV_ERR_ARG;
  Status* S = reinterpret_cast<Status*>(status_dev);
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  size_t dummy;
  SipmWs w = sipm_layout(base, *p, ngroups, nph_bound, &dummy);
  int factor = p->charge_factor > 0 ? p->charge_factor : 1;
  CK(cudaMemsetAsync(w.totals, 0, 8 * sizeof(long long), s));
  CK(cudaMemsetAsync(w.nmain, 0, sizeof(int32_t) * ngroups, s));
  CK(cudaMemsetAsync(w.nap, 0, sizeof(int32_t) * ngroups, s));
  CK(cudaMemsetAsync(g_fired, 0, sizeof(int32_t) * ngroups, s));
  {
    crv::Mark mark_("k_set_i64", s);
    k_set_i64<<<1, 1, 0, s>>>(&w.totals[0], ngroups);
  }
  {
    crv::Mark mark_("k_slot_caps", s);
    k_slot_caps<<<grid_for(ngroups, 256, 8), 256, 0, s>>>(ngroups, gcount, factor, w.slot_cap);
  }
  CK(cudaGetLastError());
  CK(exclusive_scan(w.slot_cap, ngroups, Identity(), w.slot_off, &w.totals[2], w.parts, s));
  {
    crv::Mark mark_("k_check_caps", s);
    k_check_caps<<<1, 32, 0, s>>>(&w.totals[2], w.sc, CRV_NEED_SLOTS_TOTAL, S);
  }
  SipmGroups G{};
  G.n = &w.totals[0];
  G.guard[0] = &w.totals[2];
  G.guard_cap[0] = w.sc;
  G.guard[1] = nullptr;
  G.start = reinterpret_cast<const long long*>(gstart);
  G.count = gcount;
  G.label = reinterpret_cast<const long long*>(glabel);
  G.run = grun;
  G.key32 = nullptr;
  G.key64 = reinterpret_cast<const long long*>(key);
  G.photon_id = reinterpret_cast<const long long*>(photon);
  G.id_base = nullptr;
  G.slot_off = w.slot_off;
  G.slot_cap = w.slot_cap;
  SipmOut O{w.slot_t, w.slot_v, w.slot_id, w.nmain, w.nap, g_fired};
  if (p->precision == 1)
    CK((launch_sipm<float, double>(*p, *px, G, &w.totals[0], time, O, S, s)));
  else
    CK((launch_sipm<double, double>(*p, *px, G, &w.totals[0], time, O, S, s)));
  {
    crv::Mark mark_("k_counts_total", s);
    k_counts_total<<<grid_for(ngroups, 256, 8), 256, 0, s>>>(&w.totals[0], w.nmain, w.nap, w.ntot);
  }
  CK(cudaGetLastError());
  CK(exclusive_scan(w.ntot, ngroups, Identity(), w.out_off, &w.totals[3], w.parts, s));
  {
    crv::Mark mark_("k_check_caps", s);
    k_check_caps<<<1, 32, 0, s>>>(&w.totals[3], out_cap, CRV_NEED_CHARGES_OUT, S);
  }
  {
    crv::Mark mark_("k_charge_compact", s);
    k_charge_compact<<<grid_for(ngroups, 8, 16), 256, 0, s>>>(&w.totals[0], G.label, w.slot_off, w.slot_cap, w.nmain,
                                                               w.nap, w.out_off, w.slot_t, w.slot_v, w.slot_id,
                                                               p->capacitance, p->overvoltage, p->precision == 1,
                                                            *out, out_cap);
  }
  CK(cudaGetLastError());
  if (g_charges)
    CK(cudaMemcpyAsync(g_charges, w.ntot, sizeof(int32_t) * ngroups, cudaMemcpyDeviceToDevice, s));
  {
    crv::Mark mark_("k_copy_i64", s);
    k_copy_i64<<<1, 1, 0, s>>>(&w.totals[3], reinterpret_cast<long long*>(n_out_dev));
  }
  CK(cudaGetLastError());
  return CRV_OK;
}

// ---- chain.digis ---------------------------------------------------------------------------------------------------

namespace crv {
struct DigiWs {
  int32_t *head, *gcount, *g_bound, *g_maxlen, *g_nkept, *dn;
  WfCluster* cl;                 // kept clusters by charge row (shares the group index memory, free after grouping)
  long long *gidx, *gstart, *glabel, *slot_off, *out_off, *parts, *totals;
  uint32_t* grun;
  double* g_tdc0;
  DigiSlots D;
  long long sc;
};

static DigiWs digi_layout(char* base, long long nq, long long slot_cap, int zs, size_t* bytes) {
  Carve c{base};
  DigiWs w;
  w.sc = slot_cap;
  w.head = c.take<int32_t>(nq);
  static_assert(sizeof(WfCluster) == 4 * sizeof(long long), "cluster record size");
  w.gidx = c.take<long long>(4 * nq);
  w.cl = reinterpret_cast<WfCluster*>(w.gidx);
  w.gstart = c.take<long long>(nq);
  w.glabel = c.take<long long>(nq);
  w.gcount = c.take<int32_t>(nq);
  w.grun = c.take<uint32_t>(nq);
  w.g_tdc0 = c.take<double>(nq);
  w.g_bound = c.take<int32_t>(nq);
  w.g_maxlen = c.take<int32_t>(nq);
  w.g_nkept = c.take<int32_t>(nq);
  w.slot_off = c.take<long long>(nq);
  w.dn = c.take<int32_t>(nq);
  w.out_off = c.take<long long>(nq);
  w.parts = c.take<long long>(scan_parts_len(nq) + 1);
  w.totals = c.take<long long>(8);
  w.D.off = w.slot_off;
  w.D.cap = w.g_bound;
  w.D.n = w.dn;
  w.D.chan = c.take<long long>(slot_cap);
  w.D.start = c.take<double>(slot_cap);
  w.D.tdc0 = c.take<double>(slot_cap);
  w.D.starttdc = c.take<long long>(slot_cap);
  w.D.volt = c.take<double>(slot_cap * zs);
  w.D.adc = c.take<int16_t>(slot_cap * zs);
  *bytes = c.off + 256;
  return w;
}
}  // namespace crv

extern "C" int64_t crv_digis_workspace(const CrvParams* p, int64_t ncharges, int64_t slot_cap) {
  if (!p || ncharges < 0 || slot_cap < 0 || p->samples_zs <= 0 || p->samples_zs > 32) return -1;
  size_t b = 0;
  digi_layout(nullptr, ncharges, slot_cap, p->samples_zs, &b);
  return (int64_t)b;
}

static int digis_run(const CrvParams* p, const CrvChannels* ch, int64_t ncharges, const long long* nq_dev,
                     const int64_t* label, const double* time, const double* charge, const double* tdc0_rows,
                     const double* tmpl, int32_t tlen,
                     const int64_t* ev_keys, const uint32_t* ev_runs, int64_t n_events, int64_t slot_cap,
                     CrvDigis* out, int64_t out_cap, int64_t* n_out_dev, void* workspace, int64_t workspace_bytes,
                     void* stream, CrvStatus* status_dev) {
  if (!p || !ch || !out || !n_out_dev || !status_dev || ncharges < 0 || slot_cap < 0 || out_cap < 0) return CRV_ERR_ARG;
  if (p->samples_zs <= 0 || p->samples_zs > 32 || tlen <= 0 || !tmpl) return CRV_ERR_ARG;
  if (p->precision == 1 && tlen > 1024) return CRV_ERR_ARG;      // FP32-mixed: template copy in shared memory
  if (ncharges > 0 && (!label || !time || !charge)) return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (ncharges == 0) {
    CK(cudaMemsetAsync(n_out_dev, 0, sizeof(long long), s));
    return CRV_OK;
  }
  size_t need = 0;
  digi_layout(nullptr, ncharges, slot_cap, p->samples_zs, &need);
  if (!workspace || (long long)need > workspace_bytes) return CRV_ERR_ARG;
  Status* S = reinterpret_cast<Status*>(status_dev);
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  size_t dummy;
  DigiWs w = digi_layout(base, ncharges, slot_cap, p->samples_zs, &dummy);
  if (!out->volt) w.D.volt = nullptr;       // volts not asked for: the slots keep none either
  const long long* lab = reinterpret_cast<const long long*>(label);
  CK(cudaMemsetAsync(w.totals, 0, 8 * sizeof(long long), s));
  CK(cudaMemsetAsync(w.g_maxlen, 0, sizeof(int32_t) * ncharges, s));
  CK(cudaMemsetAsync(w.g_bound, 0, sizeof(int32_t) * ncharges, s));
  CK(cudaMemsetAsync(w.dn, 0, sizeof(int32_t) * ncharges, s));
  unsigned gq = grid_for(ncharges, 256, 8);
  {
    crv::Mark mark_("k_label_heads", s);
    k_label_heads<<<gq, 256, 0, s>>>(ncharges, nq_dev, lab, w.head);
  }
  CK(exclusive_scan(w.head, ncharges, Identity(), w.gidx, &w.totals[0], w.parts, s, nq_dev));
  {
    crv::Mark mark_("k_label_groups", s);
    k_label_groups<<<gq, 256, 0, s>>>(ncharges, nq_dev, lab, w.head, w.gidx, w.gstart, w.glabel);
  }
  {
    crv::Mark mark_("k_group_counts", s);
    k_group_counts<<<gq, 256, 0, s>>>(&w.totals[0], ncharges, nq_dev, w.gstart, w.glabel, w.gcount,
                                      reinterpret_cast<const long long*>(ev_keys), ev_runs, n_events, w.grun, S);
  }
  CK(cudaGetLastError());
  WfGroups G{&w.totals[0], w.gstart, w.gcount, w.glabel, w.grun};
  if (p->precision == 1)
    CK(launch_wf_prepass<float>(*p, *ch, G, ncharges, time, tmpl, tlen, tdc0_rows, w.g_tdc0, w.g_bound,
                                w.g_maxlen, w.g_nkept, w.cl, w.head, S, s));
  else
    CK(launch_wf_prepass<double>(*p, *ch, G, ncharges, time, tmpl, tlen, tdc0_rows, w.g_tdc0, w.g_bound,
                                 w.g_maxlen, w.g_nkept, w.cl, w.head, S, s));
  CK(exclusive_scan(w.g_bound, ncharges, Identity(), w.slot_off, &w.totals[1], w.parts, s, &w.totals[0]));
  {
    crv::Mark mark_("k_check_caps", s);
    k_check_caps<<<1, 32, 0, s>>>(&w.totals[1], slot_cap, CRV_NEED_DIGIS, S);
  }
  // synthesis only when the slots fit: guard by zeroing the group count otherwise
  {
    crv::Mark mark_("k_guard_groups", s);
    k_guard_groups<<<1, 32, 0, s>>>(&w.totals[1], slot_cap, &w.totals[0], &w.totals[2]);
  }
  CK(cudaGetLastError());
  G.n = &w.totals[2];
  if (p->precision == 1)
    CK(launch_wf_synth<float>(*p, G, ncharges, time, charge, tmpl, tlen, tdc0_rows, w.g_tdc0, w.g_maxlen,
                              w.g_nkept, w.cl, w.D, S, s));
  else
    CK(launch_wf_synth<double>(*p, G, ncharges, time, charge, tmpl, tlen, tdc0_rows, w.g_tdc0, w.g_maxlen,
                               w.g_nkept, w.cl, w.D, S, s));
  CK(exclusive_scan(w.dn, ncharges, Identity(), w.out_off, &w.totals[3], w.parts, s, &w.totals[2]));
  {
    crv::Mark mark_("k_check_caps", s);
    k_check_caps<<<1, 32, 0, s>>>(&w.totals[3], out_cap, CRV_NEED_DIGIS_OUT, S);
  }
  Digis O{reinterpret_cast<long long*>(out->chan), out->start, out->tdc0, reinterpret_cast<long long*>(out->starttdc),
          out->volt, out->adc};
  {
    crv::Mark mark_("k_digi_compact", s);
    k_digi_compact<<<grid_for(ncharges, 8, 16), 256, 0, s>>>(&w.totals[2], w.D, w.out_off, p->samples_zs, O, out_cap);
  }
  {
    crv::Mark mark_("k_copy_i64", s);
    k_copy_i64<<<1, 1, 0, s>>>(&w.totals[3], reinterpret_cast<long long*>(n_out_dev));
  }
  CK(cudaGetLastError());
  return CRV_OK;
}

extern "C" int crv_digis(const CrvParams* p, const CrvChannels* ch, int64_t ncharges, const int64_t* label,
                         const double* time, const double* charge, const double* tmpl, int32_t tlen,
                         const int64_t* ev_keys, const uint32_t* ev_runs, int64_t n_events, int64_t slot_cap,
                         CrvDigis* out, int64_t out_cap, int64_t* n_out_dev, void* workspace, int64_t workspace_bytes,
                         void* stream, CrvStatus* status_dev) {
  return digis_run(p, ch, ncharges, nullptr, label, time, charge, nullptr, tmpl, tlen, ev_keys, ev_runs, n_events,
                   slot_cap, out, out_cap, n_out_dev, workspace, workspace_bytes, stream, status_dev);
}

extern "C" int crv_synthesize(const CrvParams* p, const CrvChannels* ch, int64_t ncharges, const int64_t* label,
                              const double* time, const double* charge, const double* tdc0_rows, const double* tmpl,
                              int32_t tlen, int64_t slot_cap, CrvDigis* out, int64_t out_cap, int64_t* n_out_dev,
                              void* workspace, int64_t workspace_bytes, void* stream, CrvStatus* status_dev) {
  if (ncharges > 0 && !tdc0_rows) return CRV_ERR_ARG;
  return digis_run(p, ch, ncharges, nullptr, label, time, charge, tdc0_rows, tmpl, tlen, nullptr, nullptr, 0,
                   slot_cap, out, out_cap, n_out_dev, workspace, workspace_bytes, stream, status_dev);
}

namespace crv {
__global__ void k_tdc0_labels(CrvParams p, CrvChannels ch, long long n, const long long* __restrict__ label,
                              const long long* __restrict__ ev_keys, const uint32_t* __restrict__ ev_runs,
                              long long n_ev, double* __restrict__ out, Status* status) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long lab = label[i];
    const long long c = lab % 32768;
    if (lab < 0 || c >= ch.nchan) {
      set_flag(status, CRV_ST_ORDER);
      out[i] = 0.0;
      continue;
    }
    uint32_t r = 0;
    if (ev_keys && n_ev > 0) {
      const long long k = lab / 32768;
      long long lo = 0, hi = n_ev;
      while (lo < hi) {
        long long m = (lo + hi) >> 1;
        if (ev_keys[m] < k) lo = m + 1; else hi = m;
      }
      if (lo < n_ev && ev_keys[lo] == k) r = ev_runs[lo];
      else set_flag(status, CRV_ST_ORDER);
    }
    out[i] = tdc0_of(p, ch, lab, r);
  }
}
}  // namespace crv

extern "C" int crv_tdc0_per_feb(const CrvParams* p, const CrvChannels* ch, int64_t nlabels, const int64_t* labels,
                                const int64_t* ev_keys, const uint32_t* ev_runs, int64_t n_events, double* tdc0,
                                void* stream, CrvStatus* status_dev) {
  if (!p || !ch || !status_dev || nlabels < 0 || n_events < 0) return CRV_ERR_ARG;
  if (nlabels == 0) return CRV_OK;
  if (!labels || !tdc0 || (n_events > 0 && (!ev_keys || !ev_runs))) return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  {
    crv::Mark mark_("k_tdc0_labels", s);
    k_tdc0_labels<<<grid_for(nlabels, 256, 8), 256, 0, s>>>(*p, *ch, nlabels, reinterpret_cast<const long long*>(labels),
                                                           reinterpret_cast<const long long*>(ev_keys), ev_runs,
                                                           n_events, tdc0, reinterpret_cast<Status*>(status_dev));
  }
  CK(cudaGetLastError());
  return CRV_OK;
}

// ---- pulsefit.reconstruct -----------------------------------------------------------------------------------------

namespace crv {
struct PulseWs {
  double* yscr;
  PulseRec* rec;
  long long *slot_off, *out_off, *parts, *totals;
  int32_t *cap, *count;
  long long rc;
  PfQueue q;
};

// round launches over the task list before the tail launch finishes what is left lane by lane (the counts array
// has room for the largest setting)
constexpr int kPulseRoundsMax = 32;

// launch shape of the fit rounds for later crv_pulses calls of this process (crv_pulses_shape)
struct PulseShape {
  std::atomic<int> threads{128}, blocks_per_sm{16}, rounds{0};
};
static PulseShape g_pulse_shape;

// record slots of waveform w: min(max_pulses, n/2 + 1) (every round advances the search by at least two samples)
static long long pulse_slot_bound(long long nw, long long nsamples) { return nsamples / 2 + nw + 1; }

static PulseWs pulse_layout(char* base, long long nw, long long nsamples, size_t* bytes) {
  Carve c{base};
  PulseWs w;
  w.rc = pulse_slot_bound(nw, nsamples);
  w.yscr = c.take<double>(nsamples);
  w.rec = c.take<PulseRec>(w.rc);
  w.slot_off = c.take<long long>(nw);
  w.out_off = c.take<long long>(nw);
  w.parts = c.take<long long>(scan_parts_len(nw) + 1);
  w.totals = c.take<long long>(8);
  w.cap = c.take<int32_t>(nw);
  w.count = c.take<int32_t>(nw);
  w.q.st = c.take<PfState>(nw);
  w.q.list[0] = c.take<long long>(nw);
  w.q.list[1] = c.take<long long>(nw);
  w.q.counts = c.take<long long>(kPulseRoundsMax + 2);
  w.q.rounds = g_pulse_shape.rounds.load();
  w.q.threads = g_pulse_shape.threads.load();
  w.q.blocks_per_sm = g_pulse_shape.blocks_per_sm.load();
  *bytes = c.off + 256;
  return w;
}

__global__ void k_pulse_caps(long long nw, const long long* __restrict__ nw_dev, const long long* __restrict__ off,
                             const int32_t* __restrict__ n, long long nsamples, int max_pulses,
                             int32_t* __restrict__ cap) {
  nw = bounded_count(nw, nw_dev);
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < nw; w += (long long)gridDim.x * blockDim.x) {
    if (!wave_in_bounds(off[w], n[w], nsamples)) {     // no slots: the fit skips it and reports CRV_ST_BOUNDS
      cap[w] = 0;
      continue;
    }
    int b = n[w] / 2 + 1;
    cap[w] = b < max_pulses ? b : max_pulses;
  }
}

__global__ void k_pulse_compact(long long nw, const long long* __restrict__ nw_dev,
                                const long long* __restrict__ slot_off, const int32_t* __restrict__ count,
                                const long long* __restrict__ out_off, const PulseRec* __restrict__ rec,
                                CrvPulses O, long long out_cap) {
  nw = bounded_count(nw, nw_dev);
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < nw; w += (long long)gridDim.x * blockDim.x) {
    int c = count[w];
    long long o0 = out_off[w], b0 = slot_off[w];
    if (o0 + c > out_cap) continue;
    for (int k = 0; k < c; ++k) {
      const PulseRec& r = rec[b0 + k];
      long long o = o0 + k;
      O.wf[o] = w; O.seq[o] = r.seq;
      O.pe[o] = r.pe; O.peph[o] = r.peph; O.time[o] = r.time; O.height[o] = r.height; O.beta[o] = r.beta;
      O.chi2[o] = r.chi2; O.letime[o] = r.letime; O.ped[o] = r.ped;
      O.fit_A[o] = r.A; O.fit_mu[o] = r.mu; O.fit_b[o] = r.b;
      O.failed[o] = r.failed; O.zerondf[o] = r.zerondf; O.pedfromdb[o] = r.pedfromdb;
    }
  }
}
}  // namespace crv

extern "C" int crv_pulses_shape(int32_t threads, int32_t blocks_per_sm, int32_t rounds) {
  if ((threads != 64 && threads != 128) || blocks_per_sm < 1 || blocks_per_sm > 32 || rounds < 0 ||
      rounds > kPulseRoundsMax)
    return CRV_ERR_ARG;
  g_pulse_shape.threads.store(threads);
  g_pulse_shape.blocks_per_sm.store(blocks_per_sm);
  g_pulse_shape.rounds.store(rounds);
  return CRV_OK;
}

extern "C" int64_t crv_pulses_workspace(const CrvParams* p, int64_t nw, int64_t nsamples) {
  if (!p || nw < 0 || nsamples < 0) return -1;
  size_t b = 0;
  pulse_layout(nullptr, nw, nsamples, &b);
  return (int64_t)b;
}

static int pulses_run(const CrvParams* p, int64_t nw, const long long* nw_dev, int64_t nsamples, const int64_t* off,
                      const int32_t* n, const int64_t* start_tdc, const double* ped_db, const double* area,
                      const double* height, const int16_t* adc16, const int64_t* adc64, int32_t max_pulses,
                      CrvPulses* out, int64_t out_cap, int64_t* n_out_dev, uint8_t* wf_near, void* workspace,
                      int64_t workspace_bytes, void* stream, CrvStatus* status_dev) {
  if (!p || !out || !n_out_dev || !status_dev || nw < 0 || nsamples < 0 || out_cap < 0 || max_pulses < 0)
    return CRV_ERR_ARG;
  if (nw > 0 && (!off || !n || !start_tdc || !ped_db || !area || !height || !wf_near || (!adc16 == !adc64)))
    return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (nw == 0) {
    CK(cudaMemsetAsync(n_out_dev, 0, sizeof(long long), s));
    return CRV_OK;
  }
  size_t need = 0;
  pulse_layout(nullptr, nw, nsamples, &need);
  if (!workspace || (long long)need > workspace_bytes) return CRV_ERR_ARG;
  Status* S = reinterpret_cast<Status*>(status_dev);
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  size_t dummy;
  PulseWs w = pulse_layout(base, nw, nsamples, &dummy);
  CK(cudaMemsetAsync(w.totals, 0, 8 * sizeof(long long), s));
  CK(cudaMemsetAsync(w.q.counts, 0, (kPulseRoundsMax + 2) * sizeof(long long), s));
  unsigned g = grid_for(nw, 256, 8);
  {
    crv::Mark mark_("k_pulse_caps", s);
    k_pulse_caps<<<g, 256, 0, s>>>(nw, nw_dev, reinterpret_cast<const long long*>(off), n, nsamples, max_pulses,
                                   w.cap);
  }
  CK(exclusive_scan(w.cap, nw, Identity(), w.slot_off, &w.totals[0], w.parts, s, nw_dev));
  WaveIn W{nw, nw_dev, reinterpret_cast<const long long*>(off), n, reinterpret_cast<const long long*>(start_tdc), ped_db,
           area, height, adc16, reinterpret_cast<const long long*>(adc64), nsamples};
  PulseSlots PS{w.slot_off, w.cap, w.count, wf_near, w.rec, w.rc};
  if (p->precision == 1)
    CK(launch_pulsefit<float>(*p, W, w.yscr, max_pulses, PS, w.q, S, s));
  else
    CK(launch_pulsefit<double>(*p, W, w.yscr, max_pulses, PS, w.q, S, s));
  CK(exclusive_scan(w.count, nw, Identity(), w.out_off, &w.totals[1], w.parts, s, nw_dev));
  {
    crv::Mark mark_("k_check_caps", s);
    k_check_caps<<<1, 32, 0, s>>>(&w.totals[1], out_cap, CRV_NEED_PULSES_OUT, S);
  }
  {
    crv::Mark mark_("k_pulse_compact", s);
    k_pulse_compact<<<g, 256, 0, s>>>(nw, nw_dev, w.slot_off, w.count, w.out_off, w.rec, *out, out_cap);
  }
  {
    crv::Mark mark_("k_copy_i64", s);
    k_copy_i64<<<1, 1, 0, s>>>(&w.totals[1], reinterpret_cast<long long*>(n_out_dev));
  }
  CK(cudaGetLastError());
  return CRV_OK;
}

extern "C" int crv_pulses(const CrvParams* p, int64_t nw, int64_t nsamples, const int64_t* off, const int32_t* n,
                          const int64_t* start_tdc, const double* ped_db, const double* area, const double* height,
                          const int16_t* adc16, const int64_t* adc64, int32_t max_pulses, CrvPulses* out,
                          int64_t out_cap, int64_t* n_out_dev, uint8_t* wf_near, void* workspace,
                          int64_t workspace_bytes, void* stream, CrvStatus* status_dev) {
  return pulses_run(p, nw, nullptr, nsamples, off, n, start_tdc, ped_db, area, height, adc16, adc64, max_pulses, out,
                    out_cap, n_out_dev, wf_near, workspace, workspace_bytes, stream, status_dev);
}

// ---- coincidences ---------------------------------------------------------------------------------------------------

namespace crv {
static_assert(sizeof(CrvFinderGeom) == sizeof(CoincGeom), "finder geometry layout");

struct CoincWs {
  ClusterRec* rec;
  int32_t *mem_idx, *ncl, *nmem, *deferred;
  long long *cl_off, *mem_off, *parts, *totals;
  char* gscratch;                // per-event lists of the global-memory pass
};

static CoincWs coinc_layout(char* base, long long nev, long long np, size_t* bytes) {
  Carve c{base};
  CoincWs w;
  w.rec = c.take<ClusterRec>(np);
  w.mem_idx = c.take<int32_t>(np);
  w.ncl = c.take<int32_t>(nev);
  w.nmem = c.take<int32_t>(nev);
  w.deferred = c.take<int32_t>(nev);
  w.cl_off = c.take<long long>(nev);
  w.mem_off = c.take<long long>(nev);
  w.parts = c.take<long long>(scan_parts_len(nev) + 1);
  w.totals = c.take<long long>(8);
  // event e's region of the global pass: (ev_count + 16) * COINC_GBYTES bytes, at least the per-warp layout of
  // hcap = ev_count rounded up to 16 (103 B per hit plus under 250 B of alignment and counters)
  w.gscratch = c.take<char>((np + 16 * nev + 1) * (long long)COINC_GBYTES);
  *bytes = c.off + 256;
  return w;
}

__global__ void k_coinc_compact(long long nev, const long long* __restrict__ nev_dev,
                                const long long* __restrict__ ev_start, const long long* __restrict__ ev_key,
                                const int32_t* __restrict__ ncl, const long long* __restrict__ cl_off,
                                const long long* __restrict__ mem_off, const ClusterRec* __restrict__ rec,
                                const int32_t* __restrict__ mem_idx, CrvClusters O, long long cl_cap, CrvMembers M,
                                long long mem_cap) {
  nev = bounded_count(nev, nev_dev);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nev; e += (long long)gridDim.x * blockDim.x) {
    long long r0 = ev_start[e];
    for (int k = 0; k < ncl[e]; ++k) {
      const ClusterRec& R = rec[r0 + k];
      long long o = cl_off[e] + k;
      if (o >= cl_cap) break;
      O.event[o] = ev_key[e];
      O.type[o] = R.type;
      O.pe[o] = R.pe; O.start[o] = R.start; O.end[o] = R.end; O.slope[o] = R.slope; O.avgtime[o] = R.avgtime;
      O.poscalc[o] = uint8_t(R.poscalc);
      for (int c = 0; c < 3; ++c) O.pos[o * 3 + c] = R.pos[c];
      for (int sd = 0; sd < 2; ++sd) {
        O.sidepe[o * 2 + sd] = R.sidepe[sd];
        O.sidetime[o * 2 + sd] = R.sidetime[sd];
        O.sidehits[o * 2 + sd] = R.sidehits[sd];
      }
      O.nlayers[o] = R.nlayers;
      for (int z = 0; z < R.mem_count; ++z) {
        long long q = mem_off[e] + R.mem_begin + z;
        if (q >= mem_cap) break;
        M.cl[q] = o;
        M.idx[q] = mem_idx[r0 + R.mem_begin + z];
        M.event[q] = ev_key[e];
      }
    }
  }
}
}  // namespace crv

extern "C" int64_t crv_coincidences_workspace(int64_t nevents, int64_t npulses) {
  if (nevents < 0 || npulses < 0) return -1;
  size_t b = 0;
  coinc_layout(nullptr, nevents, npulses, &b);
  return (int64_t)b;
}

static int coinc_run(const CrvParams* p, const CrvFinderGeom* g, int64_t nevents, const long long* nev_dev,
                     const int64_t* ev_start, const int32_t* ev_count, const int64_t* ev_key, int64_t npulses,
                     const int32_t* bar, const int32_t* sipm, const int32_t* seq, const double* time, const double* pe,
                     const int32_t* status, CrvClusters* out, int64_t cl_cap, int64_t* n_cl_dev, CrvMembers* mem,
                     int64_t mem_cap, int64_t* n_mem_dev, void* workspace, int64_t workspace_bytes, void* stream,
                     CrvStatus* status_dev) {
  if (!p || !g || !out || !mem || !n_cl_dev || !n_mem_dev || !status_dev || nevents < 0 || npulses < 0) return CRV_ERR_ARG;
  if (nevents > 0 && (!ev_start || !ev_count || !ev_key)) return CRV_ERR_ARG;
  if (npulses > 0 && (!bar || !sipm || !seq || !time || !pe || !status)) return CRV_ERR_ARG;
  if (g->ntypes < 0) return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (nevents == 0) {
    CK(cudaMemsetAsync(n_cl_dev, 0, sizeof(long long), s));
    CK(cudaMemsetAsync(n_mem_dev, 0, sizeof(long long), s));
    return CRV_OK;
  }
  size_t need = 0;
  coinc_layout(nullptr, nevents, npulses, &need);
  if (!workspace || (long long)need > workspace_bytes) return CRV_ERR_ARG;
  Status* S = reinterpret_cast<Status*>(status_dev);
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  size_t dummy;
  CoincWs w = coinc_layout(base, nevents, npulses, &dummy);
  CK(cudaMemsetAsync(w.totals, 0, 8 * sizeof(long long), s));
  CK(cudaMemsetAsync(w.ncl, 0, sizeof(int32_t) * nevents, s));
  CK(cudaMemsetAsync(w.nmem, 0, sizeof(int32_t) * nevents, s));
  CK(cudaMemsetAsync(w.deferred, 0, sizeof(int32_t) * nevents, s));
  CoincGeom G;
  memcpy(&G, g, sizeof(G));
  CoincIn I{nevents, nev_dev, reinterpret_cast<const long long*>(ev_start), ev_count, bar, sipm, seq, time, pe, status};
  CoincOut O{w.rec, w.mem_idx, w.ncl, w.nmem};
  const DeviceInfo& di = device_info();
  // events up to 192 hits (nearly all) at one warp per block (~11 resident warps per SM); the larger ones in a pass
  // with their lists in global memory (many warps per SM, where a 1024-hit shared-memory pass fits two)
  struct Pass { int hcap, warps; } passes[3] = {{192, 1}, {1024, 1}, {0, 1}};
  for (int k = 0; k < 3; ++k) {
    if (k == 1) continue;
    size_t per = k < 2 ? coinc_smem_per_warp(passes[k].hcap) + coinc_work_per_warp(passes[k].hcap) : 0;
    size_t smem = per * passes[k].warps;
    if (smem > di.smem_optin - 1024) return CRV_ERR_CUDA;
    long long blocks = (nevents + passes[k].warps - 1) / passes[k].warps;
    // the global pass (118 registers: 16 one-warp blocks per SM) sees the few large events of a batch, or every event
    // at full scale (~11,000 hits each)
    long long maxb = (long long)di.sms * (k == 0 ? 16 : (k == 1 ? 2 : 16));
    const unsigned grid = (unsigned)(blocks < maxb ? blocks : maxb);
    if (k < 2) {
      CK(allow_dynamic_smem(k_coinc<false>));
      crv::Mark mark_("k_coinc", s);
      k_coinc<false><<<grid, passes[k].warps * 32, smem, s>>>(*p, G, I, passes[k].hcap, k, O, w.deferred, w.gscratch,
                                                             S);
    } else {
      crv::Mark mark_("k_coinc_global", s);
      k_coinc<true><<<grid, passes[k].warps * 32, 0, s>>>(*p, G, I, 0, k, O, w.deferred, w.gscratch, S);
    }
    CK(cudaGetLastError());
  }
  CK(exclusive_scan(w.ncl, nevents, Identity(), w.cl_off, &w.totals[0], w.parts, s, nev_dev));
  CK(exclusive_scan(w.nmem, nevents, Identity(), w.mem_off, &w.totals[1], w.parts, s, nev_dev));
  {
    crv::Mark mark_("k_check_caps", s);
    k_check_caps<<<1, 32, 0, s>>>(&w.totals[0], cl_cap, CRV_NEED_CLUSTERS, S);
  }
  {
    crv::Mark mark_("k_check_caps", s);
    k_check_caps<<<1, 32, 0, s>>>(&w.totals[1], mem_cap, CRV_NEED_MEMBERS, S);
  }
  {
    crv::Mark mark_("k_coinc_compact", s);
    k_coinc_compact<<<grid_for(nevents, 256, 8), 256, 0, s>>>(nevents, nev_dev,
                                                            reinterpret_cast<const long long*>(ev_start),
                                                            reinterpret_cast<const long long*>(ev_key), w.ncl, w.cl_off,
                                                            w.mem_off, w.rec, w.mem_idx, *out, cl_cap, *mem, mem_cap);
  }
  {
    crv::Mark mark_("k_copy_i64", s);
    k_copy_i64<<<1, 1, 0, s>>>(&w.totals[0], reinterpret_cast<long long*>(n_cl_dev));
  }
  {
    crv::Mark mark_("k_copy_i64", s);
    k_copy_i64<<<1, 1, 0, s>>>(&w.totals[1], reinterpret_cast<long long*>(n_mem_dev));
  }
  CK(cudaGetLastError());
  return CRV_OK;
}

extern "C" int crv_coincidences(const CrvParams* p, const CrvFinderGeom* g, int64_t nevents, const int64_t* ev_start,
                                const int32_t* ev_count, const int64_t* ev_key, int64_t npulses, const int32_t* bar,
                                const int32_t* sipm, const int32_t* seq, const double* time, const double* pe,
                                const int32_t* status, CrvClusters* out, int64_t cl_cap, int64_t* n_cl_dev,
                                CrvMembers* mem, int64_t mem_cap, int64_t* n_mem_dev, void* workspace,
                                int64_t workspace_bytes, void* stream, CrvStatus* status_dev) {
  return coinc_run(p, g, nevents, nullptr, ev_start, ev_count, ev_key, npulses, bar, sipm, seq, time, pe, status, out,
                   cl_cap, n_cl_dev, mem, mem_cap, n_mem_dev, workspace, workspace_bytes, stream, status_dev);
}

// ---- reco waveforms and pulse glue ---------------------------------------------------------------------------------

namespace crv {
__global__ void k_wf_heads(long long nd, const long long* __restrict__ nd_dev, const long long* __restrict__ label,
                           const long long* __restrict__ tdc, int zs, int32_t* __restrict__ head) {
  nd = bounded_count(nd, nd_dev);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x)
    head[i] = (i == 0 || label[i] != label[i - 1] || tdc[i] != tdc[i - 1] + zs) ? 1 : 0;
}

__global__ void k_wf_fill(long long nd, const long long* __restrict__ nd_dev, const long long* __restrict__ label,
                          const long long* __restrict__ tdc, int zs, const int32_t* __restrict__ head,
                          const long long* __restrict__ gidx, CrvChannels ch, long long* __restrict__ w_label,
                          long long* __restrict__ w_off, int32_t* __restrict__ w_n, long long* __restrict__ w_start,
                          double* __restrict__ w_ped, double* __restrict__ w_area, double* __restrict__ w_height,
                          double* __restrict__ w_toff) {
  nd = bounded_count(nd, nd_dev);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x) {
    if (!head[i]) continue;
    long long g = gidx[i];
    long long j = i + 1;
    while (j < nd && !head[j]) ++j;
    int c = int(label[i] % 32768);
    w_label[g] = label[i];
    w_off[g] = i * zs;
    w_n[g] = int32_t((j - i) * zs);
    w_start[g] = tdc[i];
    w_ped[g] = ch.pedestal[c];
    w_area[g] = ch.pulsearea[c];
    w_height[g] = ch.pulseheight[c];
    w_toff[g] = ch.timeoffset[c];
  }
}

__global__ void k_hit_keep(const CrvParams p, const int32_t* __restrict__ status, const long long* __restrict__ w_label,
                           long long np, const long long* __restrict__ np_dev, const long long* __restrict__ p_wf,
                           int32_t* __restrict__ keep) {
  np = bounded_count(np, np_dev);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < np; i += (long long)gridDim.x * blockDim.x) {
    int c = int(w_label[p_wf[i]] % 32768);
    keep[i] = (p.ignore_channels && (status[c] & 0b010)) ? 0 : 1;
  }
}

__global__ void k_hit_fill(const CrvParams p, const long long* __restrict__ w_label, const double* __restrict__ w_toff,
                           const double* __restrict__ event_t0, long long np, const long long* __restrict__ np_dev,
                           const long long* __restrict__ p_wf, const long long* __restrict__ p_seq,
                           const double* __restrict__ p_time, const double* __restrict__ p_pe,
                           const int32_t* __restrict__ keep, const long long* __restrict__ kidx,
                           int32_t* __restrict__ bar, int32_t* __restrict__ sipm, int32_t* __restrict__ seq,
                           double* __restrict__ time, double* __restrict__ pe, long long* __restrict__ hev) {
  np = bounded_count(np, np_dev);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < np; i += (long long)gridDim.x * blockDim.x) {
    if (!keep[i]) continue;
    long long k = kidx[i];
    long long w = p_wf[i];
    long long lab = w_label[w];
    int c = int(lab % 32768);
    double t = p_time[i];
    if (p.use_time_offset_db) t = t + w_toff[w] * p.time_offset_scale;
    if (event_t0) t = t + event_t0[w];
    bar[k] = c / 4;
    sipm[k] = c % 4;
    seq[k] = int32_t(p_seq[i]);
    time[k] = t;
    pe[k] = p_pe[i];
    hev[k] = lab / 32768;
  }
}

__global__ void k_ev_heads(const long long* __restrict__ n_dev, const long long* __restrict__ hev,
                           int32_t* __restrict__ head) {
  long long n = *n_dev;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    head[i] = (i == 0 || hev[i] != hev[i - 1]) ? 1 : 0;
}

__global__ void k_ev_fill(const long long* __restrict__ n_dev, const long long* __restrict__ hev,
                          const int32_t* __restrict__ head, const long long* __restrict__ eidx,
                          long long* __restrict__ ev_start, int32_t* __restrict__ ev_count,
                          long long* __restrict__ ev_key) {
  long long n = *n_dev;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (!head[i]) continue;
    long long e = eidx[i];
    long long j = i + 1;
    while (j < n && !head[j]) ++j;
    ev_start[e] = i;
    ev_count[e] = int32_t(j - i);
    ev_key[e] = hev[i];
  }
}
}  // namespace crv

extern "C" int64_t crv_reco_waveforms_workspace(int64_t nd) {
  if (nd < 0) return -1;
  Carve c{nullptr};
  c.take<int32_t>(nd);
  c.take<long long>(nd);
  c.take<long long>(scan_parts_len(nd) + 1);
  c.take<long long>(8);
  return (int64_t)(c.off + 256);
}

static int reco_waveforms_run(const CrvParams* p, const CrvChannels* ch, int64_t nd, const long long* nd_dev,
                              const int64_t* label, const int64_t* starttdc, int64_t* w_label, int64_t* w_off,
                              int32_t* w_n, int64_t* w_start, double* w_ped, double* w_area, double* w_height,
                              double* w_toff, int64_t* n_w_dev, void* workspace, int64_t workspace_bytes, void* stream,
                              CrvStatus* status_dev) {
  if (!p || !ch || !n_w_dev || !status_dev || nd < 0) return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (nd == 0) {
    CK(cudaMemsetAsync(n_w_dev, 0, sizeof(long long), s));
    return CRV_OK;
  }
  if (crv_reco_waveforms_workspace(nd) > workspace_bytes || !workspace) return CRV_ERR_ARG;
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  Carve c{base};
  int32_t* head = c.take<int32_t>(nd);
  long long* gidx = c.take<long long>(nd);
  long long* parts = c.take<long long>(scan_parts_len(nd) + 1);
  long long* totals = c.take<long long>(8);
  const long long* lab = reinterpret_cast<const long long*>(label);
  const long long* tdc = reinterpret_cast<const long long*>(starttdc);
  unsigned g = grid_for(nd, 256, 8);
  {
    crv::Mark mark_("k_wf_heads", s);
    k_wf_heads<<<g, 256, 0, s>>>(nd, nd_dev, lab, tdc, p->samples_zs, head);
  }
  CK(exclusive_scan(head, nd, Identity(), gidx, &totals[0], parts, s, nd_dev));
  {
    crv::Mark mark_("k_wf_fill", s);
    k_wf_fill<<<g, 256, 0, s>>>(nd, nd_dev, lab, tdc, p->samples_zs, head, gidx, *ch,
                                reinterpret_cast<long long*>(w_label), reinterpret_cast<long long*>(w_off), w_n,
                                reinterpret_cast<long long*>(w_start), w_ped, w_area, w_height, w_toff);
  }
  {
    crv::Mark mark_("k_copy_i64", s);
    k_copy_i64<<<1, 1, 0, s>>>(&totals[0], reinterpret_cast<long long*>(n_w_dev));
  }
  CK(cudaGetLastError());
  return CRV_OK;
}

extern "C" int crv_reco_waveforms(const CrvParams* p, const CrvChannels* ch, int64_t nd, const int64_t* label,
                                  const int64_t* starttdc, int64_t* w_label, int64_t* w_off, int32_t* w_n,
                                  int64_t* w_start, double* w_ped, double* w_area, double* w_height, double* w_toff,
                                  int64_t* n_w_dev, void* workspace, int64_t workspace_bytes, void* stream,
                                  CrvStatus* status_dev) {
  return reco_waveforms_run(p, ch, nd, nullptr, label, starttdc, w_label, w_off, w_n, w_start, w_ped, w_area, w_height,
                            w_toff, n_w_dev, workspace, workspace_bytes, stream, status_dev);
}

extern "C" int64_t crv_pulse_hits_workspace(int64_t np) {
  if (np < 0) return -1;
  Carve c{nullptr};
  c.take<int32_t>(np);
  c.take<long long>(np);
  c.take<long long>(np);
  c.take<int32_t>(np);
  c.take<long long>(np);
  c.take<long long>(scan_parts_len(np) + 1);
  c.take<long long>(8);
  return (int64_t)(c.off + 256);
}

static int pulse_hits_run(const CrvParams* p, const int32_t* status, int64_t nw, const int64_t* w_label,
                          const double* w_toff, const double* event_t0, int64_t np, const long long* np_dev,
                          const int64_t* p_wf, const int64_t* p_seq, const double* p_time, const double* p_pe,
                          int64_t* ev_start, int32_t* ev_count, int64_t* ev_key, int32_t* bar, int32_t* sipm,
                          int32_t* seq, double* time, double* pe, int64_t* n_ev_dev, int64_t* n_hit_dev,
                          void* workspace, int64_t workspace_bytes, void* stream, CrvStatus* status_dev) {
  if (!p || !status || !n_ev_dev || !n_hit_dev || !status_dev || np < 0 || nw < 0) return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (np == 0) {
    CK(cudaMemsetAsync(n_ev_dev, 0, sizeof(long long), s));
    CK(cudaMemsetAsync(n_hit_dev, 0, sizeof(long long), s));
    return CRV_OK;
  }
  if (crv_pulse_hits_workspace(np) > workspace_bytes || !workspace) return CRV_ERR_ARG;
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  Carve c{base};
  int32_t* keep = c.take<int32_t>(np);
  long long* kidx = c.take<long long>(np);
  long long* hev = c.take<long long>(np);
  int32_t* head = c.take<int32_t>(np);
  long long* eidx = c.take<long long>(np);
  long long* parts = c.take<long long>(scan_parts_len(np) + 1);
  long long* totals = c.take<long long>(8);
  unsigned g = grid_for(np, 256, 8);
  const long long* wl = reinterpret_cast<const long long*>(w_label);
  {
    crv::Mark mark_("k_hit_keep", s);
    k_hit_keep<<<g, 256, 0, s>>>(*p, status, wl, np, np_dev, reinterpret_cast<const long long*>(p_wf), keep);
  }
  CK(exclusive_scan(keep, np, Identity(), kidx, &totals[0], parts, s, np_dev));
  {
    crv::Mark mark_("k_hit_fill", s);
    k_hit_fill<<<g, 256, 0, s>>>(*p, wl, w_toff, event_t0, np, np_dev, reinterpret_cast<const long long*>(p_wf),
                                 reinterpret_cast<const long long*>(p_seq), p_time, p_pe, keep, kidx, bar, sipm, seq,
                                 time, pe, hev);
  }
  // rows beyond the kept count stay 0 so the event scan counts kept pulses only
  CK(cudaMemsetAsync(head, 0, sizeof(int32_t) * np, s));
  {
    crv::Mark mark_("k_ev_heads", s);
    k_ev_heads<<<g, 256, 0, s>>>(&totals[0], hev, head);
  }
  CK(exclusive_scan(head, np, Identity(), eidx, &totals[1], parts, s));
  {
    crv::Mark mark_("k_ev_fill", s);
    k_ev_fill<<<g, 256, 0, s>>>(&totals[0], hev, head, eidx, reinterpret_cast<long long*>(ev_start), ev_count,
                                reinterpret_cast<long long*>(ev_key));
  }
  {
    crv::Mark mark_("k_copy_i64", s);
    k_copy_i64<<<1, 1, 0, s>>>(&totals[1], reinterpret_cast<long long*>(n_ev_dev));
  }
  {
    crv::Mark mark_("k_copy_i64", s);
    k_copy_i64<<<1, 1, 0, s>>>(&totals[0], reinterpret_cast<long long*>(n_hit_dev));
  }
  CK(cudaGetLastError());
  return CRV_OK;
}

extern "C" int crv_pulse_hits(const CrvParams* p, const int32_t* status, int64_t nw, const int64_t* w_label,
                              const double* w_toff, const double* event_t0, int64_t np, const int64_t* p_wf,
                              const int64_t* p_seq, const double* p_time, const double* p_pe, int64_t* ev_start,
                              int32_t* ev_count, int64_t* ev_key, int32_t* bar, int32_t* sipm, int32_t* seq,
                              double* time, double* pe, int64_t* n_ev_dev, int64_t* n_hit_dev, void* workspace,
                              int64_t workspace_bytes, void* stream, CrvStatus* status_dev) {
  return pulse_hits_run(p, status, nw, w_label, w_toff, event_t0, np, nullptr, p_wf, p_seq, p_time, p_pe, ev_start,
                        ev_count, ev_key, bar, sipm, seq, time, pe, n_ev_dev, n_hit_dev, workspace, workspace_bytes,
                        stream, status_dev);
}

// ---- the resident chain: steps -> clusters in one call with fixed capacities ----------------------------------------

namespace crv {
struct ChainWs {
  long long* counts;             // 0-9 raw stage counts (CRV_CHAIN_*), 16-25 the counts passed downstream
  CrvCharges Q;
  CrvDigis D;
  int64_t *w_label, *w_off, *w_start;
  int32_t* w_n;
  double *w_ped, *w_area, *w_height, *w_toff;
  CrvPulses P;
  uint8_t* near;
  int64_t *h_ev_start, *h_ev_key;
  int32_t *h_ev_count, *h_bar, *h_sipm, *h_seq;
  double *h_time, *h_pe;
  char* scratch;
  long long scratch_bytes;
};

static long long chain_scratch_bytes(const CrvParams& p, const CrvChainCaps& c, bool lookup) {
  long long zs = p.samples_zs;
  long long b = 0;
  auto up = [&](long long v) { if (v > b) b = v; };
  size_t r = 0;
  resp_layout(nullptr, p, c.events, c.steps, c.photons, &r, lookup);
  up((long long)r);
  digi_layout(nullptr, c.charges, c.slots, p.samples_zs, &r);
  up((long long)r);
  up(crv_reco_waveforms_workspace(c.digis));
  pulse_layout(nullptr, c.digis, c.digis * zs, &r);
  up((long long)r);
  up(crv_pulse_hits_workspace(c.pulses));
  coinc_layout(nullptr, c.events, c.pulses, &r);
  up((long long)r);
  return b;
}

static ChainWs chain_layout(char* base, const CrvParams& p, const CrvChainCaps& c, size_t* bytes, bool lookup = false) {
  Carve k{base};
  ChainWs w;
  const long long zs = p.samples_zs, nq = c.charges, nd = c.digis, np = c.pulses, ne = c.events;
  w.counts = k.take<long long>(32);
  w.Q.label = k.take<int64_t>(nq);
  w.Q.time = k.take<double>(nq);
  w.Q.charge = k.take<double>(nq);
  w.Q.pe = nullptr;                        // the chain's later stages read label, time and charge only
  w.Q.photon = nullptr;
  w.D.chan = k.take<int64_t>(nd);
  w.D.start = nullptr;                     // the chain's later stages read channel, start TDC and ADC only
  w.D.tdc0 = nullptr;
  w.D.starttdc = k.take<int64_t>(nd);
  w.D.volt = nullptr;
  w.D.adc = k.take<int16_t>(nd * zs);
  w.w_label = k.take<int64_t>(nd);
  w.w_off = k.take<int64_t>(nd);
  w.w_start = k.take<int64_t>(nd);
  w.w_n = k.take<int32_t>(nd);
  w.w_ped = k.take<double>(nd);
  w.w_area = k.take<double>(nd);
  w.w_height = k.take<double>(nd);
  w.w_toff = k.take<double>(nd);
  int64_t** pi[2] = {&w.P.wf, &w.P.seq};
  for (auto q : pi) *q = k.take<int64_t>(np);
  double** pf[11] = {&w.P.pe, &w.P.peph, &w.P.time, &w.P.height, &w.P.beta, &w.P.chi2, &w.P.letime, &w.P.ped,
                     &w.P.fit_A, &w.P.fit_mu, &w.P.fit_b};
  for (auto q : pf) *q = k.take<double>(np);
  uint8_t** pb[3] = {&w.P.failed, &w.P.zerondf, &w.P.pedfromdb};
  for (auto q : pb) *q = k.take<uint8_t>(np);
  w.near = k.take<uint8_t>(nd);
  w.h_ev_start = k.take<int64_t>(ne);
  w.h_ev_key = k.take<int64_t>(ne);
  w.h_ev_count = k.take<int32_t>(ne);
  w.h_bar = k.take<int32_t>(np);
  w.h_sipm = k.take<int32_t>(np);
  w.h_seq = k.take<int32_t>(np);
  w.h_time = k.take<double>(np);
  w.h_pe = k.take<double>(np);
  w.scratch_bytes = chain_scratch_bytes(p, c, lookup);
  w.scratch = k.take<char>(w.scratch_bytes);
  *bytes = k.off + 256;
  return w;
}

static bool chain_caps_ok(const CrvParams* p, const CrvChainCaps* c) {
  return p && c && c->events > 0 && c->steps > 0 && c->photons > 0 && c->charges > 0 && c->slots > 0 &&
         c->digis > 0 && c->pulses > 0 && c->max_steps_per_event > 0 && p->samples_zs > 0 && p->samples_zs <= 32;
}
}  // namespace crv

extern "C" int64_t crv_chain_workspace(const CrvParams* p, const CrvChainCaps* caps) {
  if (!chain_caps_ok(p, caps)) return -1;
  size_t b = 0;
  chain_layout(nullptr, *p, *caps, &b);
  return (int64_t)b;
}

extern "C" int64_t crv_chain_lookup_workspace(const CrvParams* p, const CrvChainCaps* caps) {
  if (!chain_caps_ok(p, caps)) return -1;
  size_t b = 0;
  chain_layout(nullptr, *p, *caps, &b, true);
  return (int64_t)b;
}

namespace crv {
static int chain_run(const CrvParams* p, const CrvChainCaps* caps, const CrvEvents* ev, const int64_t* ev_keys,
                     const uint32_t* ev_runs, const CrvSteps* st, const int64_t* nsteps_dev, const CrvBars* bars,
                     const CrvChannels* ch, const CrvPixels* px, const double* tmpl, int32_t tlen,
                     const CrvFinderGeom* g, CrvClusters* out, CrvMembers* mem, int64_t* counts_dev,
                     void* workspace, int64_t workspace_bytes, void* stream, CrvStatus* status_dev,
                     const CrvLookupChain* lk) {
  if (!chain_caps_ok(p, caps) || !ev || !ev_keys || !ev_runs || !st || !nsteps_dev || !bars || !ch || !px || !tmpl ||
      tlen <= 0 || !g || !out || !mem || !counts_dev || !status_dev)
    return CRV_ERR_ARG;
  size_t need = 0;
  chain_layout(nullptr, *p, *caps, &need, lk != nullptr);
  if (!workspace || (long long)need > workspace_bytes) return CRV_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  size_t dummy;
  ChainWs w = chain_layout(base, *p, *caps, &dummy, lk != nullptr);
  const CrvChainCaps& c = *caps;
  long long* n = w.counts;                 // raw counts
  long long* m = w.counts + 16;            // counts passed on: 0 when the stage overflowed its capacity
  const long long zs = p->samples_zs;
  CK(cudaMemsetAsync(w.counts, 0, 32 * sizeof(long long), s));
  // the stage totals that size the photon and slot capacities, from the stage workspaces (scratch is 256-aligned)
  auto keep_total = [&](const long long* total, int k) -> cudaError_t {
    crv::Mark mark_("k_copy_i64", s);
    k_copy_i64<<<1, 1, 0, s>>>(total, &n[k]);
    return cudaGetLastError();
  };
  auto N = [&](int k) { return reinterpret_cast<int64_t*>(&n[k]); };
  auto guard = [&](int k, long long cap) -> cudaError_t {
    crv::Mark mark_("k_guard_groups", s);
    k_guard_groups<<<1, 32, 0, s>>>(&n[k], cap, &n[k], &m[k]);
    return cudaGetLastError();
  };
  int rc = response_run(p, ev, c.events, st, c.steps, reinterpret_cast<const long long*>(nsteps_dev),
                        c.max_steps_per_event, bars, ch, px, c.photons, &w.Q, c.charges, N(CRV_CHAIN_CHARGES),
                        nullptr, nullptr, nullptr, 0, nullptr, w.scratch, w.scratch_bytes, stream, status_dev, lk);
  if (rc != CRV_OK) return rc;
  {
    size_t b;
    CK(keep_total(&resp_layout(w.scratch, *p, c.events, c.steps, c.photons, &b, lk != nullptr).totals[1],
                  CRV_CHAIN_PHOTONS));
  }
  CK(guard(CRV_CHAIN_CHARGES, c.charges));
  rc = digis_run(p, ch, c.charges, &m[CRV_CHAIN_CHARGES], w.Q.label, w.Q.time, w.Q.charge, nullptr, tmpl, tlen, ev_keys,
                 ev_runs, c.events, c.slots, &w.D, c.digis, N(CRV_CHAIN_DIGIS), w.scratch, w.scratch_bytes, stream,
                 status_dev);
  if (rc != CRV_OK) return rc;
  {
    size_t b;
    CK(keep_total(&digi_layout(w.scratch, c.charges, c.slots, p->samples_zs, &b).totals[1], CRV_CHAIN_SLOTS));
  }
  CK(guard(CRV_CHAIN_DIGIS, c.digis));
  rc = reco_waveforms_run(p, ch, c.digis, &m[CRV_CHAIN_DIGIS], w.D.chan, w.D.starttdc, w.w_label, w.w_off, w.w_n,
                          w.w_start, w.w_ped, w.w_area, w.w_height, w.w_toff, N(CRV_CHAIN_WAVEFORMS), w.scratch,
                          w.scratch_bytes, stream, status_dev);
  if (rc != CRV_OK) return rc;
  CK(guard(CRV_CHAIN_WAVEFORMS, c.digis));
  rc = pulses_run(p, c.digis, &m[CRV_CHAIN_WAVEFORMS], c.digis * zs, w.w_off, w.w_n, w.w_start, w.w_ped, w.w_area,
                  w.w_height, w.D.adc, nullptr, 0x7FFFFFFF, &w.P, c.pulses, N(CRV_CHAIN_PULSES), w.near, w.scratch,
                  w.scratch_bytes, stream, status_dev);
  if (rc != CRV_OK) return rc;
  CK(guard(CRV_CHAIN_PULSES, c.pulses));
  rc = pulse_hits_run(p, ch->status, c.digis, w.w_label, w.w_toff, nullptr, c.pulses, &m[CRV_CHAIN_PULSES], w.P.wf,
                      w.P.seq, w.P.time, w.P.pe, w.h_ev_start, w.h_ev_count, w.h_ev_key, w.h_bar, w.h_sipm, w.h_seq,
                      w.h_time, w.h_pe, N(CRV_CHAIN_EVENTS), N(CRV_CHAIN_HITS), w.scratch, w.scratch_bytes, stream,
                      status_dev);
  if (rc != CRV_OK) return rc;
  CK(guard(CRV_CHAIN_EVENTS, c.events));
  rc = coinc_run(p, g, c.events, &m[CRV_CHAIN_EVENTS], w.h_ev_start, w.h_ev_count, w.h_ev_key, c.pulses, w.h_bar,
                 w.h_sipm, w.h_seq, w.h_time, w.h_pe, ch->status, out, c.pulses, N(CRV_CHAIN_CLUSTERS), mem, c.pulses,
                 N(CRV_CHAIN_MEMBERS), w.scratch, w.scratch_bytes, stream, status_dev);
  if (rc != CRV_OK) return rc;
  CK(cudaMemcpyAsync(counts_dev, n, 10 * sizeof(long long), cudaMemcpyDeviceToDevice, s));
  return CRV_OK;
}
}  // namespace crv

extern "C" int crv_chain(const CrvParams* p, const CrvChainCaps* caps, const CrvEvents* ev, const int64_t* ev_keys,
                         const uint32_t* ev_runs, const CrvSteps* st, const int64_t* nsteps_dev, const CrvBars* bars,
                         const CrvChannels* ch, const CrvPixels* px, const double* tmpl, int32_t tlen,
                         const CrvFinderGeom* g, CrvClusters* out, CrvMembers* mem, int64_t* counts_dev,
                         void* workspace, int64_t workspace_bytes, void* stream, CrvStatus* status_dev) {
  return chain_run(p, caps, ev, ev_keys, ev_runs, st, nsteps_dev, bars, ch, px, tmpl, tlen, g, out, mem, counts_dev,
                   workspace, workspace_bytes, stream, status_dev, nullptr);
}

extern "C" int crv_chain_lookup(const CrvParams* p, const CrvChainCaps* caps, const CrvEvents* ev,
                                const int64_t* ev_keys, const uint32_t* ev_runs, const CrvSteps* st,
                                const int64_t* nsteps_dev, const CrvBars* bars, const CrvChannels* ch,
                                const CrvPixels* px, const double* tmpl, int32_t tlen, const CrvFinderGeom* g,
                                CrvClusters* out, CrvMembers* mem, int64_t* counts_dev, void* workspace,
                                int64_t workspace_bytes, void* stream, CrvStatus* status_dev,
                                const CrvLookupChain* lk) {
  if (!lk) return CRV_ERR_ARG;
  return chain_run(p, caps, ev, ev_keys, ev_runs, st, nsteps_dev, bars, ch, px, tmpl, tlen, g, out, mem, counts_dev,
                   workspace, workspace_bytes, stream, status_dev, lk);
}

// ---- the resident chain as one CUDA graph, re-parameterised per design point --------------------------------------

struct CrvChainGraph {
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  CrvParams p;                   // the parameter block the graph's kernels hold now
};

namespace crv {
// The serving knobs a graph's kernels may take from a new parameter block without a new capture: none of them
// changes which kernels run or their launch shapes (the host reads no other field of the block to launch the chain).
static bool only_knobs_differ(const CrvParams& a, const CrvParams& b) {
  CrvParams x = b;
  x.seed = a.seed;
  x.yield_per_mev = a.yield_per_mev;
  x.frac_short = a.frac_short;
  x.frac_long = a.frac_long;
  x.lambda_short = a.lambda_short;
  x.lambda_long = a.lambda_long;
  x.min_voltage = a.min_voltage;
  x.noise_sigma = a.noise_sigma;
  return memcmp(&x, &a, sizeof(CrvParams)) == 0;
}

typedef CUresult (*FuncGetParamInfo)(CUfunction, size_t, size_t*, size_t*);

static FuncGetParamInfo param_info_fn() {
  static FuncGetParamInfo fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuFuncGetParamInfo", &f, 12040, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<FuncGetParamInfo>(f);
  });
  return fn;
}
}  // namespace crv

namespace crv {
static int graph_create(const CrvParams* p, const CrvChainCaps* caps, const CrvEvents* ev, const int64_t* ev_keys,
                        const uint32_t* ev_runs, const CrvSteps* st, const int64_t* nsteps_dev, const CrvBars* bars,
                        const CrvChannels* ch, const CrvPixels* px, const double* tmpl, int32_t tlen,
                        const CrvFinderGeom* g, CrvClusters* out, CrvMembers* mem, int64_t* counts_dev,
                        void* workspace, int64_t workspace_bytes, void* stream, CrvStatus* status_dev,
                        const CrvLookupChain* lk, CrvChainGraph** graph_out) {
  if (!graph_out || !p || !status_dev) return CRV_ERR_ARG;
  *graph_out = nullptr;
  cudaStream_t s = (cudaStream_t)stream;
  if (!s) return CRV_ERR_ARG;                    // the legacy default stream cannot be captured
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = CRV_OK;
  if (cudaMemsetAsync(status_dev, 0, sizeof(CrvStatus), s) != cudaSuccess) rc = CRV_ERR_CUDA;
  if (rc == CRV_OK)
    rc = chain_run(p, caps, ev, ev_keys, ev_runs, st, nsteps_dev, bars, ch, px, tmpl, tlen, g, out, mem, counts_dev,
                   workspace, workspace_bytes, stream, status_dev, lk);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &graph);
  if (rc != CRV_OK || e != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    return rc != CRV_OK ? rc : CRV_ERR_CUDA;
  }
  cudaGraphExec_t exec = nullptr;
  if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
    cudaGraphDestroy(graph);
    return CRV_ERR_CUDA;
  }
  *graph_out = new CrvChainGraph{graph, exec, *p};
  return CRV_OK;
}
}  // namespace crv

extern "C" int crv_chain_graph_create(const CrvParams* p, const CrvChainCaps* caps, const CrvEvents* ev,
                                      const int64_t* ev_keys, const uint32_t* ev_runs, const CrvSteps* st,
                                      const int64_t* nsteps_dev, const CrvBars* bars, const CrvChannels* ch,
                                      const CrvPixels* px, const double* tmpl, int32_t tlen, const CrvFinderGeom* g,
                                      CrvClusters* out, CrvMembers* mem, int64_t* counts_dev, void* workspace,
                                      int64_t workspace_bytes, void* stream, CrvStatus* status_dev,
                                      CrvChainGraph** graph_out) {
  return graph_create(p, caps, ev, ev_keys, ev_runs, st, nsteps_dev, bars, ch, px, tmpl, tlen, g, out, mem,
                      counts_dev, workspace, workspace_bytes, stream, status_dev, nullptr, graph_out);
}

extern "C" int crv_chain_graph_create_lookup(const CrvParams* p, const CrvChainCaps* caps, const CrvEvents* ev,
                                             const int64_t* ev_keys, const uint32_t* ev_runs, const CrvSteps* st,
                                             const int64_t* nsteps_dev, const CrvBars* bars, const CrvChannels* ch,
                                             const CrvPixels* px, const double* tmpl, int32_t tlen,
                                             const CrvFinderGeom* g, CrvClusters* out, CrvMembers* mem,
                                             int64_t* counts_dev, void* workspace, int64_t workspace_bytes,
                                             void* stream, CrvStatus* status_dev, const CrvLookupChain* lk,
                                             CrvChainGraph** graph_out) {
  if (!lk) return CRV_ERR_ARG;
  return graph_create(p, caps, ev, ev_keys, ev_runs, st, nsteps_dev, bars, ch, px, tmpl, tlen, g, out, mem,
                      counts_dev, workspace, workspace_bytes, stream, status_dev, lk, graph_out);
}

extern "C" int crv_chain_graph_launch(CrvChainGraph* h, void* stream) {
  if (!h) return CRV_ERR_ARG;
  CK(cudaGraphLaunch(h->exec, (cudaStream_t)stream));
  return CRV_OK;
}

extern "C" int crv_chain_graph_set_params(CrvChainGraph* h, const CrvParams* p) {
  if (!h || !p) return CRV_ERR_ARG;
  if (!only_knobs_differ(h->p, *p)) return CRV_ERR_ARG;
  if (memcmp(&h->p, p, sizeof(CrvParams)) == 0) return CRV_OK;
  FuncGetParamInfo info = param_info_fn();
  if (!info) return CRV_ERR_CUDA;
  size_t nn = 0;
  CK(cudaGraphGetNodes(h->graph, nullptr, &nn));
  std::vector<cudaGraphNode_t> nodes(nn);
  CK(cudaGraphGetNodes(h->graph, nodes.data(), &nn));
  CrvParams np = *p;
  std::vector<void*> args;
  for (size_t i = 0; i < nn; ++i) {
    cudaGraphNodeType t;
    CK(cudaGraphNodeGetType(nodes[i], &t));
    if (t != cudaGraphNodeTypeKernel) continue;
    cudaKernelNodeParams kp;
    CK(cudaGraphKernelNodeGetParams(nodes[i], &kp));
    cudaFunction_t f;
    CK(cudaGetFuncBySymbol(&f, kp.func));
    size_t off = 0, size = 0;
    if (info(reinterpret_cast<CUfunction>(f), 0, &off, &size) != CUDA_SUCCESS) return CRV_ERR_CUDA;
    // a kernel whose first argument is this library's parameter block, as captured
    if (size != sizeof(CrvParams) || !kp.kernelParams || memcmp(kp.kernelParams[0], &h->p, size) != 0) continue;
    size_t na = 1;
    while (info(reinterpret_cast<CUfunction>(f), na, &off, &size) == CUDA_SUCCESS) ++na;
    args.assign(kp.kernelParams, kp.kernelParams + na);
    args[0] = &np;
    kp.kernelParams = args.data();
    kp.extra = nullptr;
    CK(cudaGraphExecKernelNodeSetParams(h->exec, nodes[i], &kp));
    CK(cudaGraphKernelNodeSetParams(nodes[i], &kp));
  }
  h->p = np;
  return CRV_OK;
}

extern "C" void crv_chain_graph_destroy(CrvChainGraph* h) {
  if (!h) return;
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  delete h;
}
