// Internal launch interface between the engine (C ABI) translation unit and the per-precision kernel units.
#pragma once
#include <cuda_runtime.h>
#include "crv_device.cuh"

namespace crv {

struct SipmGroups;
struct SipmOut;
struct WfGroups;
struct DigiSlots;
struct WaveIn;
struct PulseSlots;
struct PfQueue;
struct WfCluster;

struct DeviceInfo {
  int sms;
  size_t smem_optin;
};
const DeviceInfo& device_info();

// Allow a kernel the device's whole opt-in shared memory as dynamic shared memory (less its static part).  The
// limit is a per-kernel setting shared by every thread of the process; setting it to the same value in every call
// keeps concurrent callers (serving slots on other host threads) from lowering it under each other's launches.
template <typename K>
inline cudaError_t allow_dynamic_smem(K kern) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, kern);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              int(device_info().smem_optin - a.sharedSizeBytes));
}

// Launch accounting: every kernel launch of the library is wrapped in a Mark, which counts it and, while profiling
// is enabled (crv_profile), records CUDA events around it on its stream.
struct Mark {
  int slot;
  cudaStream_t stream;
  Mark(const char* name, cudaStream_t s);
  ~Mark();
};

template <typename R>
cudaError_t launch_photon_count(const CrvParams& p, const CrvEvents& ev, const CrvSteps& st, const CrvBars& bars,
                                const CrvChannels& ch, const int32_t* step_event, long long nsteps,
                                const long long* nsteps_dev, int masked, int32_t* count, Status* status,
                                cudaStream_t s);

template <typename R>
cudaError_t launch_photon_emit(const CrvParams& p, const CrvEvents& ev, const CrvSteps& st, const CrvBars& bars,
                               long long nsipm_bound, const long long* nsipm_dev, const int32_t* s_event,
                               const int32_t* s_chan, const long long* s_seg, const int32_t* s_nseg,
                               const int32_t* step_order, const int32_t* count, const long long* ph_off, R* ph_t,
                               uint32_t* ph_key, const long long* ph_total, long long ph_cap, cudaStream_t s);

template <typename R>
cudaError_t launch_photon_rows(const CrvParams& p, const CrvEvents& ev, const CrvSteps& st, const CrvBars& bars,
                               const int32_t* step_event, long long nsteps, const int32_t* count,
                               const long long* row_offset, int64_t* o_step, int64_t* o_chan, double* o_time,
                               int64_t* o_key, cudaStream_t s);

// SiPM simulation over groups; PT = storage type of the photon times (R for the chain, double for the stage API)
template <typename R, typename PT>
cudaError_t launch_sipm(const CrvParams& p, const CrvPixels& px, const SipmGroups& G, const long long* ngroups_dev,
                        const PT* ph_time, const SipmOut& O, Status* status, cudaStream_t s);

template <typename R>
cudaError_t launch_wf_prepass(const CrvParams& p, const CrvChannels& ch, const WfGroups& G, long long ng_bound,
                              const double* time, const double* tmpl, int tlen, const double* tdc0_rows,
                              double* g_tdc0, int32_t* g_bound, int32_t* g_maxlen, int32_t* g_nkept, WfCluster* cl,
                              int32_t* row_scratch, Status* status, cudaStream_t s);

template <typename R>
cudaError_t launch_wf_synth(const CrvParams& p, const WfGroups& G, long long ng_bound, const double* time,
                            const double* charge, const double* tmpl, int tlen, const double* tdc0_rows,
                            const double* g_tdc0, const int32_t* g_maxlen, const int32_t* g_nkept,
                            const WfCluster* cl, const DigiSlots& D, Status* status, cudaStream_t s);

// The lookup-table photon model inside the resident chain: dense rows (row 4 step + SiPM of the output channel; a
// row of no group has group -1), their arrival counts in the chain's per-(step, SiPM) count array, and the photons
// written at the offsets the chain gives each row (row_off, -1: not written).
struct LookupChainWs {
  CrvSubstepRowsOut rows;
  int8_t* row_group;
  long long* count;
  long long* row_off;
  long long* nrows;              // device: 4 x the batch's steps
  uint32_t* seed;                // device copy of the parameter block's seed
  int64_t* o_step;               // per photon: the step's row (the photon id)
  double* o_time;                // per photon: arrival time
};
cudaError_t lookup_chain_rows(const CrvParams& p, const CrvLookupChain& K, const long long* nsteps_dev,
                              long long step_cap, const LookupChainWs& w, cudaStream_t s);
cudaError_t lookup_chain_count(const CrvLookupChain& K, const LookupChainWs& w, long long row_cap, int32_t* count32,
                               Status* status, cudaStream_t s);
cudaError_t lookup_chain_emit(const CrvLookupChain& K, const LookupChainWs& w, long long row_cap,
                              const long long* total, long long cap, Status* status, cudaStream_t s);

template <typename R>
cudaError_t launch_pulsefit(const CrvParams& p, const WaveIn& W, double* yscr, int max_pulses, const PulseSlots& S,
                            const PfQueue& Q, Status* status, cudaStream_t s);

}  // namespace crv
