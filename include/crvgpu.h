/*
 * crvgpu: C ABI of the GB300 CRV response engine (CrvSteps -> SiPM charges -> digis -> reco pulses -> coincidence
 * clusters).  Plain pointers and sizes only; every array argument is a DEVICE pointer owned by the caller (the
 * Python host allocates it with PyTorch), except in the lookup-table file reader (host memory, marked below);
 * `stream` is a cudaStream_t; no call synchronises the host.
 *
 * Each entry point replaces one stage function of the reference's Python API (RobMina/mu2e-fastsim, CRV package):
 *
 *   crv_photon_counts / crv_photons  <- crvfastsim.response.photons.make_photons      (crv/crvfastsim/response/photons.py:359)
 *   crv_sipm                         <- crvfastsim.response.sipm.simulate             (crv/crvfastsim/response/sipm.py:102)
 *   crv_response                     <- crvfastsim.chain.charges                      (crv/crvfastsim/chain.py:151)
 *   crv_digis                        <- crvfastsim.chain.digis                        (crv/crvfastsim/chain.py:234)
 *   crv_synthesize                   <- crvfastsim.reco.waveform.synthesize           (crv/crvfastsim/reco/waveform.py:74)
 *   crv_tdc0_per_feb                 <- crvfastsim.chain.tdc0_per_feb                 (crv/crvfastsim/chain.py:219)
 *   crv_reco_waveforms               <- crvfastsim.chain.reco_waveforms + reco.pulsefit.concat_waveforms
 *                                                                                     (crv/crvfastsim/chain.py:273,
 *                                                                                      crv/crvfastsim/reco/pulsefit.py:319)
 *   crv_pulses                       <- crvfastsim.reco.pulsefit.reconstruct(_full) + filter_channels
 *                                                                                     (crv/crvfastsim/reco/pulsefit.py:222-316)
 *   crv_coincidences                 <- crvfastsim.reco.coinc.find_event over every event, as chain.clusters
 *                                                                                     (crv/crvfastsim/reco/coinc.py:289,
 *                                                                                      crv/crvfastsim/chain.py:296-362)
 *   crv_substep_photons              <- crvfastsim.response.photons._substep_photons   (crv/crvfastsim/response/photons.py:163)
 *   crv_lookup_rows                  <- crvfastsim.response.photons.iter_rows          (crv/crvfastsim/response/photons.py:305)
 *   crv_chain                        <- the chain above in one resident call with explicit capacities, as the
 *                                       mixing adapter's resident CRV chain (mixing/device_crv.py:127-573,
 *                                       mixing/DEVICE_CRV.md "Explicit capacities")
 *   crv_lookup_file_info / _read     <- crvfastsim.response.lookup.load (host memory; crv/crvfastsim/response/lookup.py:149)
 *   crv_lz4_block_decompress,        <- the "L4" baskets of the ROOT step tables that mu2efastsim.tables.read opens
 *   crv_xxh64                           through uproot (core/mu2efastsim/tables.py:25-27)
 *
 * Error convention: the return value is a host error code (CRV_OK, CRV_ERR_ARG for invalid arguments, CRV_ERR_CUDA
 * for a failed launch).  Data-dependent conditions are reported in the device status block (CrvStatus): capacity
 * overflows carry the size they needed in need[], so the caller can re-run with larger buffers; nothing is ever
 * silently truncated.
 */
#ifndef CRVGPU_H
#define CRVGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CRVGPU_VERSION 1

/* host return codes */
#define CRV_OK 0
#define CRV_ERR_ARG 1
#define CRV_ERR_CUDA 2
#define CRV_ERR_TOO_LARGE 3 /* crv_pulses_static: the call needs more scratch than CRV_PULSES_STATIC_MAX_BYTES */

/* device status flags */
#define CRV_ST_CAPACITY 1      /* a buffer was too small; need[] has the required size */
#define CRV_ST_LIMIT 2         /* a draw-key limit was exceeded (65,536 steps per event or photons per step row,
                                  16 cross-talk generations, 64 nodes per generation) */
#define CRV_ST_NONFINITE 4     /* a non-finite input where a finite one is required */
#define CRV_ST_ORDER 8         /* input not grouped/sorted as the entry point requires */
#define CRV_ST_BOUNDS 16       /* crv_pulses: a waveform's samples [off, off + n) outside the sample array (or its
                                  record slots outside the workspace); that waveform is skipped, nothing is read */

/* need[] slots */
#define CRV_NEED_STEPS_PER_EVENT 0
#define CRV_NEED_PHOTONS_PER_SIPM 1
#define CRV_NEED_CHARGE_FACTOR 2   /* charges per SiPM beyond the slot: slot = factor * photons + 16 */
#define CRV_NEED_DIGIS 3
#define CRV_NEED_SAMPLES 4
#define CRV_NEED_PULSES 5
#define CRV_NEED_HITS_PER_EVENT 6
#define CRV_NEED_CLUSTERS 7
#define CRV_NEED_PHOTONS_TOTAL 8
#define CRV_NEED_SLOTS_TOTAL 9
#define CRV_NEED_CHARGES_OUT 10
#define CRV_NEED_DIGIS_OUT 11
#define CRV_NEED_WAVEFORMS 12
#define CRV_NEED_PULSES_OUT 13
#define CRV_NEED_MEMBERS 14
#define CRV_NEED_PHOTONS_OUT 15      /* crv_substep_photons output */

typedef struct CrvStatus {
    int32_t flags;
    int32_t pad;
    long long need[16];
} CrvStatus;

/* Physics and configuration knobs (all runtime data: no recompilation per design point). */
typedef struct CrvParams {
    uint32_t seed;
    int32_t precision;           /* 0 = FP64 plain, 1 = FP32 mixed */
    /* photons: analytic yield and two-exponential attenuation */
    double yield_per_mev, frac_short, frac_long, lambda_short, lambda_long, signal_speed, decay_time;
    /* SiPM */
    double overvoltage, time_constant, capacitance, p1, p2, q_ct, q_t0, q_t1, trap0_lifetime, trap1_lifetime;
    double t_end;
    int32_t n_pixels_x, n_pixels_y;
    int32_t uniform_map;         /* 1: photon map is uniform (pixel = floor(u * 1600)) */
    int32_t charge_factor;       /* charge slots per SiPM = charge_factor * photons + 16 */
    /* waveforms */
    double period, spe_precision, spe_max_time, spe_ref_charge, min_voltage, noise_sigma, adc_conversion;
    double window_lo, window_hi, feb_phase_width;
    int32_t samples_zs, adc_pedestal, min_adc, max_adc, template_len, feb_key_mode; /* 0 roc*1000+feb, 1 feb */
    int32_t noise_on;
    int32_t pixel_lrint;         /* SiPM pixel id of a photon-map point: 0 "truncate" (the bin), 1 "lrint" (rounded) */
    /* pulse reconstruction */
    double min_adc_difference, default_beta, min_beta, max_beta, max_time_difference, min_height_ratio;
    double max_height_ratio, le_time_factor, pedestal_undershoot, time_offset_scale, limit_tolerance, knife_edge_adc;
    int32_t samples_before, samples_after, max_pulses, lm_iterations, use_time_offset_db, ignore_channels;
    /* coincidence finder */
    double fiber_signal_speed, max_time_interval, time_offset;
    int32_t compensate_mask, ignore_secondary, big_cluster_threshold, add_opposite;
} CrvParams;

/* Events: the steps of event e are rows [first_step[e], first_step[e] + nsteps[e]) of the step table. */
typedef struct CrvEvents {
    const uint32_t *event, *subrun, *run;
    const int64_t *first_step;
    const int32_t *nsteps;
} CrvEvents;

/* SoA step table: midpoint position (Mu2e frame, mm), midpoint time (ns), deposited energy (MeV), bar index.
 * x, y, z, t, edep are float32 (real_bytes 4) or float64 (real_bytes 8). */
typedef struct CrvSteps {
    const void *x, *y, *z, *t, *edep;
    const int32_t *bar;
    int32_t real_bytes;
    int32_t pad;
} CrvSteps;

/* Per bar: axis of the length direction (0 x, 1 y, 2 z), centre and half length along it (mm). */
typedef struct CrvBars {
    const int8_t *length_axis;
    const double *center_l, *half_l;
    int32_t nbars;
    int32_t pad;
} CrvBars;

/* Per channel (4 * bar + SiPM): photon-yield factor, effective status, ROC, FEB, CRVCalib constants. */
typedef struct CrvChannels {
    const double *yield_factor;
    const int32_t *status, *roc, *feb;
    const double *pedestal, *pulsearea, *pulseheight, *timeoffset;
    int32_t nchan;
    int32_t pad;
} CrvChannels;

/* SiPM pixel model tables: photon-map running sums (1,600 bins x * 40 + y) and the dead-pixel bitmap over pixel ids
 * x * 41 + y, x and y in 0..40 (53 words; crv/crvfastsim/response/sipm.py:22 NPIX = 41). */
typedef struct CrvPixels {
    const double *cum;
    const uint32_t *dead_bits;
} CrvPixels;

/* SiPM charges sorted by (label, time): label = event key * 32768 + channel, event key = subrun << 20 | event. */
typedef struct CrvCharges {
    int64_t *label;
    double *time, *charge, *pe;
    int64_t *photon;             /* step row of the photon that started the avalanche */
} CrvCharges;

/* Zero-suppressed digis sorted by (label, start): label, start (ns), TDC0 (ns), start TDC, volt[n][12], adc[n][12]. */
typedef struct CrvDigis {
    int64_t *chan;
    double *start, *tdc0;
    int64_t *starttdc;
    double *volt;
    int16_t *adc;
} CrvDigis;

/* Pulses in (waveform, sequence) order, the reference's reconstruct() columns. */
typedef struct CrvPulses {
    int64_t *wf, *seq;
    double *pe, *peph, *time, *height, *beta, *chi2, *letime, *ped, *fit_A, *fit_mu, *fit_b;
    uint8_t *failed, *zerondf, *pedfromdb;
} CrvPulses;

/* Coincidence-finder geometry and cuts (SectorGeom + FinderConfig cuts, flattened).  cuts: per cut set 10 values
 * (pe_threshold, max_dt_adjacent, max_dt, min_slope, max_slope, max_slope_diff, coincidence_layers, min_cluster_pes,
 * initial_max_distance, final_max_distance); sec_cut = -1 for sectors without cuts.  Types ascending, with their
 * readout-end extremes p0/p1, half length, largest max_dt and instrumented sides. */
typedef struct CrvFinderGeom {
    const int32_t *bar_sector, *bar_layer, *bar_counter;
    const double *bar_x, *bar_y, *bar_pos;
    const int32_t *sec_type, *sec_cut, *sec_length_dir;
    const double *sec_pos0, *sec_pos1;
    const double *cuts;
    const int32_t *type_id;
    const double *type_p0, *type_p1, *type_half, *type_maxdt;
    const int32_t *type_side0, *type_side1;
    int32_t ntypes;
    int32_t pad;
} CrvFinderGeom;

/* Coincidence clusters (event order, then sector type, then cluster order) and their member pulses. */
typedef struct CrvClusters {
    int64_t *event;
    int32_t *type;
    double *pe, *start, *end, *slope, *avgtime;
    uint8_t *poscalc;
    double *pos;                 /* [n][3] */
    double *sidepe, *sidetime;   /* [n][2] */
    int32_t *sidehits;           /* [n][2] */
    int32_t *nlayers;
} CrvClusters;

typedef struct CrvMembers {
    int64_t *cl;                 /* cluster row */
    int32_t *idx;                /* pulse index inside its event */
    int64_t *event;
} CrvMembers;

/* ---- version / status / accounting ---- */
int crv_version(void);
const char *crv_status_string(int32_t flags);
/* Kernel launches issued by this library since load (every entry point's launches). */
long long crv_launch_count(void);
/* Profiling: crv_profile(1) clears the record and records CUDA events around every later launch (on its stream);
 * crv_profile_read synchronises on the recorded events and returns their count, with up to cap kernel names (64 bytes
 * each) and durations in ms.  crv_profile(0) stops recording. */
void crv_profile(int on);
int crv_profile_read(int cap, char *names, float *ms);

/* Size in bytes of the caller-provided device workspace of crv_response for the given sizes (photon_cap: photons
 * the batch may produce; max_steps_per_event: largest event of the batch). */
int64_t crv_response_workspace(const CrvParams *p, int64_t nevents, int64_t nsteps, int64_t photon_cap,
                               int32_t max_steps_per_event);

/*
 * chain.charges: steps -> photons (analytic model, keyed draws) -> SiPM charges, for every unmasked channel
 * ((status & 0b101) == 0).  Outputs (capacity out_cap) in label/time order; *n_out_dev (device int64) receives the
 * count.  Per-SiPM diagnostics (optional, NULL to skip; capacity sipm_cap): label, photons, fired pixels; their count
 * goes to *n_sipm_dev.
 */
int crv_response(const CrvParams *p, const CrvEvents *ev, int64_t nevents, const CrvSteps *st, int64_t nsteps,
                 int32_t max_steps_per_event, const CrvBars *bars, const CrvChannels *ch, const CrvPixels *px,
                 int64_t photon_cap, CrvCharges *out, int64_t out_cap, int64_t *n_out_dev, int64_t *sipm_label,
                 int32_t *sipm_photons, int32_t *sipm_fired, int64_t sipm_cap, int64_t *n_sipm_dev, void *workspace,
                 int64_t workspace_bytes, void *stream, CrvStatus *status_dev);

/*
 * photons.make_photons, first half: photon count of every (step, SiPM) row, count[4 * step + sipm] (every channel,
 * masked or not, as the reference stage); step_event[step] receives the step's event index.
 */
int crv_photon_counts(const CrvParams *p, const CrvEvents *ev, int64_t nevents, const CrvSteps *st, int64_t nsteps,
                      const CrvBars *bars, const CrvChannels *ch, int32_t *step_event, int32_t *count, void *stream,
                      CrvStatus *status_dev);

/*
 * photons.make_photons, second half: emit the photons of every row given row offsets (exclusive prefix of count in
 * the reference's block order: SiPM 0..3, then step, then photon).  Outputs per photon: step row, channel, arrival
 * time, draw key (step-in-event << 16 | photon).
 */
int crv_photons(const CrvParams *p, const CrvEvents *ev, int64_t nevents, const CrvSteps *st, int64_t nsteps,
                const CrvBars *bars, const int32_t *step_event, const int32_t *count, const int64_t *row_offset,
                int64_t *o_step, int64_t *o_chan, double *o_time, int64_t *o_key, void *stream,
                CrvStatus *status_dev);

/*
 * sipm.simulate: photons grouped by SiPM (group g = rows [gstart[g], gstart[g] + gcount[g]), label glabel[g], run
 * grun[g]); any order inside a group.  Charges in group order, time order inside a group (out capacity out_cap);
 * per-group charge counts and fired-pixel counts.  key: per-photon draw key (step-in-event << 16 | photon).
 */
int64_t crv_sipm_workspace(const CrvParams *p, int64_t ngroups, int64_t nphotons);
int crv_sipm(const CrvParams *p, const CrvPixels *px, int64_t ngroups, int64_t nphotons, const int64_t *gstart, const int32_t *gcount,
             const int64_t *glabel, const uint32_t *grun, const double *time, const int64_t *key,
             const int64_t *photon, CrvCharges *out, int64_t out_cap, int64_t *n_out_dev, int32_t *g_charges,
             int32_t *g_fired, void *workspace, int64_t workspace_bytes, void *stream, CrvStatus *status_dev);

/*
 * chain.digis / waveform.synthesize: SiPM charges sorted by (label, time) -> digis.  TDC0 is one keyed uniform x
 * feb_phase_width per (event, FEB); electronics noise is keyed by (event, channel, sample tick).  tmpl: the single-PE
 * template (tlen samples at spe_precision).  ev_keys/ev_runs (optional, n_events sorted event keys and their runs)
 * give the run of each event for the keys; without them run 0 is used.  slot_cap: digi slots of the workspace
 * (an upper bound is computed on the device; CRV_NEED_DIGIS reports the bound when it exceeds slot_cap).
 */
int64_t crv_digis_workspace(const CrvParams *p, int64_t ncharges, int64_t slot_cap);
int crv_digis(const CrvParams *p, const CrvChannels *ch, int64_t ncharges, const int64_t *label, const double *time,
              const double *charge, const double *tmpl, int32_t tlen, const int64_t *ev_keys, const uint32_t *ev_runs,
              int64_t n_events, int64_t slot_cap, CrvDigis *out, int64_t out_cap, int64_t *n_out_dev, void *workspace,
              int64_t workspace_bytes, void *stream, CrvStatus *status_dev);

/*
 * waveform.synthesize with the caller's TDC0 (crv/crvfastsim/reco/waveform.py:74-172, whose tdc0_of_chan gives one
 * TDC0 per charge cluster): as crv_digis, but tdc0_rows[q] is the TDC0 (ns) of the cluster that charge row q belongs
 * to (read at the first charge of every cluster; the host broadcasts the caller's per-cluster values), and no run
 * table is needed (the TDC0 draw is the caller's).  Workspace: crv_digis_workspace.
 */
int crv_synthesize(const CrvParams *p, const CrvChannels *ch, int64_t ncharges, const int64_t *label, const double *time,
                   const double *charge, const double *tdc0_rows, const double *tmpl, int32_t tlen, int64_t slot_cap,
                   CrvDigis *out, int64_t out_cap, int64_t *n_out_dev, void *workspace, int64_t workspace_bytes,
                   void *stream, CrvStatus *status_dev);

/*
 * chain.tdc0_per_feb (crv/crvfastsim/chain.py:219-231): TDC0 (ns) of every SiPM label, one keyed uniform x
 * feb_phase_width per (event, FEB key) (feb_key_mode 0: ROC * 1000 + FEB, 1: FEB), the draw crv_digis makes.
 * ev_keys / ev_runs (optional, n_events sorted event keys and their runs) give the run of each label's event (run 0
 * without them; a label whose event is missing, or whose channel is outside the channel table, sets CRV_ST_ORDER).
 */
int crv_tdc0_per_feb(const CrvParams *p, const CrvChannels *ch, int64_t nlabels, const int64_t *labels,
                     const int64_t *ev_keys, const uint32_t *ev_runs, int64_t n_events, double *tdc0, void *stream,
                     CrvStatus *status_dev);

/*
 * pulsefit.reconstruct: nw waveforms; waveform w has n[w] valid samples at sample rows [off[w], off[w] + n[w]) of
 * adc16 (int16) or adc64 (int64; exactly one is non-null), start TDC, DB pedestal, calibration area and height;
 * nsamples: rows of the sample array.  max_pulses: rounds per waveform (reconstruct_full passes max(cfg max, longest
 * waveform)).  Outputs: pulses (capacity out_cap) and per-waveform wf_near_threshold.
 */
int64_t crv_pulses_workspace(const CrvParams *p, int64_t nw, int64_t nsamples);
int crv_pulses(const CrvParams *p, int64_t nw, int64_t nsamples, const int64_t *off, const int32_t *n,
               const int64_t *start_tdc, const double *ped_db, const double *area, const double *height,
               const int16_t *adc16, const int64_t *adc64, int32_t max_pulses, CrvPulses *out, int64_t out_cap,
               int64_t *n_out_dev, uint8_t *wf_near, void *workspace, int64_t workspace_bytes, void *stream,
               CrvStatus *status_dev);

/*
 * Launch shape of the pulse fit for later crv_pulses calls of this process (no counterpart in the reference; chosen
 * per size bucket by the host's autotuner): threads per block 64 or 128, blocks per SM 1..32, and rounds: 0 = one
 * persistent launch whose lanes claim waveforms from a device head as they finish (the default), 1..32 = that many
 * round launches over a task list before a tail launch.  Results do not depend on the shape.  Returns CRV_ERR_ARG
 * outside those ranges.  Default 128 / 16 / 0.
 */
int crv_pulses_shape(int32_t threads, int32_t blocks_per_sm, int32_t rounds);

/*
 * crv_pulses without a caller workspace (no counterpart in the reference): the scratch is a file-scope device array of
 * CRV_PULSES_STATIC_MAX_BYTES per device, so the call allocates nothing (launch profiler off).  For callers that must
 * not allocate once running: cudaMalloc/cudaFree synchronise the device and stall other streams sharing it, and plain
 * C FFI hosts have no caching allocator.  Limits: crv_pulses_workspace(p, nw, nsamples) must not exceed the maximum
 * (else CRV_ERR_TOO_LARGE, nothing launched).  Every call looks up the array's address on the current device (so a
 * device reset does not leave a stale address); the first call on a device loads the library's device code there,
 * which is when the array is reserved under lazy module loading (the CUDA default since 12.2; with
 * CUDA_MODULE_LOADING=EAGER every device the library touches reserves it at load), and should precede any stream
 * capture.  The scratch needs no zeroing; calls overlapping in time on one device share the scratch and race, so
 * serialise them.  Arguments and results as crv_pulses.
 */
#define CRV_PULSES_STATIC_MAX_BYTES (64ll << 20)
int crv_pulses_static(const CrvParams *p, int64_t nw, int64_t nsamples, const int64_t *off, const int32_t *n,
                      const int64_t *start_tdc, const double *ped_db, const double *area, const double *height,
                      const int16_t *adc16, const int64_t *adc64, int32_t max_pulses, CrvPulses *out, int64_t out_cap,
                      int64_t *n_out_dev, uint8_t *wf_near, void *stream, CrvStatus *status_dev);

/*
 * coinc.find_event over every event (chain.clusters' loop): pulses sorted by (event, waveform, sequence); event e owns
 * pulse rows [ev_start[e], ev_start[e] + ev_count[e]) and reports ev_key[e].  Per pulse: bar, SiPM, sequence, time,
 * PE; status: per-channel status (compensated-partner bits).  Limits of the geometry tables: fewer than 65536 bars and
 * counters per sector type, at most 255 cut sets and 255 sector types.
 */
int64_t crv_coincidences_workspace(int64_t nevents, int64_t npulses);
int crv_coincidences(const CrvParams *p, const CrvFinderGeom *g, int64_t nevents, const int64_t *ev_start,
                     const int32_t *ev_count, const int64_t *ev_key, int64_t npulses, const int32_t *bar,
                     const int32_t *sipm, const int32_t *seq, const double *time, const double *pe,
                     const int32_t *status, CrvClusters *out, int64_t cl_cap, int64_t *n_cl_dev, CrvMembers *mem,
                     int64_t mem_cap, int64_t *n_mem_dev, void *workspace, int64_t workspace_bytes, void *stream,
                     CrvStatus *status_dev);

/*
 * chain.reco_waveforms: digis sorted by (label, start) -> reco waveforms (consecutive digis of one channel whose TDCs
 * continue, pulsefit.concat_waveforms' rule).  Waveform w: label, first sample row (digi row * samples_zs) of the digi
 * ADC array, valid samples, start TDC, and the channel's pedestal / pulse area / pulse height / time offset.
 */
int64_t crv_reco_waveforms_workspace(int64_t ndigis);
int crv_reco_waveforms(const CrvParams *p, const CrvChannels *ch, int64_t ndigis, const int64_t *label,
                       const int64_t *starttdc, int64_t *w_label, int64_t *w_off, int32_t *w_n, int64_t *w_start,
                       double *w_ped, double *w_area, double *w_height, double *w_toff, int64_t *n_w_dev,
                       void *workspace, int64_t workspace_bytes, void *stream, CrvStatus *status_dev);

/*
 * chain.clusters' pulse glue: pulses in (waveform, sequence) order of waveforms grouped by event -> finder input.
 * Drops pulses of status-bit-1 channels (ignore_channels), adds the DB time offset x time_offset_scale
 * (use_time_offset_db) and the optional per-waveform event_t0, and segments the kept pulses by event
 * (ev_start / ev_count / ev_key; idx inside the event is the position in the segment).
 */
int64_t crv_pulse_hits_workspace(int64_t npulses);
int crv_pulse_hits(const CrvParams *p, const int32_t *status, int64_t nw, const int64_t *w_label,
                   const double *w_toff, const double *event_t0, int64_t npulses, const int64_t *p_wf,
                   const int64_t *p_seq, const double *p_time, const double *p_pe, int64_t *ev_start,
                   int32_t *ev_count, int64_t *ev_key, int32_t *bar, int32_t *sipm, int32_t *seq, double *time,
                   double *pe, int64_t *n_ev_dev, int64_t *n_hit_dev, void *workspace, int64_t workspace_bytes,
                   void *stream, CrvStatus *status_dev);

/*
 * The whole chain, steps -> clusters, in one call that reads no size back to the host, so a stream capture of it is a
 * CUDA graph that can be replayed batch after batch.  Capacities are explicit static bounds, not physics cuts
 * (CrvChainCaps, every entry positive); every intermediate lives in the workspace.  Inputs:
 *   - the event table has caps->events rows; a batch with fewer events fills the rest with nsteps 0;
 *   - ev_keys / ev_runs: the event keys (subrun << 20 | event) of those rows in ascending order and their runs (rows
 *     past the batch: keys above every real key, e.g. INT64_MAX);
 *   - the step table has caps->steps rows, of which the first *nsteps_dev (device int64) are the batch's;
 *   - tmpl / tlen: the single-PE template; g: the finder tables; per-channel status in ch.
 * Outputs: clusters and members (capacity caps->pulses each) as crv_coincidences; counts_dev[10] (device int64): the
 * CRV_CHAIN_* counts of the stages, which may exceed a capacity when the status says so (a trial batch with ample
 * capacities gives every figure the capacities are sized from).
 * A capacity overflow sets CRV_ST_CAPACITY with the size needed; later stages then see no items, so the outputs of a
 * batch with any status flag set are not a result and the batch is to be rejected (re-run with larger capacities).
 * Pulse reconstruction runs as the chain's (every pulse of a waveform, reconstruct_full's bound).  The caller zeroes the
 * status block before the call (or inside the captured graph).
 */
typedef struct CrvChainCaps {
    int64_t events;              /* rows of the event table */
    int64_t steps;               /* rows of the step table */
    int64_t photons;             /* photons of a batch */
    int64_t charges;             /* SiPM charges of a batch */
    int64_t slots;               /* digi slots before zero suppression */
    int64_t digis;               /* digis; also bounds the reco waveforms (samples = digis * samples_zs) */
    int64_t pulses;              /* pulses; also bounds the finder hits, clusters and members */
    int32_t max_steps_per_event; /* largest event of any batch run with these capacities */
    int32_t pad;
} CrvChainCaps;

#define CRV_CHAIN_CHARGES 0
#define CRV_CHAIN_DIGIS 1
#define CRV_CHAIN_WAVEFORMS 2
#define CRV_CHAIN_PULSES 3
#define CRV_CHAIN_EVENTS 4           /* events with finder hits */
#define CRV_CHAIN_HITS 5
#define CRV_CHAIN_CLUSTERS 6
#define CRV_CHAIN_MEMBERS 7
#define CRV_CHAIN_PHOTONS 8
#define CRV_CHAIN_SLOTS 9            /* digi slots before zero suppression */

int64_t crv_chain_workspace(const CrvParams *p, const CrvChainCaps *caps);
int crv_chain(const CrvParams *p, const CrvChainCaps *caps, const CrvEvents *ev, const int64_t *ev_keys,
              const uint32_t *ev_runs, const CrvSteps *st, const int64_t *nsteps_dev, const CrvBars *bars,
              const CrvChannels *ch, const CrvPixels *px, const double *tmpl, int32_t tlen, const CrvFinderGeom *g,
              CrvClusters *out, CrvMembers *mem, int64_t *counts_dev, void *workspace, int64_t workspace_bytes,
              void *stream, CrvStatus *status_dev);

/*
 * The resident chain as one CUDA graph (no counterpart in the reference; the reference's resident JAX chain compiles
 * one program per shape): crv_chain_graph_create captures one crv_chain call with these arguments (plus the zeroing
 * of the status block) on `stream`, which must be a created stream, in thread-local capture mode, and instantiates
 * it; crv_chain_graph_launch replays it on any stream, the default one included (a new batch: new contents in the
 * same buffers); crv_chain_graph_set_params
 * gives every kernel of the graph a new parameter block without a new capture, provided it differs from the current
 * one only in the serving knobs (seed, yield_per_mev, frac_short, frac_long, lambda_short, lambda_long, min_voltage,
 * noise_sigma; else CRV_ERR_ARG); crv_chain_graph_destroy frees it.  The design point's finder cuts live in the
 * finder tables, which the caller may overwrite in place between launches.
 */
typedef struct CrvChainGraph CrvChainGraph;
int crv_chain_graph_create(const CrvParams *p, const CrvChainCaps *caps, const CrvEvents *ev, const int64_t *ev_keys,
                           const uint32_t *ev_runs, const CrvSteps *st, const int64_t *nsteps_dev, const CrvBars *bars,
                           const CrvChannels *ch, const CrvPixels *px, const double *tmpl, int32_t tlen,
                           const CrvFinderGeom *g, CrvClusters *out, CrvMembers *mem, int64_t *counts_dev,
                           void *workspace, int64_t workspace_bytes, void *stream, CrvStatus *status_dev,
                           CrvChainGraph **graph_out);
int crv_chain_graph_launch(CrvChainGraph *graph, void *stream);
int crv_chain_graph_set_params(CrvChainGraph *graph, const CrvParams *p);
void crv_chain_graph_destroy(CrvChainGraph *graph);

/*
 * Lookup-table photon model (crvfastsim.response.photons._substep_photons, crv/crvfastsim/response/photons.py:163-224,
 * tables as crv/crvfastsim/response/lookup.py:70-98): every (step, SiPM) row is cut into nsub substeps along its step
 * vector; at each substep the position selects a bin of the scintillation table (inside the scintillator), of the
 * Cherenkov-in-scintillator table (also by beta) and of the Cherenkov-in-fibre table (inside a fibre hole, by beta,
 * theta, phi, r); the arrivals of each are Binomial(photons per substep, min(prob * dev * exp(-mu z), 1)), each
 * delayed by a draw from the bin's delay weights (1 ns bins) and, with a fibre decay time, by a Gamma(emissions, decay
 * time) whose emission count is drawn from the bin's emission weights.  Draws are keyed Philox blocks (key = (seed, 0);
 * counter = (step low, step high, stage 7 | table | call | channel, substep << 12 | arrival)), so results do not depend
 * on batching.  Limits (CRV_ST_LIMIT): 2^20 substeps per row, 4096 arrivals per (substep, table), 128 emissions.
 */
typedef struct CrvLookupTable {
    const float *prob;           /* [nbins] arrival probability */
    const uint8_t *delays;       /* [nbins][ndelay] delay weights (1 ns bins) */
    const int32_t *delay_sum;    /* [nbins] */
    const uint8_t *emis;         /* [nbins][nemis] emission-count weights */
    const int32_t *emis_sum;     /* [nbins] */
    int32_t nbins, ndelay, nemis, pad;
} CrvLookupTable;

typedef struct CrvLookup {
    double half_thickness, half_width, half_length, fiber_separation, hole_radius_x, hole_radius_y, fiber_radius,
        corner_radius, fiber_decay_time;
    const double *edges[7];      /* ascending bin edges of x, y, z, beta, theta, phi, r */
    int32_t nedges[7];
    int32_t precision;           /* 0: FP64 (bit-exact with the CPU oracle); 1: FP32-mixed (geometry, arrival draws
                                    and delays in FP32 with 24-bit uniforms, absolute photon times FP64) */
    const double *cos_phi_edges; /* cos of the phi edges: phi bins are found on cos phi (no arccos per substep) */
    CrvLookupTable table[3];     /* scintillation, Cherenkov in scintillator, Cherenkov in fibre */
    const double *cos_theta_edges; /* cos of the theta edges (rows that carry cos theta instead of theta) */
} CrvLookup;

/* Rows: local start s[3] and step vector d[3] (thickness, width, length; mm), start/end time, beta, theta, yield
 * deviation factor, optional extra attenuation per mm (NULL: none), substeps, step index, channel, and the photons per
 * substep of the three tables; theta may be NULL when cos_theta is given (bins on the cos of the theta edges). */
typedef struct CrvSubstepRows {
    const double *s, *d, *t0, *t1, *beta, *theta, *dev, *mu;
    const int64_t *nsub, *step, *chan, *n_scint, *n_ck_s, *n_ck_f;
    const double *cos_theta;
} CrvSubstepRows;

/*
 * Row preparation of the lookup-table model (photons.iter_rows, crv/crvfastsim/response/photons.py:292-356) for one
 * (lookup table, reflector) group of sectors: per step of a bar in the group with finite start and end times, for each
 * simulated SiPM (0..3 with reflector 0, else 0 and 2) a row: local start and step vector (z mirrored for reflector
 * -1 and SiPMs 1, 3; y for SiPMs 2, 3), times with the extra delay k (z + half length), substeps of 0.1 mm, beta from
 * the mean energy (stock), cos theta, the yield factor of channel 4 bar + s, the bar's extra attenuation, the output
 * channel (4 bar + s, + 1 for reflector -1) and the photons per substep: rint(draw / nsub) of Gauss(avg, sqrt avg) for
 * avg > 10 else Poisson(avg), avg = yield x edep (scintillation) and Cherenkov photons per mm x length, keyed by (seed,
 * step, count type, channel).  Rows are written SiPM block by SiPM block, steps in order inside a block.
 */
typedef struct CrvLookupSteps {
    const double *x0, *y0, *z0, *x1, *y1, *z1, *px0, *py0, *pz0, *p1, *t0, *t1, *edep, *len;
    const int32_t *bar;
    const int64_t *pdg;
} CrvLookupSteps;

typedef struct CrvLookupGroup {
    const double *center;        /* [nbars][3] bar centre (Mu2e frame, mm) */
    const int8_t *l2w;           /* [nbars][3] world axis of the local thickness, width and length axes */
    const int32_t *in_group;     /* [nbars] 1 when the bar's sector is simulated with this group */
    const double *yield;         /* [nbars] photons per MeV of the bar's sector */
    const double *speed_k;       /* [nbars] extra delay per mm to the SiPM end (ns/mm) */
    const double *mu;            /* [nbars] extra attenuation (1/mm) */
    const double *dev;           /* [4 nbars] photon-yield factor per channel */
    const double *ck_scint, *ck_fiber; /* [n][2] (beta, photons per mm), beta ascending */
    const int64_t *pdg_code;     /* [npdg] ascending particle codes; ions (|code| >= 1e9) are decoded */
    const double *pdg_mass, *pdg_charge;
    double half_length;          /* of the group's table (mm) */
    int32_t reflector, nbars, nck_scint, nck_fiber, npdg, pad;
} CrvLookupGroup;

typedef struct CrvSubstepRowsOut {
    double *s, *d, *t0, *t1, *beta, *cos_theta, *dev, *mu;
    int64_t *nsub, *step, *chan, *n_scint, *n_ck_s, *n_ck_f;
} CrvSubstepRowsOut;

int64_t crv_lookup_rows_workspace(int64_t nsteps);
int crv_lookup_rows(const CrvLookupGroup *G, uint32_t seed, const CrvLookupSteps *st, int64_t nsteps,
                    CrvSubstepRowsOut *out, int64_t cap, int64_t *n_rows_dev, void *workspace, int64_t workspace_bytes,
                    void *stream, CrvStatus *status_dev);

int64_t crv_substeps_workspace(int64_t nrows);
/* Photons of every row, in (row, substep, table, arrival) order: step index, channel, arrival time (capacity cap;
 * *n_out_dev receives the count). */
int crv_substep_photons(const CrvLookup *L, uint32_t seed, const CrvSubstepRows *rows, int64_t nrows,
                        int64_t *o_step, int64_t *o_chan, double *o_time, int64_t cap, int64_t *n_out_dev,
                        void *workspace, int64_t workspace_bytes, void *stream, CrvStatus *status_dev);

/*
 * The resident chain with the lookup-table photon model: chain.charges with lookup tables (crv/crvfastsim/chain.py:
 * 197-213) inside crv_chain.  The photons of every (step, SiPM) row come from the lookup model instead of the analytic
 * one: rows as crv_lookup_rows makes them (keyed by the step's row in the batch), photons as crv_substep_photons draws
 * them; SiPMs with status bit 0 or 2 get none; a SiPM's photons are in (step, substep, table, arrival) order, with
 * draw key = their index in the SiPM and photon id = the step's row, as chain.charges with lookup tables gives them to
 * sipm.simulate.  lk: the model's (table, reflector) groups (at most CRV_LOOKUP_CHAIN_GROUPS) with the table of each,
 * and the batch's steps in the model's form (row i of lk->steps is row i of st, whose bar column the chain groups
 * by).  The workspace holds 4 rows per step of caps->steps and the photons' times and ids (crv_chain_lookup_workspace).
 * crv_chain_graph_create_lookup captures a crv_chain_lookup call as crv_chain_graph_create captures crv_chain; the
 * lookup kernels read the seed from the graph's parameter block, so crv_chain_graph_set_params covers them too.
 */
#define CRV_LOOKUP_CHAIN_GROUPS 8
typedef struct CrvLookupChain {
    CrvLookupSteps steps;
    int32_t ngroups, pad;
    CrvLookupGroup group[CRV_LOOKUP_CHAIN_GROUPS];
    CrvLookup table[CRV_LOOKUP_CHAIN_GROUPS];   /* the lookup table of group g */
} CrvLookupChain;

int64_t crv_chain_lookup_workspace(const CrvParams *p, const CrvChainCaps *caps);
int crv_chain_lookup(const CrvParams *p, const CrvChainCaps *caps, const CrvEvents *ev, const int64_t *ev_keys,
                     const uint32_t *ev_runs, const CrvSteps *st, const int64_t *nsteps_dev, const CrvBars *bars,
                     const CrvChannels *ch, const CrvPixels *px, const double *tmpl, int32_t tlen,
                     const CrvFinderGeom *g, CrvClusters *out, CrvMembers *mem, int64_t *counts_dev, void *workspace,
                     int64_t workspace_bytes, void *stream, CrvStatus *status_dev, const CrvLookupChain *lk);
int crv_chain_graph_create_lookup(const CrvParams *p, const CrvChainCaps *caps, const CrvEvents *ev,
                                  const int64_t *ev_keys, const uint32_t *ev_runs, const CrvSteps *st,
                                  const int64_t *nsteps_dev, const CrvBars *bars, const CrvChannels *ch,
                                  const CrvPixels *px, const double *tmpl, int32_t tlen, const CrvFinderGeom *g,
                                  CrvClusters *out, CrvMembers *mem, int64_t *counts_dev, void *workspace,
                                  int64_t workspace_bytes, void *stream, CrvStatus *status_dev,
                                  const CrvLookupChain *lk, CrvChainGraph **graph_out);

/* ---- Lookup-table files (HOST memory, no device work) ------------------------------------------------------------
 * The Mu2e CRV photon lookup table, format version 6 (Offline CRVResponse MakeCrvPhotons), parsed from a file image:
 * replaces the reference's reader crvfastsim.response.lookup.load / _read_bins (crv/crvfastsim/response/lookup.py:
 * 108-179).  crv_lookup_file_info validates the whole image and fills the sizes; crv_lookup_file_read copies the
 * content into caller-allocated host arrays sized from them.  A malformed image returns CRV_ERR_ARG with
 * info->error set: */
#define CRV_LUTF_VERSION 1     /* error_a.error_b = the file's version (6.x expected) */
#define CRV_LUTF_BIN_NUMBER 2  /* bin number error_a found at position error_b */
#define CRV_LUTF_TRAILING 3    /* error_a bytes after the last bin */
#define CRV_LUTF_TRUNCATED 4   /* the image ends inside a record (at byte error_a) */
#define CRV_LUTF_SIZE 5        /* an empty bin-edge vector (error_a = its index) or table sizes beyond the image */

typedef struct CrvLookupFileInfo {
    int32_t version_major, version_minor, reflector;
    int32_t error;
    int64_t error_a, error_b;
    double constants[10];        /* half_thickness, half_width, half_length, fiber_separation, hole_radius_x,
                                    hole_radius_y, fiber_radius, corner_radius, birks, fiber_decay_time */
    int64_t n_ck[2];             /* Cerenkov map entries: scintillator, fibre */
    int64_t n_edges[7];          /* bin edges: x, y, z, beta, theta, phi, r */
    int64_t n_bins[3];           /* scint [x,y,z], ckscint [x,y,z,beta], ckfiber [beta,theta,phi,r,z] */
    int64_t delay_width[3];      /* longest delay-weight vector of each table (at least 1) */
    int64_t emis_width[3];       /* longest emission-weight vector of each table (at least 1) */
} CrvLookupFileInfo;

typedef struct CrvLookupFileTable {
    float *prob;                 /* [n_bins] arrival probability */
    uint8_t *delays;             /* [n_bins][delay_width] weights, zero-padded */
    int32_t *delay_sum;          /* [n_bins] */
    uint8_t *emis;               /* [n_bins][emis_width] weights, zero-padded */
    int32_t *emis_sum;           /* [n_bins] */
} CrvLookupFileTable;

typedef struct CrvLookupFileOut {
    double *ck[2];               /* [n_ck][2] (beta, photons per mm) */
    double *edges[7];            /* [n_edges] */
    CrvLookupFileTable tables[3];
} CrvLookupFileOut;

int crv_lookup_file_info(const uint8_t *image, int64_t size, CrvLookupFileInfo *info);
int crv_lookup_file_read(const uint8_t *image, int64_t size, const CrvLookupFileInfo *info,
                         const CrvLookupFileOut *out);

/* ROOT "L4" compression blocks (host code).  crv_lz4_block_decompress decodes one LZ4 block (src, n bytes) into dst
 * (cap bytes) and returns the bytes written, or a negative status for a malformed block (nothing is read or written
 * outside the two buffers).  crv_xxh64 is the XXH64 hash ROOT stores, big-endian, in front of each block. */
int64_t crv_lz4_block_decompress(const uint8_t *src, int64_t n, uint8_t *dst, int64_t cap);
uint64_t crv_xxh64(const uint8_t *data, int64_t n, uint64_t seed);

#ifdef __cplusplus
}
#endif
#endif
