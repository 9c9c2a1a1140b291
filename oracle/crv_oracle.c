/*
 * CPU oracle for the CRV response chain: TEST INFRASTRUCTURE ONLY.
 *
 * Only the test suite, the smoke check and the CPU-baseline leg of the benchmark load this library, and only as
 * the checker (never as the product path).  It restates, in plain C and serially, the stochastic stages of the
 * reference CRV response with the project's keyed Philox draws:
 *
 *   - photon counts per (step, SiPM): Gauss(mean, sqrt mean) if mean > 10 else Poisson(mean), then rint and a floor
 *     at zero  (crv/crvfastsim/response/photons.py:102-112, _draw_counts/_per_substep with one substep);
 *   - per-SiPM mirroring of the readout end (photons.py:333-356): SiPMs 0 and 2 read the -length end, 1 and 3 the
 *     +length end; the lookup-table probabilities are replaced by the analytic yield x two-exponential attenuation;
 *   - SiPM pixel draw from the photon-map CDF (crv/crvfastsim/response/sipm.py:80-91; "truncate" or "lrint" pixel
 *     ids over the 41 x 41 pixel state);
 *   - the serial SiPM model (sipm.py:141-198): per SiPM, photons in time order; a pixel fires with
 *     p1 (1 - exp(-v/p2)), v = Vov (1 - exp(-(t - t_last)/tau)); cross-talk breadth-first to the 4 neighbours with
 *     multiplicity merging 1 - (1 - p)^m; trap afterpulses scheduled per firing and processed after all photons in
 *     time order; charges sorted by time (stable).
 *
 * Every draw is keyed by (seed, run, subrun, event, channel, step-in-event, photon, node) through Philox4x32-10
 * (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy as 1, 2, 3", SC'11), written from the paper.
 * The exponential, logarithm and sin/cos(pi x) used by the draws and the SiPM recovery are this project's own
 * (Cody-Waite reduction + Taylor series; atanh series; Taylor series of sin/cos(pi x) on [0, 1/4]), so that the
 * FP64 device kernels, which implement the same steps with the same fused multiply-adds, agree bit for bit.
 *
 * Build: gcc -O2 -fPIC -shared -ffp-contract=off (no contraction: every fma below is explicit).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------------------------------------------ */
/* Philox4x32-10                                                                                                  */

#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void orc_philox(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += PHILOX_W0; k1 += PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Stage tags and counter layout (word 2): bits 0-14 channel, 15-17 call, 18-23 node index, 24-27 generation,
 * 28-31 stage.  Word 3: step-in-event << 16 | photon (or a stage-specific id).  Word 0 = event, word 1 = subrun.
 * Key = (seed, run). */
enum { ST_COUNT = 1, ST_PHOTON = 2, ST_SIPM = 3, ST_TDC0 = 4, ST_NOISE = 5, ST_STEPS = 6 };

static inline void keyed(uint32_t seed, uint32_t run, uint32_t event, uint32_t subrun, uint32_t w2, uint32_t w3,
                         uint32_t out[4]) {
    uint32_t c[4] = {event, subrun, w2, w3};
    uint32_t k[2] = {seed, run};
    orc_philox(c, k, out);
}

static inline uint32_t w2_of(int stage, int gen, int idx, int call, int chan) {
    return ((uint32_t)stage << 28) | ((uint32_t)gen << 24) | ((uint32_t)idx << 18) | ((uint32_t)call << 15)
           | ((uint32_t)chan & 0x7FFFu);
}

/* 53-bit uniforms from two words: [0, 1) and (0, 1]. */
static inline uint64_t bits53(uint32_t a, uint32_t b) { return (((uint64_t)a << 32) | b) >> 11; }
static inline double u01(uint32_t a, uint32_t b) { return (double)bits53(a, b) * 0x1p-53; }
static inline double u01_open(uint32_t a, uint32_t b) { return (double)(bits53(a, b) + 1) * 0x1p-53; }

/* ------------------------------------------------------------------------------------------------------------ */
/* exp, log, sincospi                                                                                             */

static const double LN2_HI = 0x1.62e42fefa39efp-1;     /* ln 2 rounded to double            */
static const double LN2_LO = 0x1.abc9e3b39803fp-56;    /* ln 2 - LN2_HI rounded to double   */
static const double INV_LN2 = 0x1.71547652b82fep+0;    /* 1 / ln 2 rounded to double        */

static inline double pow2i(int n) {                     /* 2^n for -1022 <= n <= 1023, exact */
    uint64_t b = (uint64_t)(n + 1023) << 52;
    double r;
    memcpy(&r, &b, 8);
    return r;
}

double orc_exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.2) return 0.0;
    double n = rint(x * INV_LN2);
    double r = fma(-n, LN2_HI, x);
    r = fma(-n, LN2_LO, r);
    /* Taylor series of e^r to degree 13 (|r| <= ln2/2 + tiny: truncation < 5e-18), coefficients 1/k!. */
    double p = 1.6059043836821613e-10;         /* 1/13! */
    p = fma(p, r, 2.08767569878681e-09);       /* 1/12! */
    p = fma(p, r, 2.505210838544172e-08);      /* 1/11! */
    p = fma(p, r, 2.755731922398589e-07);      /* 1/10! */
    p = fma(p, r, 2.7557319223985893e-06);     /* 1/9!  */
    p = fma(p, r, 2.48015873015873e-05);       /* 1/8!  */
    p = fma(p, r, 0.0001984126984126984);      /* 1/7!  */
    p = fma(p, r, 0.001388888888888889);       /* 1/6!  */
    p = fma(p, r, 0.008333333333333333);       /* 1/5!  */
    p = fma(p, r, 0.041666666666666664);       /* 1/4!  */
    p = fma(p, r, 0.16666666666666666);        /* 1/3!  */
    p = fma(p, r, 0.5);
    p = fma(p, r, 1.0);
    p = fma(p, r, 1.0);
    int k = (int)n;
    if (k > 1023) return (p * pow2i(1023)) * pow2i(k - 1023);
    if (k < -1020) return (p * pow2i(-60)) * pow2i(k + 60);
    return p * pow2i(k);
}

double orc_log(double x) {
    if (x != x || x < 0.0) return NAN;
    if (x == 0.0) return -INFINITY;
    if (isinf(x)) return x;
    int e = 0;
    if (x < 0x1p-1022) { x *= 0x1p54; e = -54; }       /* subnormal: scale up exactly */
    uint64_t b;
    memcpy(&b, &x, 8);
    e += (int)((b >> 52) & 0x7FF) - 1023;
    b = (b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;   /* m in [1, 2) */
    double m;
    memcpy(&m, &b, 8);
    if (m > 1.4142135623730951) { m *= 0.5; e += 1; }          /* m in (sqrt2/2, sqrt2] */
    double f = m - 1.0;
    double s = f / (2.0 + f);
    double w = s * s;
    /* log m = 2 atanh s = 2 s (1 + w/3 + w^2/5 + ... + w^11/23) */
    double q = 0.043478260869565216;           /* 1/23 */
    q = fma(q, w, 0.047619047619047616);       /* 1/21 */
    q = fma(q, w, 0.05263157894736842);        /* 1/19 */
    q = fma(q, w, 0.058823529411764705);       /* 1/17 */
    q = fma(q, w, 0.06666666666666667);        /* 1/15 */
    q = fma(q, w, 0.07692307692307693);        /* 1/13 */
    q = fma(q, w, 0.09090909090909091);        /* 1/11 */
    q = fma(q, w, 0.1111111111111111);         /* 1/9  */
    q = fma(q, w, 0.14285714285714285);        /* 1/7  */
    q = fma(q, w, 0.2);                        /* 1/5  */
    q = fma(q, w, 0.3333333333333333);         /* 1/3  */
    double t = 2.0 * s;
    double lm = fma(t * w, q, t);
    double de = (double)e;
    return fma(de, LN2_HI, fma(de, LN2_LO, lm));
}

/* sin(pi b), cos(pi b) for b in [0, 1/4]: Taylor series in b. */
static inline double sinpi_q(double b) {
    double w = b * b;
    double p = 7.952054001475513e-07;
    p = fma(p, w, -2.1915353447830217e-05);
    p = fma(p, w, 0.00046630280576761255);
    p = fma(p, w, -0.0073704309457143504);
    p = fma(p, w, 0.08214588661112823);
    p = fma(p, w, -0.5992645293207921);
    p = fma(p, w, 2.5501640398773455);
    p = fma(p, w, -5.16771278004997);
    p = fma(p, w, 3.141592653589793);
    return p * b;
}

static inline double cospi_q(double b) {
    double w = b * b;
    double p = -1.3878952462213771e-07;
    p = fma(p, w, 4.303069587032947e-06);
    p = fma(p, w, -0.0001046381049248457);
    p = fma(p, w, 0.0019295743094039231);
    p = fma(p, w, -0.02580689139001406);
    p = fma(p, w, 0.2353306303588932);
    p = fma(p, w, -1.3352627688545895);
    p = fma(p, w, 4.0587121264167685);
    p = fma(p, w, -4.934802200544679);
    p = fma(p, w, 1.0);
    return p;
}

/* sin(pi x), cos(pi x) for x in [0, 2]. */
void orc_sincospi(double x, double *sp, double *cp) {
    double y = x - 2.0 * rint(0.5 * x);         /* y in [-1, 1], exact */
    double sg = 1.0;
    if (y < 0.0) { y = -y; sg = -1.0; }         /* sin odd, cos even */
    double s, c;
    if (y <= 0.25) {
        s = sinpi_q(y); c = cospi_q(y);
    } else if (y <= 0.75) {
        double b = 0.5 - y;                     /* exact */
        s = cospi_q(b); c = sinpi_q(b);
    } else {
        double b = 1.0 - y;                     /* exact */
        s = sinpi_q(b); c = -cospi_q(b);
    }
    *sp = sg * s;
    *cp = c;
}

/* Box-Muller pair from one Philox block (u1 in (0,1] from words 0,1; u2 in [0,1) from words 2,3). */
static inline void normal_pair(const uint32_t w[4], double *z0, double *z1) {
    double u1 = u01_open(w[0], w[1]);
    double u2 = u01(w[2], w[3]);
    double r = sqrt(-2.0 * orc_log(u1));
    double s, c;
    orc_sincospi(2.0 * u2, &s, &c);
    *z0 = r * c;
    *z1 = r * s;
}

/* Poisson(lam) by inversion for lam <= 10 (u in [0, 1)). */
static inline int64_t poisson_inv(double lam, double u) {
    double p = orc_exp(-lam);
    double F = p;
    int64_t k = 0;
    while (u >= F && k < 200) {
        k += 1;
        p = p * lam / (double)k;
        F = F + p;
    }
    return k;
}

/* Photon count for one (step, SiPM) row: the reference rule with one substep. */
static inline int64_t draw_count(double avg, const uint32_t w[4]) {
    double x;
    if (avg > 10.0) {
        double z0, z1;
        normal_pair(w, &z0, &z1);
        x = avg + sqrt(avg) * z0;
    } else {
        double lam = avg > 0.0 ? avg : 0.0;
        x = (double)poisson_inv(lam, u01(w[0], w[1]));
    }
    x = rint(x);
    return x > 0.0 ? (int64_t)x : 0;
}

/* ------------------------------------------------------------------------------------------------------------ */
/* Parameters                                                                                                     */

typedef struct {
    uint32_t seed;
    uint32_t pad0;
    /* photons */
    double yield_per_mev;       /* PE per MeV per SiPM */
    double frac_short;          /* attenuation: frac_short e^{-d/lambda_short} + frac_long e^{-d/lambda_long} */
    double frac_long;
    double lambda_short;        /* mm */
    double lambda_long;         /* mm */
    double signal_speed;        /* mm/ns along the fibre */
    double decay_time;          /* ns, exponential emission delay */
    /* SiPM */
    double overvoltage, time_constant, capacitance, p1, p2;
    double q_ct;                /* per-neighbour cross-talk probability per firing */
    double q_t0, q_t1;          /* trap probability per firing */
    double trap0_lifetime, trap1_lifetime;
    double t_end;
    int32_t n_pixels_x, n_pixels_y;
    int32_t pixel_lrint, pad1;            /* pixel id: 0 "truncate", 1 "lrint" */
} OrcParams;

static inline double p_fire(const OrcParams *P, double v) { return P->p1 * (1.0 - orc_exp(-v / P->p2)); }

/* ------------------------------------------------------------------------------------------------------------ */
/* Photon stage                                                                                                   */

/* Readout distance of SiPM s from a step at length coordinate z (relative to the bar centre). */
static inline double readout_distance(double z, double half, int s) {
    double d = (s % 2 == 0) ? (z + half) : (half - z);
    if (d < 0.0) d = 0.0;
    if (d > 2.0 * half) d = 2.0 * half;
    return d;
}

static inline double mean_photons(const OrcParams *P, double edep, double dev, double d) {
    double att = P->frac_short * orc_exp(-d / P->lambda_short) + P->frac_long * orc_exp(-d / P->lambda_long);
    return P->yield_per_mev * edep * dev * att;
}

/* Per step and SiPM s: photon count (rows = nsteps x 4, row = step * 4 + s).  zloc: length coordinate of the step
 * relative to the bar centre, half: half length of the step's bar, dev: yield factor of the row's channel.
 * sie: step index inside its event.  Rows with a non-finite time get 0. */
void orc_photon_counts(const OrcParams *P, int64_t nsteps, const int32_t *bar, const double *zloc, const double *t,
                       const double *edep, const double *half, const double *dev_chan, const uint32_t *event,
                       const uint32_t *subrun, const uint32_t *run, const int32_t *sie, int64_t *count) {
    for (int64_t i = 0; i < nsteps; ++i) {
        for (int s = 0; s < 4; ++s) {
            int64_t row = i * 4 + s;
            if (!isfinite(t[i])) { count[row] = 0; continue; }
            int chan = bar[i] * 4 + s;
            double d = readout_distance(zloc[i], half[i], s);
            double avg = mean_photons(P, edep[i], dev_chan[chan], d);
            uint32_t w[4];
            keyed(P->seed, run[i], event[i], subrun[i], w2_of(ST_COUNT, 0, 0, 0, chan), (uint32_t)sie[i], w);
            count[row] = draw_count(avg, w);
        }
    }
}

/* Emission delays of a row's n photons in increasing order, in units of the decay time: the order statistics of n
 * exponential delays by the Renyi representation, S_j = sum_{i <= j} X_i / (n - i) with X_i = -log u_i and u_i photon
 * i's keyed uniform.  The set of delays has the distribution of n independent exponential delays (the reference's
 * model); photon j of the row (key j) takes the j-th smallest, so a row's photons come out in time order.  The sums
 * run in the GPU's order: chunks of 32 photons, an inclusive Hillis-Steele scan inside a chunk (offsets 1, 2, 4, 8,
 * 16), the running total of the earlier chunks added in front. */
static void row_delays(uint32_t seed, uint32_t run, uint32_t ev, uint32_t sub, int chan, int32_t sie, int64_t n,
                       double *S) {
    double carry = 0.0;
    for (int64_t c0 = 0; c0 < n; c0 += 32) {
        double v[32], nx[32];
        for (int l = 0; l < 32; ++l) {
            int64_t j = c0 + l;
            v[l] = 0.0;
            if (j < n) {
                uint32_t w[4];
                keyed(seed, run, ev, sub, w2_of(ST_PHOTON, 0, 0, 0, chan), ((uint32_t)sie << 16) | (uint32_t)(j >> 1),
                      w);
                int h = (int)(j & 1) * 2;
                v[l] = (-orc_log(u01_open(w[h], w[h + 1]))) / (double)(n - j);
            }
        }
        for (int off = 1; off < 32; off <<= 1) {
            for (int l = 0; l < 32; ++l) nx[l] = l >= off ? v[l] + v[l - off] : v[l];
            memcpy(v, nx, sizeof v);
        }
        for (int l = 0; l < 32 && c0 + l < n; ++l) S[c0 + l] = carry + v[l];
        carry = carry + v[31];
    }
}

/* Emit photons for rows with precomputed counts and offsets (row order = caller's).  Per photon: step row, channel,
 * time = step time + distance / signal speed + decay time x S_j (row_delays), key = (step-in-event << 16) | j. */
void orc_photon_emit(const OrcParams *P, int64_t nrows, const int64_t *row_step, const int32_t *row_s,
                     const int64_t *row_count, const int64_t *row_off, const int32_t *bar, const double *zloc,
                     const double *t, const double *half, const uint32_t *event, const uint32_t *subrun,
                     const uint32_t *run, const int32_t *sie, int64_t *o_step, int64_t *o_chan, double *o_time,
                     int64_t *o_key) {
    double *S = NULL;
    int64_t scap = 0;
    for (int64_t r = 0; r < nrows; ++r) {
        int64_t i = row_step[r];
        int s = row_s[r];
        int chan = bar[i] * 4 + s;
        int64_t n = row_count[r];
        if (n > scap) {
            scap = n;
            S = realloc(S, (size_t)scap * sizeof(double));
        }
        row_delays(P->seed, run[i], event[i], subrun[i], chan, sie[i], n, S);
        double d = readout_distance(zloc[i], half[i], s);
        for (int64_t j = 0; j < n; ++j) {
            int64_t o = row_off[r] + j;
            o_step[o] = i;
            o_chan[o] = chan;
            o_time[o] = t[i] + d / P->signal_speed + P->decay_time * S[j];
            o_key[o] = ((int64_t)sie[i] << 16) | j;
        }
    }
    free(S);
}

/* ------------------------------------------------------------------------------------------------------------ */
/* SiPM stage                                                                                                     */

#define NPX 1600                          /* photon-map bins, x * 40 + y */
#define PXS 41                            /* pixel ids x * 41 + y over the 41 x 41 state (sipm.py:22 NPIX = 41) */
#define NPS (PXS * PXS)
#define MAX_GEN 15
#define MAX_IDX 63

typedef struct { double t; int64_t key; int64_t photon; } Ph;
typedef struct { int pix; int m; } Node;
typedef struct { double t; int pix; int64_t photon; double u_fire; int64_t ord; } Trap;

static int cmp_ph(const void *a, const void *b) {
    const Ph *x = a, *y = b;
    if (x->t < y->t) return -1;
    if (x->t > y->t) return 1;
    return (x->key < y->key) ? -1 : (x->key > y->key);
}

static int cmp_trap(const void *a, const void *b) {
    const Trap *x = a, *y = b;
    if (x->t < y->t) return -1;
    if (x->t > y->t) return 1;
    return (x->ord < y->ord) ? -1 : (x->ord > y->ord);
}

typedef struct { double t; int64_t ord; } TimeOrd;

static int cmp_time_ord(const void *a, const void *b) {
    const TimeOrd *x = a, *y = b;
    if (x->t < y->t) return -1;
    if (x->t > y->t) return 1;
    return (x->ord < y->ord) ? -1 : (x->ord > y->ord);
}

static int cmp_int(const void *a, const void *b) { return *(const int *)a - *(const int *)b; }

typedef struct {
    double *t, *v;
    int64_t *photon;
    int64_t n, cap;
} ChargeBuf;

static void push_charge(ChargeBuf *C, double t, double v, int64_t photon) {
    if (C->n == C->cap) {
        C->cap = C->cap ? 2 * C->cap : 256;
        C->t = realloc(C->t, C->cap * sizeof(double));
        C->v = realloc(C->v, C->cap * sizeof(double));
        C->photon = realloc(C->photon, C->cap * sizeof(int64_t));
    }
    C->t[C->n] = t; C->v[C->n] = v; C->photon[C->n] = photon;
    C->n++;
}

/* Pixel of a photon (crv/crvfastsim/response/sipm.py:80-91): the photon-map bin by the CDF (cum: 1600 running sums
 * over bins x * 40 + y), then its pixel id x * 41 + y: "truncate" keeps the bin, "lrint" rounds the point in it, i.e.
 * adds 1 to x and to y each with probability 1/2 (bits 0 and 1 of `half`, the draw word whose low 11 bits the bin
 * uniform drops).  Returns -1 for a dead pixel. */
static inline int draw_pixel(const double *cum, const uint8_t *dead, double u, int lrint, uint32_t half) {
    double v = u * cum[NPX - 1];
    int lo = 0, hi = NPX;                        /* first index with cum > v (searchsorted side="right") */
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (cum[mid] <= v) lo = mid + 1; else hi = mid;
    }
    if (lo >= NPX) lo = NPX - 1;
    int x = lo / 40, y = lo % 40;
    if (lrint) { x += (int)(half & 1u); y += (int)((half >> 1) & 1u); }
    int q = x * PXS + y;
    return dead[q] ? -1 : q;
}

/* Simulate one SiPM.  photons sorted by (t, key) already, t <= t_end.  Returns status (0 ok, 2 limit). */
static int sipm_one(const OrcParams *P, const double *cum, const uint8_t *dead, uint32_t run, uint32_t ev,
                    uint32_t sub, int chan, const Ph *ph, int64_t n, ChargeBuf *out, int64_t *n_fired_pix) {
    double last[NPS];
    for (int i = 0; i < NPS; ++i) last[i] = -INFINITY;
    Trap *traps = NULL;
    int64_t ntr = 0, captr = 0;
    int status = 0;
    const int NX = P->n_pixels_x, NY = P->n_pixels_y;
    for (int64_t k = 0; k < n; ++k) {
        uint32_t w3 = (uint32_t)ph[k].key;
        uint32_t w[4];
        keyed(P->seed, run, ev, sub, w2_of(ST_SIPM, 0, 0, 0, chan), w3, w);
        int pix = draw_pixel(cum, dead, u01(w[0], w[1]), P->pixel_lrint, w[1]);
        if (pix < 0) continue;
        double t = ph[k].t;
        Node fr[MAX_IDX + 1], nx[4 * (MAX_IDX + 1)];
        int nfr = 1;
        fr[0].pix = pix; fr[0].m = 1;
        int gen = 0;
        while (nfr > 0) {
            int fired[MAX_IDX + 1];
            double fv[MAX_IDX + 1];
            int nf = 0;
            for (int i = 0; i < nfr; ++i) {
                int p = fr[i].pix;
                double v = P->overvoltage * (1.0 - orc_exp(-(t - last[p]) / P->time_constant));
                double pf = p_fire(P, v);
                double q = 1.0 - pf, qm = q;
                for (int mm = 1; mm < fr[i].m; ++mm) qm = qm * q;
                double pm = 1.0 - qm;
                uint32_t wf[4];
                if (gen == 0) { wf[2] = w[2]; wf[3] = w[3]; }
                else keyed(P->seed, run, ev, sub, w2_of(ST_SIPM, gen, i, 0, chan), w3, wf);
                if (u01(wf[2], wf[3]) < pm) { fired[nf] = i; fv[nf] = v; nf++; }
            }
            for (int a = 0; a < nf; ++a) {
                int p = fr[fired[a]].pix;
                last[p] = t;
                push_charge(out, t, fv[a], ph[k].photon);
            }
            /* traps: call 1 -> (u_trap0, u_trap0_time), call 4 -> (u_trap0_fire, u_trap1),
             *        call 5 -> (u_trap1_time, u_trap1_fire) */
            if (P->q_t0 > 0.0 || P->q_t1 > 0.0) {
                for (int a = 0; a < nf; ++a) {
                    int i = fired[a];
                    uint32_t w1[4], w4[4], w5[4];
                    keyed(P->seed, run, ev, sub, w2_of(ST_SIPM, gen, i, 1, chan), w3, w1);
                    keyed(P->seed, run, ev, sub, w2_of(ST_SIPM, gen, i, 4, chan), w3, w4);
                    for (int tr = 0; tr < 2; ++tr) {
                        double q = tr ? P->q_t1 : P->q_t0;
                        if (!(q > 0.0)) continue;
                        double ud, ut, uf;
                        if (tr == 0) { ud = u01(w1[0], w1[1]); ut = u01_open(w1[2], w1[3]); uf = u01(w4[0], w4[1]); }
                        else {
                            keyed(P->seed, run, ev, sub, w2_of(ST_SIPM, gen, i, 5, chan), w3, w5);
                            ud = u01(w4[2], w4[3]); ut = u01_open(w5[0], w5[1]); uf = u01(w5[2], w5[3]);
                        }
                        if (ud < q) {
                            double life = tr ? P->trap1_lifetime : P->trap0_lifetime;
                            if (ntr == captr) { captr = captr ? 2 * captr : 64; traps = realloc(traps, captr * sizeof(Trap)); }
                            traps[ntr].t = t - life * orc_log(ut);
                            traps[ntr].pix = fr[i].pix;
                            traps[ntr].photon = ph[k].photon;
                            traps[ntr].u_fire = uf;
                            traps[ntr].ord = ntr;
                            ntr++;
                        }
                    }
                }
            }
            /* cross-talk: call 2 -> (u_ct0, u_ct1), call 3 -> (u_ct2, u_ct3); neighbours x-1, x+1, y-1, y+1 */
            int nn = 0;
            for (int a = 0; a < nf; ++a) {
                int i = fired[a];
                int p = fr[i].pix, x = p / PXS, y = p % PXS;
                uint32_t c2[4], c3[4];
                keyed(P->seed, run, ev, sub, w2_of(ST_SIPM, gen, i, 2, chan), w3, c2);
                keyed(P->seed, run, ev, sub, w2_of(ST_SIPM, gen, i, 3, chan), w3, c3);
                double u[4] = {u01(c2[0], c2[1]), u01(c2[2], c2[3]), u01(c3[0], c3[1]), u01(c3[2], c3[3])};
                int nxp[4] = {(x - 1) * PXS + y, (x + 1) * PXS + y, x * PXS + y - 1, x * PXS + y + 1};
                int ok[4] = {x > 0, x + 1 < NX, y > 0, y + 1 < NY};
                for (int q = 0; q < 4; ++q)
                    if (ok[q] && u[q] < P->q_ct) { nx[nn].pix = nxp[q]; nn++; }
            }
            /* next frontier: unique pixels in increasing order with multiplicity, dead removed */
            int pl[4 * (MAX_IDX + 1)];
            for (int a = 0; a < nn; ++a) pl[a] = nx[a].pix;
            qsort(pl, nn, sizeof(int), cmp_int);
            nfr = 0;
            for (int a = 0; a < nn;) {
                int b = a;
                while (b < nn && pl[b] == pl[a]) b++;
                if (!dead[pl[a]]) {
                    if (nfr > MAX_IDX) { status = 2; break; }
                    fr[nfr].pix = pl[a]; fr[nfr].m = b - a; nfr++;
                }
                a = b;
            }
            gen++;
            if (nfr > 0 && gen > MAX_GEN) { status = 2; nfr = 0; }
        }
    }
    /* afterpulses: after all photons, in time order, no cascades */
    if (ntr) {
        qsort(traps, ntr, sizeof(Trap), cmp_trap);
        for (int64_t a = 0; a < ntr; ++a) {
            double t1 = traps[a].t;
            if (t1 > P->t_end) continue;
            int p = traps[a].pix;
            double v = P->overvoltage * (1.0 - orc_exp(-(t1 - last[p]) / P->time_constant));
            if (traps[a].u_fire < p_fire(P, v)) {
                last[p] = t1;
                push_charge(out, t1, v, traps[a].photon);
            }
        }
    }
    free(traps);
    int64_t nfp = 0;
    for (int i = 0; i < NPS; ++i) nfp += (last[i] > -INFINITY);
    if (n_fired_pix) *n_fired_pix = nfp;
    return status;
}

/* Stable merge of the SiPM's charge records [a0, n) by time (records before the afterpulses are already in
 * non-decreasing time order; afterpulses are sorted by time). */
static void stable_time_sort(ChargeBuf *C, int64_t a0) {
    int64_t n = C->n - a0;
    if (n < 2) return;
    TimeOrd *k = malloc(n * sizeof(TimeOrd));
    for (int64_t i = 0; i < n; ++i) { k[i].t = C->t[a0 + i]; k[i].ord = i; }
    qsort(k, n, sizeof(TimeOrd), cmp_time_ord);
    double *t = malloc(n * sizeof(double)), *v = malloc(n * sizeof(double));
    int64_t *ph = malloc(n * sizeof(int64_t));
    for (int64_t i = 0; i < n; ++i) {
        t[i] = C->t[a0 + k[i].ord]; v[i] = C->v[a0 + k[i].ord]; ph[i] = C->photon[a0 + k[i].ord];
    }
    memcpy(C->t + a0, t, n * sizeof(double));
    memcpy(C->v + a0, v, n * sizeof(double));
    memcpy(C->photon + a0, ph, n * sizeof(int64_t));
    free(k); free(t); free(v); free(ph);
}

/* Test hook: the pixel ids (x * 41 + y, -1 for a dead pixel) drawn for photons with the given draw keys on one SiPM
 * (channel chan of event (run, subrun, event)), as the SiPM stage draws them. */
void orc_sipm_pixels(const OrcParams *P, const double *cum, const uint8_t *dead, uint32_t run, uint32_t ev,
                     uint32_t sub, int chan, const int64_t *key, int64_t n, int32_t *out) {
    for (int64_t k = 0; k < n; ++k) {
        uint32_t w[4];
        keyed(P->seed, run, ev, sub, w2_of(ST_SIPM, 0, 0, 0, chan), (uint32_t)key[k], w);
        out[k] = draw_pixel(cum, dead, u01(w[0], w[1]), P->pixel_lrint, w[1]);
    }
}

/* SiPM stage over photons grouped by SiPM: groups [gstart[g], gstart[g] + gcount[g]) of the photon arrays, each
 * one SiPM (channel chan_of[g] of event (run, subrun, event)[g]).  Photons need not be sorted.  Outputs are
 * allocated here (free with orc_free) in group order, time-sorted within a group.  Per group: charge count and
 * fired-pixel count. */
int orc_sipm_groups(const OrcParams *P, const double *cum, const uint8_t *dead, int64_t ngroups,
                    const int64_t *gstart, const int64_t *gcount, const int32_t *chan_of, const uint32_t *g_event,
                    const uint32_t *g_subrun, const uint32_t *g_run, const double *time, const int64_t *key,
                    const int64_t *photon, int64_t *n_charges_per_group, int64_t *n_fired_pix_per_group,
                    int64_t *n_out, double **o_time, double **o_v, int64_t **o_photon) {
    ChargeBuf C = {0};
    int status = 0;
    Ph *buf = NULL;
    int64_t capb = 0;
    for (int64_t g = 0; g < ngroups; ++g) {
        int64_t n = 0;
        if (gcount[g] > capb) { capb = gcount[g]; buf = realloc(buf, capb * sizeof(Ph)); }
        for (int64_t i = 0; i < gcount[g]; ++i) {
            int64_t a = gstart[g] + i;
            if (!(time[a] <= P->t_end)) continue;
            buf[n].t = time[a]; buf[n].key = key[a]; buf[n].photon = photon[a]; n++;
        }
        qsort(buf, n, sizeof(Ph), cmp_ph);
        int64_t a0 = C.n;
        int st = sipm_one(P, cum, dead, g_run[g], g_event[g], g_subrun[g], chan_of[g], buf, n, &C,
                          &n_fired_pix_per_group[g]);
        if (st) status = st;
        stable_time_sort(&C, a0);
        n_charges_per_group[g] = C.n - a0;
    }
    free(buf);
    *n_out = C.n;
    *o_time = C.t; *o_v = C.v; *o_photon = C.photon;
    return status;
}

void orc_free(void *p) { free(p); }

/* ------------------------------------------------------------------------------------------------------------ */
/* TDC0 and electronics noise                                                                                     */

/* One uniform in [0, 1) per (event, FEB key). */
void orc_tdc0_uniform(uint32_t seed, int64_t n, const uint32_t *run, const uint32_t *event, const uint32_t *subrun,
                      const uint32_t *febkey, double *u) {
    for (int64_t i = 0; i < n; ++i) {
        uint32_t w[4];
        keyed(seed, run[i], event[i], subrun[i], (uint32_t)ST_TDC0 << 28, febkey[i], w);
        u[i] = u01(w[0], w[1]);
    }
}

/* Standard normal per (event, channel, tick). */
void orc_noise_normal(uint32_t seed, int64_t n, const uint32_t *run, const uint32_t *event, const uint32_t *subrun,
                      const int32_t *chan, const int64_t *tick, double *z) {
    for (int64_t i = 0; i < n; ++i) {
        uint32_t w[4];
        int64_t tk = tick[i];
        int64_t pair = tk >> 1;              /* arithmetic shift (floor division by 2) */
        keyed(seed, run[i], event[i], subrun[i], ((uint32_t)ST_NOISE << 28) | ((uint32_t)chan[i] & 0x7FFFu),
              (uint32_t)pair, w);
        double z0, z1;
        normal_pair(w, &z0, &z1);
        z[i] = (tk & 1) ? z1 : z0;
    }
}

/* Raw keyed block (for tests of the key layout). */
void orc_keyed_block(uint32_t seed, uint32_t run, uint32_t event, uint32_t subrun, uint32_t w2, uint32_t w3,
                     uint32_t out[4]) {
    keyed(seed, run, event, subrun, w2, w3, out);
}

/* Vector forms of the math functions (tests against libm). */
void orc_exp_v(int64_t n, const double *x, double *y) { for (int64_t i = 0; i < n; ++i) y[i] = orc_exp(x[i]); }
void orc_log_v(int64_t n, const double *x, double *y) { for (int64_t i = 0; i < n; ++i) y[i] = orc_log(x[i]); }
void orc_sincospi_v(int64_t n, const double *x, double *s, double *c) {
    for (int64_t i = 0; i < n; ++i) orc_sincospi(x[i], s + i, c + i);
}
/* Photon counts from given means (distribution tests): one row per mean, keyed by (event = i). */
void orc_counts_from_mean(uint32_t seed, int64_t n, const double *avg, int64_t *count) {
    for (int64_t i = 0; i < n; ++i) {
        uint32_t w[4];
        keyed(seed, 0, (uint32_t)i, 0, w2_of(ST_COUNT, 0, 0, 0, 0), 0, w);
        count[i] = draw_count(avg[i], w);
    }
}

/* ------------------------------------------------------------------------------------------------------------ */
/* Lookup-table photon model: photons._substep_photons (crv/crvfastsim/response/photons.py:139-224) over (step,   */
/* SiPM) rows with keyed draws: Binomial arrivals per (substep, table), delay and emission counts from the bin's  */
/* weights, Gamma(emissions) fibre decay as a sum of exponentials.                                              */

enum { ST_SUBSTEP = 7, SUB_CALL_BINOMIAL = 0, SUB_CALL_PHOTON = 1, SUB_CALL_GAMMA = 2 };
#define SUB_MAX_SUBSTEPS (1ll << 20)
#define SUB_MAX_ARRIVALS 4096
#define SUB_MAX_EMISSIONS 128

typedef struct {
    const float *prob;
    const uint8_t *delays;
    const int32_t *delay_sum;
    const uint8_t *emis;
    const int32_t *emis_sum;
    int32_t nbins, ndelay, nemis, pad;
} OrcLookupTable;

typedef struct {
    double half_thickness, half_width, half_length, fiber_separation, hole_radius_x, hole_radius_y, fiber_radius,
        corner_radius, fiber_decay_time;
    const double *edges[7];
    int32_t nedges[7];
    int32_t pad;
    const double *cos_phi_edges;
    OrcLookupTable table[3];
    const double *cos_theta_edges;
} OrcLookup;

typedef struct {
    const double *s, *d, *t0, *t1, *beta, *theta, *dev, *mu;
    const int64_t *nsub, *step, *chan, *n_scint, *n_ck_s, *n_ck_f;
    const double *cos_theta;
} OrcSubstepRows;

static inline void sub_block(uint32_t seed, int64_t step, int64_t chan, int tb, int call, int idx, int64_t k, int j,
                             uint32_t out[4]) {
    uint32_t c[4] = {(uint32_t)step, (uint32_t)((uint64_t)step >> 32), w2_of(ST_SUBSTEP, tb, idx, call, (int)chan),
                     ((uint32_t)k << 12) | (uint32_t)j};
    uint32_t key[2] = {seed, 0u};
    orc_philox(c, key, out);
}

/* Binomial(n, p): inversion on min(p, 1 - p) while the mean is at most 256 (Kachitvichyanukul & Schmeiser's BINV),
 * else the normal approximation, clipped to [0, n]. */
static int64_t sub_binomial(int64_t n, double p, const uint32_t w[4]) {
    if (n <= 0 || !(p > 0.0)) return 0;
    if (p >= 1.0) return n;
    int flip = p > 0.5;
    double q = flip ? 1.0 - p : p;
    double mean = (double)n * q;
    int64_t k;
    if (mean > 256.0) {
        double z0, z1;
        normal_pair(w, &z0, &z1);
        double x = rint(mean + sqrt(mean * (1.0 - q)) * z0);
        k = x < 0.0 ? 0 : (x > (double)n ? n : (int64_t)x);
    } else {
        double u = u01(w[0], w[1]);
        double s = q / (1.0 - q);
        double a = (double)(n + 1) * s;
        double r = orc_exp((double)n * orc_log(1.0 - q));
        k = 0;
        while (u > r && k < n) {
            u = u - r;
            k += 1;
            r = r * (a / (double)k - s);
        }
    }
    return flip ? n - k : k;
}

static int sub_find_bin(const double *e, int ne, double v) {
    if (!(v >= e[0]) || !(v <= e[ne - 1])) return -1;
    if (v == e[0]) return 0;
    int lo = 0, hi = ne;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (e[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo - 1;
}

static int sub_find_bin_cos(const double *ce, int ne, double c) {
    if (!(c <= ce[0]) || !(c >= ce[ne - 1])) return -1;
    if (c == ce[0]) return 0;
    int lo = 0, hi = ne;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (ce[mid] > c) lo = mid + 1; else hi = mid;
    }
    return lo - 1;
}

static int sub_first_reaching(const uint8_t *wts, int n, double thr) {
    int cum = 0;
    for (int j = 0; j < n; ++j) {
        cum += wts[j];
        if (!((double)cum < thr)) return j;
    }
    return n;
}

static void sub_bins(const OrcLookup *L, const OrcSubstepRows *R, int64_t r, int64_t k, int64_t nsub, int bb, int bth,
                     int bin[3], double *t_out, double *z_out) {
    double frac = ((double)k + 0.5) / (double)nsub;
    double x = R->s[3 * r] + R->d[3 * r] * frac;
    double y = R->s[3 * r + 1] + R->d[3 * r + 1] * frac;
    double z = R->s[3 * r + 2] + R->d[3 * r + 2] * frac;
    double t = R->t0[r] + (R->t1[r] - R->t0[r]) * frac;
    double half_sep = L->fiber_separation / 2.0;
    double ax = fabs(x), ay = fabs(y);
    int insc = ax < L->half_thickness && ay < L->half_width && fabs(z) < L->half_length;
    double ex = ax / L->hole_radius_x, ey = (ay - half_sep) / L->hole_radius_y;
    insc = insc && (ex * ex + ey * ey >= 1.0);
    double cx = L->half_thickness - L->corner_radius, cy = L->half_width - L->corner_radius;
    if (ax > cx && ay > cy) {
        double qx = ax - cx, qy = ay - cy;
        if (sqrt(qx * qx + qy * qy) > L->corner_radius) insc = 0;
    }
    double y0 = y + half_sep, y1 = y - half_sep;
    double r0 = sqrt(x * x + y0 * y0), r1 = sqrt(x * x + y1 * y1);
    int in0 = r0 <= L->fiber_radius, in1 = r1 <= L->fiber_radius;
    double ry = in1 ? y1 : y0, rr = in1 ? r1 : r0;
    double dx = R->d[3 * r], dy = R->d[3 * r + 1];
    double norm = sqrt(dx * dx + dy * dy) * rr;
    double c = 1.0;
    if (norm > 0.0) {
        c = (dx * x + dy * ry) / norm;
        c = c < -1.0 ? -1.0 : (c > 1.0 ? 1.0 : c);
    }
    int infb = fabs(z) < L->half_length && (in0 || in1) && !insc;
    int ny = L->nedges[1] - 1, nz = L->nedges[2] - 1, nb = L->nedges[3] - 1;
    int nth = L->nedges[4] - 1, nph = L->nedges[5] - 1, nr = L->nedges[6] - 1;
    int bx = sub_find_bin(L->edges[0], L->nedges[0], ax), by = sub_find_bin(L->edges[1], L->nedges[1], y);
    int bz = sub_find_bin(L->edges[2], L->nedges[2], z);
    int geo = bx >= 0 && by >= 0 && bz >= 0;
    bin[0] = (insc && geo) ? bz + by * nz + bx * ny * nz : -1;
    bin[1] = (insc && geo && bb >= 0) ? bb + bz * nb + by * nz * nb + bx * ny * nz * nb : -1;
    bin[2] = -1;
    if (infb && bb >= 0 && bth >= 0 && bz >= 0) {
        int bph = sub_find_bin_cos(L->cos_phi_edges, L->nedges[5], c);
        int br = sub_find_bin(L->edges[6], L->nedges[6], rr);
        if (bph >= 0 && br >= 0) bin[2] = bz + br * nz + bph * nr * nz + bth * nph * nr * nz + bb * nth * nph * nr * nz;
    }
    *t_out = t;
    *z_out = z;
}

static int64_t sub_arrivals(const OrcLookup *L, const OrcSubstepRows *R, uint32_t seed, int64_t r, int64_t k, int tb,
                            int bin, double z) {
    double pr = (double)L->table[tb].prob[bin] * R->dev[r];
    if (R->mu) pr = pr * orc_exp(-R->mu[r] * z);
    pr = pr < 1.0 ? pr : 1.0;
    int64_t n = tb == 0 ? R->n_scint[r] : (tb == 1 ? R->n_ck_s[r] : R->n_ck_f[r]);
    uint32_t w[4];
    sub_block(seed, R->step[r], R->chan[r], tb, SUB_CALL_BINOMIAL, 0, k, 0, w);
    return sub_binomial(n, pr, w);
}

static double sub_time(const OrcLookup *L, uint32_t seed, int64_t step, int64_t chan, int64_t k, int tb, int bin,
                       int j, double t, int *limit) {
    const OrcLookupTable *T = &L->table[tb];
    uint32_t w[4];
    sub_block(seed, step, chan, tb, SUB_CALL_PHOTON, 0, k, j, w);
    double thr = u01(w[0], w[1]) * (double)T->delay_sum[bin];
    double tt = t + (double)sub_first_reaching(T->delays + (int64_t)bin * T->ndelay, T->ndelay, thr);
    if (L->fiber_decay_time > 0.0) {
        double thr2 = u01(w[2], w[3]) * (double)T->emis_sum[bin];
        int ne = sub_first_reaching(T->emis + (int64_t)bin * T->nemis, T->nemis, thr2);
        if (ne > SUB_MAX_EMISSIONS) {
            *limit = 1;
        } else if (ne > 0) {
            double g = 0.0;
            for (int i = 0; i < ne; i += 2) {
                uint32_t v[4];
                sub_block(seed, step, chan, tb, SUB_CALL_GAMMA, i >> 1, k, j, v);
                g = g - orc_log(u01_open(v[0], v[1]));
                if (i + 1 < ne) g = g - orc_log(u01_open(v[2], v[3]));
            }
            tt = tt + g * L->fiber_decay_time;
        }
    }
    return tt;
}

/* Photons of every row in (row, substep, table, arrival) order.  Pass o_time = NULL to count only.  Returns the
 * photon count; *limit is set when a key limit was exceeded (those arrivals are dropped, as on the device). */
int64_t orc_substep_photons(const OrcLookup *L, uint32_t seed, const OrcSubstepRows *R, int64_t nrows, int64_t *o_step,
                            int64_t *o_chan, double *o_time, int *limit) {
    int64_t o = 0;
    *limit = 0;
    for (int64_t r = 0; r < nrows; ++r) {
        int64_t nsub = R->nsub[r];
        if (nsub > SUB_MAX_SUBSTEPS) { *limit = 1; continue; }
        if (nsub <= 0) continue;
        int bb = sub_find_bin(L->edges[3], L->nedges[3], R->beta[r]);
        int bth = R->theta ? sub_find_bin(L->edges[4], L->nedges[4], R->theta[r])
                           : sub_find_bin_cos(L->cos_theta_edges, L->nedges[4], R->cos_theta[r]);
        for (int64_t k = 0; k < nsub; ++k) {
            int bin[3];
            double t, z;
            sub_bins(L, R, r, k, nsub, bb, bth, bin, &t, &z);
            for (int tb = 0; tb < 3; ++tb) {
                if (bin[tb] < 0) continue;
                int64_t a = sub_arrivals(L, R, seed, r, k, tb, bin[tb], z);
                if (a >= SUB_MAX_ARRIVALS) { *limit = 1; continue; }
                for (int j = 0; j < (int)a; ++j, ++o) {
                    if (!o_time) continue;
                    o_step[o] = R->step[r];
                    o_chan[o] = R->chan[r];
                    o_time[o] = sub_time(L, seed, R->step[r], R->chan[r], k, tb, bin[tb], j, t, limit);
                }
            }
        }
    }
    return o;
}

/* Binomial draws of the substep sampler for tests: n[i], p[i] with the block keyed by (step i, chan 0, table 0, k 0). */
void orc_binomial_v(uint32_t seed, int64_t cnt, const int64_t *n, const double *p, int64_t *out) {
    for (int64_t i = 0; i < cnt; ++i) {
        uint32_t w[4];
        sub_block(seed, i, 0, 0, SUB_CALL_BINOMIAL, 0, 0, 0, w);
        out[i] = sub_binomial(n[i], p[i], w);
    }
}

/* Row preparation of the lookup-table model (photons.iter_rows, crv/crvfastsim/response/photons.py:292-356) for one
 * (table, reflector) group, with keyed per-substep counts; rows SiPM block by SiPM block, steps in order. */
enum { ST_LROWS = 8 };
#define AMU_MEV 931.49410242

typedef struct {
    const double *x0, *y0, *z0, *x1, *y1, *z1, *px0, *py0, *pz0, *p1, *t0, *t1, *edep, *len;
    const int32_t *bar;
    const int64_t *pdg;
} OrcLookupSteps;

typedef struct {
    const double *center;
    const int8_t *l2w;
    const int32_t *in_group;
    const double *yield, *speed_k, *mu, *dev, *ck_scint, *ck_fiber;
    const int64_t *pdg_code;
    const double *pdg_mass, *pdg_charge;
    double half_length;
    int32_t reflector, nbars, nck_scint, nck_fiber, npdg, pad;
} OrcLookupGroup;

static void lrow_particle(const OrcLookupGroup *G, int64_t pdg, double *m, double *q) {
    int lo = 0, hi = G->npdg;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (G->pdg_code[mid] < pdg) lo = mid + 1; else hi = mid;
    }
    if (lo < G->npdg && G->pdg_code[lo] == pdg) { *m = G->pdg_mass[lo]; *q = G->pdg_charge[lo]; return; }
    int64_t a = pdg < 0 ? -pdg : pdg;
    if (a >= 1000000000ll) {
        *m = (double)((a / 10) % 1000) * AMU_MEV;
        *q = (double)((a / 10000) % 1000) * (pdg < 0 ? -1.0 : 1.0);
    } else {
        *m = 0.0;
        *q = 0.0;
    }
}

/* stock beta from the mean of the start and end energies (massless: 1) */
static double lrow_beta(double m, double p0, double p1) {
    double e = 0.5 * (sqrt(p0 * p0 + m * m) + sqrt(p1 * p1 + m * m));
    double beta = 1.0;
    if (m > 0.0) {
        double g = e / m;
        double b2 = 1.0 - 1.0 / (g * g);
        b2 = b2 < 0.0 ? 0.0 : (b2 > 1.0 ? 1.0 : b2);
        beta = sqrt(b2);
    }
    return beta;
}

static double lrow_cerenkov(const double *map, int n, double beta, double q) {
    double x0 = 0.0, y0 = 0.0, v;
    int j = 0;
    while (j < n && map[2 * j] <= beta) { x0 = map[2 * j]; y0 = map[2 * j + 1]; ++j; }
    if (beta < 0.0) v = 0.0;
    else if (j == n) v = n > 0 ? map[2 * (n - 1) + 1] : 0.0;
    else v = (map[2 * j + 1] - y0) / (map[2 * j] - x0) * (beta - x0) + y0;
    return v * fabs(q);
}

static int64_t lrow_per_substep(double avg, int64_t nsub, const uint32_t w[4]) {
    double x;
    if (avg > 10.0) {
        double z0, z1;
        normal_pair(w, &z0, &z1);
        x = avg + sqrt(avg) * z0;
    } else {
        x = (double)poisson_inv(avg > 0.0 ? avg : 0.0, u01(w[0], w[1]));
    }
    double n = rint(x / (double)nsub);
    return n > 0.0 ? (int64_t)n : 0;
}

/* Returns the number of rows written (nsim x steps of the group). */
int64_t orc_lookup_rows(const OrcLookupGroup *G, uint32_t seed, const OrcLookupSteps *S, int64_t nsteps, double *o_s,
                        double *o_d, double *o_t0, double *o_t1, double *o_beta, double *o_ct, double *o_dev,
                        double *o_mu, int64_t *o_nsub, int64_t *o_step, int64_t *o_chan, int64_t *o_ns,
                        int64_t *o_ncs, int64_t *o_ncf) {
    int nsim = G->reflector == 0 ? 4 : 2;
    int64_t ng = 0;
    for (int64_t i = 0; i < nsteps; ++i) {
        int b = S->bar[i];
        if (b >= 0 && b < G->nbars && G->in_group[b] && isfinite(S->t0[i]) && isfinite(S->t1[i])) ++ng;
    }
    int64_t r0 = 0;
    for (int64_t i = 0; i < nsteps; ++i) {
        int b = S->bar[i];
        if (!(b >= 0 && b < G->nbars && G->in_group[b] && isfinite(S->t0[i]) && isfinite(S->t1[i]))) continue;
        const double *c = G->center + 3 * b;
        double ws[3] = {S->x0[i] - c[0], S->y0[i] - c[1], S->z0[i] - c[2]};
        double we[3] = {S->x1[i] - c[0], S->y1[i] - c[1], S->z1[i] - c[2]};
        double sl[3], el[3];
        for (int k = 0; k < 3; ++k) { int ax = G->l2w[3 * b + k]; sl[k] = ws[ax]; el[k] = we[ax]; }
        if (G->reflector < 0) { sl[2] = -sl[2]; el[2] = -el[2]; }
        double m, q;
        lrow_particle(G, S->pdg[i], &m, &q);
        double p0 = sqrt(S->px0[i] * S->px0[i] + S->py0[i] * S->py0[i] + S->pz0[i] * S->pz0[i]);
        double beta = lrow_beta(m, p0, S->p1[i]);
        double avg_s = G->yield[b] * S->edep[i];
        double avg_cs = lrow_cerenkov(G->ck_scint, G->nck_scint, beta, q) * S->len[i];
        double avg_cf = lrow_cerenkov(G->ck_fiber, G->nck_fiber, beta, q) * S->len[i];
        double k = G->speed_k[b];
        for (int si = 0; si < nsim; ++si) {
            int s = G->reflector == 0 ? si : 2 * si;
            double a[3] = {sl[0], sl[1], sl[2]}, bb[3] = {el[0], el[1], el[2]};
            if (s == 1 || s == 3) { a[2] = -a[2]; bb[2] = -bb[2]; }
            if (s == 2 || s == 3) { a[1] = -a[1]; bb[1] = -bb[1]; }
            double d[3] = {bb[0] - a[0], bb[1] - a[1], bb[2] - a[2]};
            double dl = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            double ct = 1.0;
            if (dl > 0.0) { ct = d[2] / dl; ct = ct < -1.0 ? -1.0 : (ct > 1.0 ? 1.0 : ct); }
            int64_t nsub = (int64_t)(dl / 0.1);
            nsub = nsub > 1 ? nsub : 1;
            int64_t chan_dev = 4ll * b + s;
            int64_t o = (int64_t)si * ng + r0;
            for (int x = 0; x < 3; ++x) { o_s[3 * o + x] = a[x]; o_d[3 * o + x] = d[x]; }
            o_t0[o] = S->t0[i] + k * (a[2] + G->half_length);
            o_t1[o] = S->t1[i] + k * (bb[2] + G->half_length);
            o_nsub[o] = nsub;
            o_beta[o] = beta;
            o_ct[o] = ct;
            o_dev[o] = G->dev[chan_dev];
            o_mu[o] = G->mu[b];
            o_step[o] = i;
            o_chan[o] = 4ll * b + (G->reflector < 0 ? s + 1 : s);
            uint32_t w[4];
            uint32_t ctr[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), 0, 0};
            uint32_t key[2] = {seed, 0u};
            ctr[2] = w2_of(ST_LROWS, 0, 0, 0, (int)chan_dev); orc_philox(ctr, key, w);
            o_ns[o] = lrow_per_substep(avg_s, nsub, w);
            ctr[2] = w2_of(ST_LROWS, 1, 0, 0, (int)chan_dev); orc_philox(ctr, key, w);
            o_ncs[o] = lrow_per_substep(avg_cs, nsub, w);
            ctr[2] = w2_of(ST_LROWS, 2, 0, 0, (int)chan_dev); orc_philox(ctr, key, w);
            o_ncf[o] = lrow_per_substep(avg_cf, nsub, w);
        }
        ++r0;
    }
    return nsim * ng;
}

/* Test hooks for the lookup model's helpers (the reference's own helper tests: crv/tests/test_photons.py:13-29). */
void orc_find_bin_v(const double *e, int ne, int64_t n, const double *v, int32_t *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = sub_find_bin(e, ne, v[i]);
}
void orc_find_bin_cos_v(const double *ce, int ne, int64_t n, const double *c, int32_t *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = sub_find_bin_cos(ce, ne, c[i]);
}
void orc_cerenkov_v(const double *map, int nmap, int64_t n, const double *beta, const double *q, double *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = lrow_cerenkov(map, nmap, beta[i], q[i]);
}
/* mass, charge and stock beta (mean of start and end energies) of particle codes with momenta p0, p1 */
void orc_particle_beta_v(const int64_t *code, int ncode, const double *mass, const double *charge, int64_t n,
                         const int64_t *pdg, const double *p0, const double *p1, double *m_out, double *q_out,
                         double *beta_out) {
    OrcLookupGroup G;
    memset(&G, 0, sizeof(G));
    G.pdg_code = code;
    G.pdg_mass = mass;
    G.pdg_charge = charge;
    G.npdg = ncode;
    for (int64_t i = 0; i < n; ++i) {
        double m, q;
        lrow_particle(&G, pdg[i], &m, &q);
        m_out[i] = m;
        q_out[i] = q;
        beta_out[i] = lrow_beta(m, p0[i], p1[i]);
    }
}

/* Bins of every substep of every row (row-major; -1: none): out[3 * s + table]. */
void orc_substep_bins(const OrcLookup *L, const OrcSubstepRows *R, int64_t nrows, int32_t *out) {
    int64_t o = 0;
    for (int64_t r = 0; r < nrows; ++r) {
        int64_t nsub = R->nsub[r];
        int bb = sub_find_bin(L->edges[3], L->nedges[3], R->beta[r]);
        int bth = R->theta ? sub_find_bin(L->edges[4], L->nedges[4], R->theta[r])
                           : sub_find_bin_cos(L->cos_theta_edges, L->nedges[4], R->cos_theta[r]);
        for (int64_t k = 0; k < nsub; ++k, ++o) {
            int bin[3];
            double t, z;
            sub_bins(L, R, r, k, nsub, bb, bth, bin, &t, &z);
            for (int tb = 0; tb < 3; ++tb) out[3 * o + tb] = bin[tb];
        }
    }
}

/* The delay / emission index search for given bins and thresholds (test hook): out[i] = first j of row bins[i] of
 * wts (n per row) whose running sum reaches thr[i]. */
void orc_first_reaching_v(const uint8_t *wts, int n, int64_t m, const int64_t *bins, const double *thr, int32_t *out) {
    for (int64_t i = 0; i < m; ++i) out[i] = sub_first_reaching(wts + bins[i] * (int64_t)n, n, thr[i]);
}
