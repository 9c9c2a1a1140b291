// Device building blocks of the CRV response engine: keyed Philox draws, the project's own FP64 exp/log/sin-cos(pi x)
// (the same steps and fused multiply-adds as the CPU oracle, so FP64 draws and SiPM recoveries agree bit for bit),
// status reporting and warp helpers.
//
// Philox4x32-10 follows Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11).
// Counter layout of a draw block: word 0 event, word 1 subrun, word 2 = stage << 28 | generation << 24 |
// node index << 18 | call << 15 | channel, word 3 = step-in-event << 16 | photon (or a stage id); key = (seed, run).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "crvgpu.h"

namespace crv {

constexpr int NPX = 1600;          // photon-map bins: 40 x 40, bin = x * 40 + y
// Pixel ids x * 41 + y over a 41 x 41 state (crv/crvfastsim/response/sipm.py:22 NPIX = 41): "lrint" rounds a
// photon-map point to pixel 40 at the far edge of bin 39
constexpr int PXS = 41;
constexpr int NPS = PXS * PXS;     // 1,681 pixel states
constexpr int NPS_ALLOC = 1688;    // NPS rounded up to 8 (keeps the following shared arrays 16-byte aligned)
constexpr int DEAD_WORDS = 53;     // dead-pixel bitmap words over the 1,681 ids
constexpr int MAX_GEN = 15;        // cross-talk generations per photon
constexpr int MAX_IDX = 63;        // nodes per generation
constexpr uint32_t ST_COUNT = 1, ST_PHOTON = 2, ST_SIPM = 3, ST_TDC0 = 4, ST_NOISE = 5, ST_STEPS = 6;

__host__ __device__ __forceinline__ uint32_t w2_of(uint32_t stage, uint32_t gen, uint32_t idx, uint32_t call,
                                                    uint32_t chan) {
  return (stage << 28) | (gen << 24) | (idx << 18) | (call << 15) | (chan & 0x7FFFu);
}

struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  return {c0, c1, c2, c3};
}

struct EvKey { uint32_t event, subrun, run; };

__device__ __forceinline__ U4 keyed(uint32_t seed, const EvKey& e, uint32_t w2, uint32_t w3) {
  return philox(e.event, e.subrun, w2, w3, seed, e.run);
}

__device__ __forceinline__ uint64_t bits53(uint32_t a, uint32_t b) { return ((uint64_t(a) << 32) | b) >> 11; }
__device__ __forceinline__ double u01(uint32_t a, uint32_t b) { return double(bits53(a, b)) * 0x1p-53; }
__device__ __forceinline__ double u01_open(uint32_t a, uint32_t b) { return double(bits53(a, b) + 1) * 0x1p-53; }
// 24-bit uniforms for the FP32-mixed path (top bits of the same words)
__device__ __forceinline__ float f01(uint32_t a) { return float(a >> 8) * 0x1p-24f; }
__device__ __forceinline__ float f01_open(uint32_t a) { return float((a >> 8) + 1) * 0x1p-24f; }

// ---------------------------------------------------------------------------------------------------------------------
// FP64 exp / log / sincospi: Cody-Waite reduction + degree-13 Taylor series; atanh series; Taylor series of
// sin/cos(pi b) on [0, 1/4].  Every multiply-add is an explicit __fma_rn; the translation unit is built without
// contraction, so the remaining operations round exactly as written.

__device__ __forceinline__ double pow2i(int n) { return __longlong_as_double((long long)(n + 1023) << 52); }

__device__ __forceinline__ double dexp(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return __longlong_as_double(0x7FF0000000000000ll);
  if (x < -745.2) return 0.0;
  const double LN2_HI = 0x1.62e42fefa39efp-1, LN2_LO = 0x1.abc9e3b39803fp-56, INV_LN2 = 0x1.71547652b82fep+0;
  double n = rint(x * INV_LN2);
  double r = __fma_rn(-n, LN2_HI, x);
  r = __fma_rn(-n, LN2_LO, r);
  double p = 1.6059043836821613e-10;
  p = __fma_rn(p, r, 2.08767569878681e-09);
  p = __fma_rn(p, r, 2.505210838544172e-08);
  p = __fma_rn(p, r, 2.755731922398589e-07);
  p = __fma_rn(p, r, 2.7557319223985893e-06);
  p = __fma_rn(p, r, 2.48015873015873e-05);
  p = __fma_rn(p, r, 0.0001984126984126984);
  p = __fma_rn(p, r, 0.001388888888888889);
  p = __fma_rn(p, r, 0.008333333333333333);
  p = __fma_rn(p, r, 0.041666666666666664);
  p = __fma_rn(p, r, 0.16666666666666666);
  p = __fma_rn(p, r, 0.5);
  p = __fma_rn(p, r, 1.0);
  p = __fma_rn(p, r, 1.0);
  int k = int(n);
  if (k > 1023) return (p * pow2i(1023)) * pow2i(k - 1023);
  if (k < -1020) return (p * pow2i(-60)) * pow2i(k + 60);
  return p * pow2i(k);
}

__device__ __forceinline__ double dlog(double x) {
  if (x != x || x < 0.0) return __longlong_as_double(0x7FF8000000000000ll);
  if (x == 0.0) return __longlong_as_double((long long)0xFFF0000000000000ull);
  if (x == __longlong_as_double(0x7FF0000000000000ll)) return x;
  int e = 0;
  if (x < 0x1p-1022) { x *= 0x1p54; e = -54; }
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  e += int((b >> 52) & 0x7FF) - 1023;
  b = (b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;
  double m = __longlong_as_double((long long)b);
  if (m > 1.4142135623730951) { m *= 0.5; e += 1; }
  double f = m - 1.0;
  double s = f / (2.0 + f);
  double w = s * s;
  double q = 0.043478260869565216;
  q = __fma_rn(q, w, 0.047619047619047616);
  q = __fma_rn(q, w, 0.05263157894736842);
  q = __fma_rn(q, w, 0.058823529411764705);
  q = __fma_rn(q, w, 0.06666666666666667);
  q = __fma_rn(q, w, 0.07692307692307693);
  q = __fma_rn(q, w, 0.09090909090909091);
  q = __fma_rn(q, w, 0.1111111111111111);
  q = __fma_rn(q, w, 0.14285714285714285);
  q = __fma_rn(q, w, 0.2);
  q = __fma_rn(q, w, 0.3333333333333333);
  double t = 2.0 * s;
  double lm = __fma_rn(t * w, q, t);
  double de = double(e);
  return __fma_rn(de, 0x1.62e42fefa39efp-1, __fma_rn(de, 0x1.abc9e3b39803fp-56, lm));
}

__device__ __forceinline__ double sinpi_q(double b) {
  double w = b * b;
  double p = 7.952054001475513e-07;
  p = __fma_rn(p, w, -2.1915353447830217e-05);
  p = __fma_rn(p, w, 0.00046630280576761255);
  p = __fma_rn(p, w, -0.0073704309457143504);
  p = __fma_rn(p, w, 0.08214588661112823);
  p = __fma_rn(p, w, -0.5992645293207921);
  p = __fma_rn(p, w, 2.5501640398773455);
  p = __fma_rn(p, w, -5.16771278004997);
  p = __fma_rn(p, w, 3.141592653589793);
  return p * b;
}

__device__ __forceinline__ double cospi_q(double b) {
  double w = b * b;
  double p = -1.3878952462213771e-07;
  p = __fma_rn(p, w, 4.303069587032947e-06);
  p = __fma_rn(p, w, -0.0001046381049248457);
  p = __fma_rn(p, w, 0.0019295743094039231);
  p = __fma_rn(p, w, -0.02580689139001406);
  p = __fma_rn(p, w, 0.2353306303588932);
  p = __fma_rn(p, w, -1.3352627688545895);
  p = __fma_rn(p, w, 4.0587121264167685);
  p = __fma_rn(p, w, -4.934802200544679);
  p = __fma_rn(p, w, 1.0);
  return p;
}

__device__ __forceinline__ void dsincospi(double x, double* sp, double* cp) {
  double y = x - 2.0 * rint(0.5 * x);
  double sg = 1.0;
  if (y < 0.0) { y = -y; sg = -1.0; }
  double s, c;
  if (y <= 0.25) { s = sinpi_q(y); c = cospi_q(y); }
  else if (y <= 0.75) { double b = 0.5 - y; s = cospi_q(b); c = sinpi_q(b); }
  else { double b = 1.0 - y; s = sinpi_q(b); c = -cospi_q(b); }
  *sp = sg * s;
  *cp = c;
}

// ---------------------------------------------------------------------------------------------------------------------
// Precision policy: the FP64 path uses the project's functions above (bit-exact with the oracle); the FP32-mixed path
// uses 24-bit uniforms and hardware float transcendentals.

// FP32 <-> FP64 moves by integer bit arithmetic.  On this GPU a conversion instruction issues on the FP64 pipe, as
// slowly as an FP64 multiply; these forms run on the integer pipe and fall back to the instruction only outside the
// normal range.  f2d is exact; d2f_trunc truncates the mantissa (at most one FP32 ulp below round-to-nearest).
__device__ __forceinline__ double f2d(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  if ((u & 0x7FFFFFFFu) == 0u) return __longlong_as_double((long long)((unsigned long long)u << 32));
  if (e == 0u || e == 0xFFu) return (double)f;
  const unsigned long long d = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)d);
}

__device__ __forceinline__ float d2f_trunc(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = int((b >> 52) & 0x7FFu);
  if (E < 897 || E > 1150) return (float)x;
  const uint32_t u = uint32_t((b >> 32) & 0x80000000ull) | (uint32_t(E - 896) << 23) | uint32_t((b >> 29) & 0x7FFFFFull);
  return __uint_as_float(u);
}

// finite and non-zero, tested on the bits
__device__ __forceinline__ bool finite_nonzero(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b & 0x7FFFFFFFFFFFFFFFull) != 0ull && ((b >> 52) & 0x7FFull) != 0x7FFull;
}

template <typename R> struct Math;

template <> struct Math<double> {
  static __device__ __forceinline__ double exp(double x) { return dexp(x); }
  static __device__ __forceinline__ double log(double x) { return dlog(x); }
  static __device__ __forceinline__ double uni(const U4& w, int h) { return h ? u01(w.z, w.w) : u01(w.x, w.y); }
  static __device__ __forceinline__ double uni_open(const U4& w, int h) {
    return h ? u01_open(w.z, w.w) : u01_open(w.x, w.y);
  }
  static __device__ __forceinline__ void normal_pair(const U4& w, double* z0, double* z1) {
    double u1 = u01_open(w.x, w.y), u2 = u01(w.z, w.w);
    double r = sqrt(-2.0 * dlog(u1));
    double s, c;
    dsincospi(2.0 * u2, &s, &c);
    *z0 = r * c;
    *z1 = r * s;
  }
};

template <> struct Math<float> {
  static __device__ __forceinline__ float exp(float x) { return __expf(x); }
  static __device__ __forceinline__ float log(float x) { return __logf(x); }
  static __device__ __forceinline__ float uni(const U4& w, int h) { return h ? f01(w.z) : f01(w.x); }
  static __device__ __forceinline__ float uni_open(const U4& w, int h) { return h ? f01_open(w.z) : f01_open(w.x); }
  static __device__ __forceinline__ void normal_pair(const U4& w, float* z0, float* z1) {
    float u1 = f01_open(w.x), u2 = f01(w.z);
    float r = sqrtf(-2.0f * __logf(u1));
    float s, c;
    __sincosf(6.283185307179586f * u2, &s, &c);
    *z0 = r * c;
    *z1 = r * s;
  }
};

// ---------------------------------------------------------------------------------------------------------------------
// status word (device): bit flags OR-ed by any thread; "need" slots hold the largest capacity any item required.

struct Status {
  int32_t flags;
  int32_t pad;
  long long need[16];  // see CRV_NEED_* in crvgpu.h
};

__device__ __forceinline__ void set_flag(Status* s, int32_t f) { atomicOr(&s->flags, f); }
__device__ __forceinline__ void need_at_least(Status* s, int slot, long long v) {
  atomicMax(reinterpret_cast<unsigned long long*>(&s->need[slot]), (unsigned long long)v);
}

// Item count of an array sized by an upper bound: the host bound n, or the device count *n_dev when that is smaller
// (n_dev null: n itself).  Entry points that run inside a captured graph take their counts this way.
__device__ __forceinline__ long long bounded_count(long long n, const long long* n_dev) {
  if (!n_dev) return n;
  long long m = *n_dev;
  return m < n ? m : n;
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ int warp_in_block() { return threadIdx.x >> 5; }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// exclusive prefix over the warp (int)
__device__ __forceinline__ int warp_excl(int v, int* total) {
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane_id() >= o) x += y;
  }
  *total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

__device__ __forceinline__ long long warp_excl_ll(long long v, long long* total) {
  long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane_id() >= o) x += y;
  }
  *total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

}  // namespace crv
