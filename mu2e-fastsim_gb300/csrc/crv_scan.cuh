// Device-wide exclusive prefix sums (int64 out) over int32/int64 inputs, in three launches:
// per-block reduction, a single-block scan of the block sums, per-block scan with the block offset.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "crv_launch.h"

namespace crv {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 8;                        // items per thread
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// effective length: the host bound n, or the device count *n_dev when it is smaller (arrays sized by an upper bound)
__device__ __forceinline__ long long scan_len(long long n, const long long* n_dev) { return bounded_count(n, n_dev); }

template <typename T, typename F>
__global__ void k_scan_reduce(const T* __restrict__ in, long long n, const long long* __restrict__ n_dev, F f,
                              long long* __restrict__ part) {
  __shared__ long long red[SCAN_THREADS / 32];
  n = scan_len(n, n_dev);
  long long base = (long long)blockIdx.x * SCAN_TILE;
  long long s = 0;
  if (base < n) {
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
      long long i = base + (long long)j * SCAN_THREADS + threadIdx.x;
      if (i < n) s += f(in[i]);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    long long v = threadIdx.x < SCAN_THREADS / 32 ? red[threadIdx.x] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}

// exclusive scan of part[0..nb) in place by one block; total -> *total (device)
__global__ void k_scan_parts(long long* __restrict__ part, long long nb, long long* __restrict__ total);

// Tile of SCAN_TILE items: coalesced loads into shared memory, each thread scans SCAN_ITEMS consecutive items there,
// coalesced stores of the results.
template <typename T, typename F>
__global__ void k_scan_down(const T* __restrict__ in, long long n, const long long* __restrict__ n_dev, F f,
                            const long long* __restrict__ part, long long* __restrict__ out) {
  __shared__ long long tile[SCAN_TILE];
  __shared__ long long wsum[SCAN_THREADS / 32];
  n = scan_len(n, n_dev);
  long long base = (long long)blockIdx.x * SCAN_TILE;
  if (base >= n) return;                                      // the whole block: uniform
  long long off = part[blockIdx.x];
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    int k = j * SCAN_THREADS + threadIdx.x;
    long long i = base + k;
    tile[k] = i < n ? f(in[i]) : 0;
  }
  __syncthreads();
  long long v[SCAN_ITEMS];
  long long s = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    v[j] = tile[threadIdx.x * SCAN_ITEMS + j];
    s += v[j];
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    long long q = lane < SCAN_THREADS / 32 ? wsum[lane] : 0;
    long long qq = q;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(0xffffffffu, qq, o);
      if (lane >= o) qq += y;
    }
    if (lane < SCAN_THREADS / 32) wsum[lane] = qq - q;
  }
  __syncthreads();
  long long run = off + wsum[w] + (x - s);
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    tile[threadIdx.x * SCAN_ITEMS + j] = run;
    run += v[j];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    int k = j * SCAN_THREADS + threadIdx.x;
    long long i = base + k;
    if (i < n) out[i] = tile[k];
  }
}

struct Identity {
  template <typename T>
  __device__ __forceinline__ long long operator()(T v) const { return (long long)v; }
};

inline long long scan_parts_len(long long n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

// out[i] = sum_{j<i} f(in[j]); *total = sum f(in).  part: scratch of scan_parts_len(n) + 1 entries.  n_dev (may be
// null): device count of valid items when n is only an upper bound; items beyond it are neither read nor written.
template <typename T, typename F>
cudaError_t exclusive_scan(const T* in, long long n, F f, long long* out, long long* total, long long* part,
                           cudaStream_t s, const long long* n_dev = nullptr) {
  long long nb = scan_parts_len(n);
  if (nb == 0) {
    cudaMemsetAsync(total, 0, sizeof(long long), s);
    return cudaGetLastError();
  }
  {
    crv::Mark mark_("k_scan_reduce", s);
    k_scan_reduce<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, n_dev, f, part);
  }
  {
    crv::Mark mark_("k_scan_parts", s);
    k_scan_parts<<<1, 1024, 0, s>>>(part, nb, total);
  }
  {
    crv::Mark mark_("k_scan_down", s);
    k_scan_down<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, n_dev, f, part, out);
  }
  return cudaGetLastError();
}

}  // namespace crv
