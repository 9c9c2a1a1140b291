// Host-side reader of the Mu2e CRV photon lookup tables, format version 6: the layout Offline's CRVResponse
// (MakeCrvPhotons) writes and crv/crvfastsim/response/lookup.py:149-179 (load, _read_bins) reads.  Two calls over a
// file image in host memory: crv_lookup_file_info validates the whole image and reports every size,
// crv_lookup_file_read fills caller-allocated arrays.  Each is one linear pass over the bins (the reference walks
// them with a Python loop, then gathers the variable-length weight vectors with NumPy).
//
// Layout (little-endian, as the C++ structs are written):
//   int32 version major, minor, reflector; 4 bytes padding; float64 constants[10]
//   two Cerenkov maps (scintillator, fibre): uint64 n, then n (beta, photons per mm) float64 pairs
//   seven bin-edge vectors (x, y, z, beta, theta, phi, r): uint64 n, then n float64
//   the bins of the scint [x,y,z], ckscint [x,y,z,beta] and ckfiber [beta,theta,phi,r,z] tables, each bin:
//   uint32 bin number (= its position), float32 arrival probability, uint64 n + n uint8 delay weights,
//   uint64 n + n uint8 emission weights
#include <cstdint>
#include <cstring>

#include "crvgpu.h"

namespace {

// Bounds-checked little-endian cursor over the image (both supported hosts are little-endian).
struct Cursor {
  const uint8_t* p;
  int64_t n;
  int64_t o;
  bool ok;

  bool has(uint64_t k) const { return ok && o <= n && k <= uint64_t(n - o); }
  template <typename T>
  T get() {
    T v;
    std::memset(&v, 0, sizeof(T));
    if (!has(sizeof(T))) { ok = false; return v; }
    std::memcpy(&v, p + o, sizeof(T));
    o += int64_t(sizeof(T));
    return v;
  }
  const uint8_t* take(uint64_t k) {
    if (!has(k)) { ok = false; return nullptr; }
    const uint8_t* q = p + o;
    o += int64_t(k);
    return q;
  }
};

void fail(CrvLookupFileInfo* info, int code, int64_t a, int64_t b) {
  info->error = code;
  info->error_a = a;
  info->error_b = b;
}

// a * b, or -1 when it exceeds lim (bin counts are bounded by the image size)
int64_t mul_bounded(int64_t a, int64_t b, int64_t lim) {
  if (a == 0 || b == 0) return 0;
  if (a > lim / b) return -1;
  return a * b;
}

constexpr int64_t BIN_MIN_BYTES = 24;   // bin number, probability, two vector lengths

// Table sizes from the edge counts: scint = x y z, ckscint = scint * beta, ckfiber = beta theta phi r z.
bool bin_counts(const int64_t* ne, int64_t lim, int64_t* nb) {
  int64_t b[7];
  for (int e = 0; e < 7; ++e) b[e] = ne[e] - 1;
  int64_t s = mul_bounded(mul_bounded(b[0], b[1], lim), b[2], lim);
  if (s < 0) return false;
  int64_t ck = mul_bounded(s, b[3], lim);
  static const int fibre_axes[4] = {4, 5, 6, 2};   // theta, phi, r, z after beta
  int64_t f = b[3];
  for (int a = 0; a < 4; ++a) {
    f = mul_bounded(f, b[fibre_axes[a]], lim);
    if (f < 0) return false;
  }
  if (ck < 0) return false;
  nb[0] = s;
  nb[1] = ck;
  nb[2] = f;
  return true;
}

// Header, constants, Cerenkov maps and edges; returns false (info->error set) on a malformed image.
bool read_head(Cursor& c, CrvLookupFileInfo* info, const uint8_t** ck, const uint8_t** edges) {
  info->version_major = c.get<int32_t>();
  info->version_minor = c.get<int32_t>();
  info->reflector = c.get<int32_t>();
  c.take(4);
  for (int i = 0; i < 10; ++i) info->constants[i] = c.get<double>();
  if (!c.ok) { fail(info, CRV_LUTF_TRUNCATED, c.o, -1); return false; }
  if (info->version_major != 6) {
    fail(info, CRV_LUTF_VERSION, info->version_major, info->version_minor);
    return false;
  }
  for (int m = 0; m < 2; ++m) {
    uint64_t k = c.get<uint64_t>();
    if (!c.ok || k > uint64_t(c.n - c.o) / 16) { fail(info, CRV_LUTF_TRUNCATED, c.o, -1); return false; }
    info->n_ck[m] = int64_t(k);
    ck[m] = c.take(16 * k);
  }
  for (int e = 0; e < 7; ++e) {
    uint64_t k = c.get<uint64_t>();
    if (!c.ok || k > uint64_t(c.n - c.o) / 8) { fail(info, CRV_LUTF_TRUNCATED, c.o, -1); return false; }
    info->n_edges[e] = int64_t(k);
    edges[e] = c.take(8 * k);
  }
  for (int e = 0; e < 7; ++e)
    if (info->n_edges[e] < 1) { fail(info, CRV_LUTF_SIZE, e, info->n_edges[e]); return false; }
  if (!bin_counts(info->n_edges, c.n / BIN_MIN_BYTES + 1, info->n_bins)) {
    fail(info, CRV_LUTF_SIZE, -1, -1);
    return false;
  }
  return true;
}

}  // namespace

extern "C" int crv_lookup_file_info(const uint8_t* image, int64_t size, CrvLookupFileInfo* info) {
  if (info == nullptr || size < 0 || (image == nullptr && size > 0)) return CRV_ERR_ARG;
  std::memset(info, 0, sizeof(*info));
  Cursor c{image, size, 0, true};
  const uint8_t* ck[2];
  const uint8_t* edges[7];
  if (!read_head(c, info, ck, edges)) return CRV_ERR_ARG;
  for (int t = 0; t < 3; ++t) {
    uint64_t dw = 1, ew = 1;
    for (int64_t i = 0; i < info->n_bins[t]; ++i) {
      const int64_t at = c.o;
      uint32_t num = c.get<uint32_t>();
      c.get<float>();
      if (!c.ok) { fail(info, CRV_LUTF_TRUNCATED, at, t); return CRV_ERR_ARG; }
      if (int64_t(num) != i) { fail(info, CRV_LUTF_BIN_NUMBER, num, i); return CRV_ERR_ARG; }
      uint64_t nd = c.get<uint64_t>();
      c.take(nd);
      uint64_t ne = c.get<uint64_t>();
      c.take(ne);
      if (!c.ok) { fail(info, CRV_LUTF_TRUNCATED, at, t); return CRV_ERR_ARG; }
      if (nd > dw) dw = nd;
      if (ne > ew) ew = ne;
    }
    info->delay_width[t] = int64_t(dw);
    info->emis_width[t] = int64_t(ew);
  }
  if (c.o != size) { fail(info, CRV_LUTF_TRAILING, size - c.o, c.o); return CRV_ERR_ARG; }
  return CRV_OK;
}

extern "C" int crv_lookup_file_read(const uint8_t* image, int64_t size, const CrvLookupFileInfo* info,
                                    const CrvLookupFileOut* out) {
  if (info == nullptr || out == nullptr || info->error != 0 || size < 0 || (image == nullptr && size > 0))
    return CRV_ERR_ARG;
  CrvLookupFileInfo chk;
  std::memset(&chk, 0, sizeof(chk));
  Cursor c{image, size, 0, true};
  const uint8_t* ck[2];
  const uint8_t* edges[7];
  if (!read_head(c, &chk, ck, edges)) return CRV_ERR_ARG;
  for (int m = 0; m < 2; ++m) {
    if (chk.n_ck[m] != info->n_ck[m]) return CRV_ERR_ARG;
    if (chk.n_ck[m] > 0) {
      if (out->ck[m] == nullptr) return CRV_ERR_ARG;
      std::memcpy(out->ck[m], ck[m], size_t(16 * chk.n_ck[m]));
    }
  }
  for (int e = 0; e < 7; ++e) {
    if (chk.n_edges[e] != info->n_edges[e] || out->edges[e] == nullptr) return CRV_ERR_ARG;
    std::memcpy(out->edges[e], edges[e], size_t(8 * chk.n_edges[e]));
  }
  for (int t = 0; t < 3; ++t) {
    const int64_t nb = chk.n_bins[t];
    if (nb != info->n_bins[t]) return CRV_ERR_ARG;
    const CrvLookupFileTable& T = out->tables[t];
    const int64_t dw = info->delay_width[t], ew = info->emis_width[t];
    if (nb > 0 && (T.prob == nullptr || T.delays == nullptr || T.delay_sum == nullptr || T.emis == nullptr ||
                   T.emis_sum == nullptr || dw < 1 || ew < 1))
      return CRV_ERR_ARG;
    for (int64_t i = 0; i < nb; ++i) {
      uint32_t num = c.get<uint32_t>();
      float prob = c.get<float>();
      if (!c.ok || int64_t(num) != i) return CRV_ERR_ARG;
      T.prob[i] = prob;
      for (int v = 0; v < 2; ++v) {
        const int64_t w = v ? ew : dw;
        uint8_t* row = (v ? T.emis : T.delays) + i * w;
        uint64_t k = c.get<uint64_t>();
        const uint8_t* src = c.take(k);
        if (!c.ok || k > uint64_t(w)) return CRV_ERR_ARG;
        uint32_t sum = 0;                  // int32 sum with wrap-around, as NumPy's sum(dtype=int32)
        for (uint64_t j = 0; j < k; ++j) sum += src[j];
        std::memcpy(row, src, size_t(k));
        std::memset(row + k, 0, size_t(w - int64_t(k)));
        (v ? T.emis_sum : T.delay_sum)[i] = int32_t(sum);
      }
    }
  }
  return c.o == size ? CRV_OK : CRV_ERR_ARG;
}
