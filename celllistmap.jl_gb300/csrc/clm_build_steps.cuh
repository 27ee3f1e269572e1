// Per-particle and per-copy steps of the cell-list build (wrap and images, keys, in-cell rank, gather) and the
// device copy of the box geometry.  The build kernels (clm_build.cu) call them on the device; the CPU tests
// compile the same functions for the host (g++ with -ffp-contract=off) and compare the copies, cells and
// coordinates they give with the oracle's serial cell list, without a GPU.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>

#include "clm_device.cuh"
#include "clm_geometry.hpp"

namespace clm {

// The few operations that differ between the device and the host build of the steps below.
__host__ __device__ __forceinline__ void flag_error(int* err, int bits) {
#ifdef __CUDA_ARCH__
  atomicOr(err, bits);
#else
  *err |= bits;
#endif
}
__host__ __device__ __forceinline__ int lowest_bit(uint32_t m) {  // index of the lowest set bit, m != 0
#ifdef __CUDA_ARCH__
  return __ffs(m) - 1;
#else
  return __builtin_ctz(m);
#endif
}
__host__ __device__ __forceinline__ float bits_as_float(int v) {
#ifdef __CUDA_ARCH__
  return __int_as_float(v);
#else
  float f;
  std::memcpy(&f, &v, sizeof f);
  return f;
#endif
}
// NaN test on the bit pattern (a magnitude above that of inf), on the integer pipe
__host__ __device__ __forceinline__ bool is_nan(double v) {
  return (unsigned long long)(dbits(v) & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000ULL;
}
__host__ __device__ __forceinline__ bool is_nan(float v) {
#ifdef __CUDA_ARCH__
  const unsigned b = __float_as_uint(v);
#else
  unsigned b;
  std::memcpy(&b, &v, sizeof b);
#endif
  return (b & 0x7FFFFFFFu) > 0x7F800000u;
}

// The value with order key q (order_key is its own inverse on the bit pattern).
template <class T> T from_order_key(typename OrderKey<T>::type q) {
  const auto b = q ^ (decltype(q))((typename std::make_unsigned<decltype(q)>::type)(q >> (8 * sizeof(q) - 1)) >> 1);
  T v;
  std::memcpy(&v, &b, sizeof v);
  return v;
}

// The smallest order key q with RN(value(q) + s) >= b.  RN(p + s) does not decrease as p grows, so the p that
// pass the test `b <= p + s` are those with key(p) >= q.  Bisection over [key(-inf), key(+inf)] (+inf passes
// for finite s and b), bracketed first within 4 keys of RN(b - s), where q almost always lies.
template <class T> typename OrderKey<T>::type first_key_at_least(T s, T b) {
  using K = typename OrderKey<T>::type;
  const auto pass = [&](K q) { return from_order_key<T>(q) + s >= b; };
  K lo = order_key(-std::numeric_limits<T>::infinity()), hi = order_key(std::numeric_limits<T>::infinity());
  const K q = std::min(std::max(order_key((T)(b - s)), lo), hi);
  const K a = q - 4 > lo ? q - 4 : lo, z = q + 4 < hi ? q + 4 : hi;
  if (!pass(a)) lo = a;
  if (pass(z)) hi = z;
  while (lo + 1 < hi) {
    const K mid = (lo >> 1) + (hi >> 1) + (lo & hi & 1);
    if (pass(mid)) hi = mid;
    else lo = mid;
  }
  return pass(lo) ? lo : hi;
}

template <class T> void fill_devgeom(const Geometry<T>& g, int precision, DevGeom<T>& d) {
  std::memset(&d, 0, sizeof(d));
  (void)precision;
  d.dim = g.dim;
  d.kind = g.kind;
  d.lcell = g.lcell;
  d.ncells = (int)g.ncells();
  for (int i = 0; i < 3; i++) {
    d.nc[i] = (int)g.nc[i];
    d.cbmin[i] = g.cbmin[i];
    d.cbmax[i] = g.cbmax[i];
    d.cs[i] = g.cs[i];
    d.inv_cs[i] = T(1) / g.cs[i];
    d.csf[i] = (float)g.cs[i];
    d.csf_lo[i] = (float)((double)g.cs[i] - (double)d.csf[i]);
    d.cbf_hi[i] = (float)g.cbmin[i];
    d.cbf_lo[i] = (float)((double)g.cbmin[i] - (double)d.cbf_hi[i]);
    for (int j = 0; j < 3; j++) {
      d.Min[i][j] = g.Min[i][j];
      d.R[i][j] = g.R[i][j];
      d.Rinv[i][j] = g.Rinv[i][j];
    }
  }
  d.det_in = g.det_in;
  d.inv_det = T(1) / g.det_in;
  {
    // the cofactors of the 3D solve, separately rounded in the handle dtype (wrap_point)
    const auto& a = g.Min;
    const auto c = [](T p, T q, T r, T s) { return xsub(xmul(p, q), xmul(r, s)); };
    const T cof[3][3] = {{c(a[1][1], a[2][2], a[1][2], a[2][1]), c(a[0][2], a[2][1], a[0][1], a[2][2]),
                          c(a[0][1], a[1][2], a[0][2], a[1][1])},
                         {c(a[1][2], a[2][0], a[1][0], a[2][2]), c(a[0][0], a[2][2], a[0][2], a[2][0]),
                          c(a[0][2], a[1][0], a[0][0], a[1][2])},
                         {c(a[1][0], a[2][1], a[1][1], a[2][0]), c(a[0][1], a[2][0], a[0][0], a[2][1]),
                          c(a[0][0], a[1][1], a[0][1], a[1][0])}};
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) d.cof[i][j] = cof[i][j];
  }
  d.shape = kShapeGeneral;
  if (g.dim == 3 && g.kind != NONPERIODIC) {
    bool lower = true, upper = true, rid = true;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        if (i > j && (g.Min[i][j] != T(0) || d.cof[i][j] != T(0))) lower = false;
        if (i < j && (g.Min[i][j] != T(0) || d.cof[i][j] != T(0))) upper = false;
        if (g.R[i][j] != (i == j ? T(1) : T(0))) rid = false;
      }
    if (lower) d.shape = (upper && rid) ? kShapeDiag : kShapeUpper;
  }
  d.cutoff = g.cutoff;
  d.cutoff_sqr = g.cutoff_sqr;
  d.margin_wide = (double)g.cutoff * (1.0 + std::sqrt((double)g.dim) / 2.0);
  d.nimg = (g.dim == 3) ? 27 : 9;
  // With exact zeros below the diagonal, component i of an image shift depends only on s_i..s_dim-1, so
  // the image tests can run dimension by dimension from the last one (img_tree 2); with exact zeros in the
  // last row only, the last component depends only on s_dim-1 and is tested once per value of it (1).
  // Same values as testing every image, fewer tests.
  bool upper = true, last_row = true;
  for (int i = 0; i < g.dim; i++)
    for (int j = 0; j < i; j++)
      if (g.Mal[i][j] != T(0)) {
        upper = false;
        if (i == g.dim - 1) last_row = false;
      }
  d.img_tree = upper ? 2 : (last_row ? 1 : 0);
  d.zero_code = (g.dim == 3) ? 13 : 4;
  // translation_image: x + Mal * s, s in {-1,0,1}^N with the first index fastest
  for (int k = 0; k < d.nimg; k++) {
    int s[3], kk = k;
    for (int i = 0; i < g.dim; i++) {
      s[i] = kk % 3 - 1;
      kk /= 3;
    }
    for (int i = 0; i < g.dim; i++) {
      T acc = g.Mal[i][0] * T(s[0]);
      for (int j = 1; j < g.dim; j++) acc = acc + g.Mal[i][j] * T(s[j]);
      d.shift[k][i] = acc;
      d.img_lo[k][i] = first_key_at_least<T>(acc, g.cbmin[i]);
      d.img_hi[k][i] = first_key_at_least<T>(acc, g.cbmax[i]);
    }
  }
  // FP32 prefilter band around cutoff^2 (relative 2^-13, far above the FP32
  // error of d2 computed from cell-relative offsets, ~2^-18 relative).
  double c2 = (double)g.cutoff_sqr;
  d.thr_hi = std::nextafter((float)(c2 * (1.0 + std::ldexp(1.0, -13))), INFINITY);
  d.thr_lo = std::nextafter((float)(c2 * (1.0 - std::ldexp(1.0, -13))), 0.0f);
}

// ------------------------------------------------------------------ wrap, images, copy count
// Particle i: its wrapped position p, the mask of its images inside the computing box and its number of
// copies.  Returns false if the particle has a NaN coordinate (it then gets no copy: p = 0, m = 0, cnt = 0).
template <class T, int N, int SH = kShapeGeneral>
__host__ __device__ __forceinline__ bool wrap_count_regs(const DevGeom<T>& g, const T* __restrict__ x, int i, T* p,
                                                         uint32_t& mask_out, int& cnt_out) {
  T xi[N];
  bool bad = false;
#pragma unroll
  for (int k = 0; k < N; k++) {
    xi[k] = x[(int64_t)i * N + k];
    bad = bad || is_nan(xi[k]);
  }
  if (bad) {
#pragma unroll
    for (int k = 0; k < N; k++) p[k] = T(0);
    mask_out = 0;
    cnt_out = 0;
    return false;
  }
  if (g.kind == NONPERIODIC) {
#pragma unroll
    for (int k = 0; k < N; k++) p[k] = xi[k];
  } else {
    wrap_point<T, N, SH>(g, xi, p);
  }
  uint32_t m = 0;
  int cnt = 1;
  // image tests on the order keys of p (image_in): the same decisions as cbmin <= p + shift < cbmax
  typename OrderKey<T>::type pk[N];
#pragma unroll
  for (int k = 0; k < N; k++) pk[k] = order_key(p[k]);
  if (g.kind != NONPERIODIC && g.img_tree == 2) {
    // image k = (s0+1) + 3(s1+1) [+ 9(s2+1)]: the last component is tested once per s_last, the next
    // once per (s_mid, s_last), the first per image; each test uses the shift of the image itself
    // (equal, for the components tested early, across the images that share their s values)
#pragma unroll
    for (int sl = -1; sl <= 1; sl++) {
      const int kl = (N == 3) ? 9 * (sl + 1) + 4 : 3 * (sl + 1) + 1;
      if (!image_in(g, kl, N - 1, pk[N - 1])) continue;
      if (N == 3) {
#pragma unroll
        for (int sm = -1; sm <= 1; sm++) {
          const int km = 9 * (sl + 1) + 3 * (sm + 1) + 1;
          if (!image_in(g, km, 1, pk[1])) continue;
#pragma unroll
          for (int s0 = -1; s0 <= 1; s0++) {
            const int k = 9 * (sl + 1) + 3 * (sm + 1) + (s0 + 1);
            if (k == g.zero_code) continue;
            if (image_in(g, k, 0, pk[0])) {
              m |= 1u << k;
              cnt++;
            }
          }
        }
      } else {
#pragma unroll
        for (int s0 = -1; s0 <= 1; s0++) {
          const int k = 3 * (sl + 1) + (s0 + 1);
          if (k == g.zero_code) continue;
          if (image_in(g, k, 0, pk[0])) {
            m |= 1u << k;
            cnt++;
          }
        }
      }
    }
  } else if (g.kind != NONPERIODIC && g.img_tree == 1) {
    // the last component once per s_last (equal across the images that share it), then the other
    // components of each of those images
#pragma unroll
    for (int sl = -1; sl <= 1; sl++) {
      constexpr int NR = (N == 3) ? 9 : 3;  // images per value of s_last
      if (!image_in(g, NR * (sl + 1), N - 1, pk[N - 1])) continue;
#pragma unroll
      for (int r = 0; r < NR; r++) {
        const int k = NR * (sl + 1) + r;
        if (k == g.zero_code) continue;
        bool in = true;
#pragma unroll
        for (int d = 0; d < N - 1; d++) in = in && image_in(g, k, d, pk[d]);
        if (in) {
          m |= 1u << k;
          cnt++;
        }
      }
    }
  } else if (g.kind != NONPERIODIC) {
    for (int k = 0; k < g.nimg; k++) {
      if (k == g.zero_code) continue;
      bool in = true;
#pragma unroll
      for (int d = 0; d < N; d++) in = in && image_in(g, k, d, pk[d]);
      if (in) {
        m |= 1u << k;
        cnt++;
      }
    }
  }
  mask_out = m;
  cnt_out = cnt;
  return true;
}

// The same into the arrays of the build (wrapped positions, image masks, copy counts).
template <class T, int N>
__host__ __device__ __forceinline__ bool wrap_count_at(const DevGeom<T>& g, const T* __restrict__ x, int i,
                                              T* __restrict__ wrapped, uint32_t* __restrict__ mask,
                                              int* __restrict__ ncopy) {
  T p[N];
  uint32_t m = 0;
  int cnt = 0;
  const bool ok = wrap_count_regs<T, N>(g, x, i, p, m, cnt);
#pragma unroll
  for (int k = 0; k < N; k++) wrapped[(int64_t)i * N + k] = p[k];
  mask[i] = m;
  ncopy[i] = cnt;
  return ok;
}

// ------------------------------------------------------------------ keys of every copy
// The cell of image k of a particle at wrapped position p (k = zero_code: the real copy, with the border-case
// shift); an out-of-range cell is flagged and mapped to cell 0.
template <class T, int N>
__host__ __device__ __forceinline__ int copy_cell(const DevGeom<T>& g, const T* p, int k, int* __restrict__ err) {
  int li;
  if (k == g.zero_code) {
    li = cell_of<T, N>(g, p, true);
  } else {
    T q[N];
#pragma unroll
    for (int d = 0; d < N; d++) q[d] = xadd(p[d], g.shift[k][d]);
    li = cell_of<T, N>(g, q, false);
  }
  if (li < 0) {
    flag_error(err, DERR_CELL_RANGE);
    li = 0;
  }
  return li;
}

// The copies of particle i (wrapped position p, image mask m, ncp copies) at copy positions base .. base+ncp-1:
// the key is the copy's cell (the real copy first, with the border-case shift, then the images in
// increasing image code), the value (i << 5) | image code.  `cb` is the first global cell of the particle's
// system (0 for one system).
template <class T, int N>
__host__ __device__ __forceinline__ void emit_copies(const DevGeom<T>& g, int cb, const T* p, uint32_t m, int ncp,
                                                     int i, int base, int cap, uint32_t* __restrict__ keys,
                                                     uint32_t* __restrict__ vals, int* __restrict__ err) {
  if (ncp == 0) return;
  if (base < 0 || base + ncp > cap) {
    flag_error(err, DERR_COPY_OVERFLOW);
    return;
  }
  keys[base] = (uint32_t)(copy_cell<T, N>(g, p, g.zero_code, err) + cb);
  vals[base] = ((uint32_t)i << 5) | (uint32_t)g.zero_code;
  int t = 1;
  while (m) {
    int k = lowest_bit(m);
    m &= m - 1;
    keys[base + t] = (uint32_t)(copy_cell<T, N>(g, p, k, err) + cb);
    vals[base + t] = ((uint32_t)i << 5) | (uint32_t)k;
    t++;
  }
}

// The same from the arrays the wrap step wrote and the scanned copy offsets.
template <class T, int N>
__host__ __device__ __forceinline__ void emit_at(const DevGeom<T>& g, int cb, const T* __restrict__ wrapped,
                                        const uint32_t* __restrict__ mask, const int* __restrict__ ncopy,
                                        const int* __restrict__ copy_off, int i, int cap, uint32_t* __restrict__ keys,
                                        uint32_t* __restrict__ vals, int* __restrict__ err) {
  if (ncopy[i] == 0) return;
  T p[N];
#pragma unroll
  for (int k = 0; k < N; k++) p[k] = wrapped[(int64_t)i * N + k];
  emit_copies<T, N>(g, cb, p, mask[i], ncopy[i], i, copy_off[i], cap, keys, vals, err);
}

// ------------------------------------------------------------------ gather in cell order
// origin of cell c along one axis as an unevaluated float pair (hi + lo): cbmin + cs*(c-1) with the
// product and the sum carried exactly (TwoProduct with an FMA, TwoSum)
__host__ __device__ __forceinline__ void origin_ff(float cb_hi, float cb_lo, float cs_hi, float cs_lo, int c1, float& hi,
                                          float& lo) {
  const float k = (float)c1;
  const float p = cs_hi * k;
  const float pe = fmaf(cs_hi, k, -p) + cs_lo * k;
  const float s = cb_hi + p;
  const float bb = s - cb_hi;
  const float se = (cb_hi - (s - bb)) + (p - bb);
  hi = s;
  lo = se + pe + cb_lo;
}

// The float pair of a double: hi = (float)q and lo = (float)(q - (double)hi), both rounded to nearest even.
// float_pair takes them from q's bit pattern with integer operations when 2^-74 <= |q| < 2^126 (q and both
// parts normal): hi keeps the top 23 of q's 52 fraction bits, rounded by the 29 dropped ones (a carry runs
// into the exponent), and the difference q - hi is exactly the dropped bits' signed remainder r (|r| <= 2^28)
// times 2^(E - 52), E the exponent of q; converting r to float rounds it as converting the exact double
// difference does, and the power-of-two scale is exact.  Other values take the conversions (a call on the
// device, so that they stay off the common path).  Off the FP64 pipe: the gather's FP32 offsets need three
// components per copy.
#ifdef __CUDA_ARCH__
static __device__ __noinline__
#else
inline
#endif
float2 float_pair_call(double q) {
  const float hi = (float)q;
  return make_float2(hi, (float)(q - (double)hi));
}
__host__ __device__ __forceinline__ void float_pair(double q, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)dbits(q);
  const int e = (int)((b >> 52) & 0x7ff);  // biased exponent
  if (e < 1023 - 74 || e > 1023 + 125) {
    const float2 r = float_pair_call(q);
    hi = r.x;
    lo = r.y;
    return;
  }
  const unsigned rem = (unsigned)(b & 0x1FFFFFFFull);                  // the 29 dropped fraction bits
  const unsigned top = (unsigned)((b >> 29) & 0x7FFFFFull);            // the 23 kept ones
  const bool up = rem > 0x10000000u || (rem == 0x10000000u && (top & 1u));
  const bool neg = (b >> 63) != 0;
  const unsigned hb = ((neg ? 1u : 0u) << 31) | ((((unsigned)(e - (1023 - 127)) << 23) | top) + (up ? 1u : 0u));
  int r = (int)rem - (up ? 0x20000000 : 0);
  if (neg) r = -r;
  const unsigned sb = (unsigned)(e - (1023 + 52 - 127)) << 23;         // 2^(E - 52) as a float
#ifdef __CUDA_ARCH__
  hi = __uint_as_float(hb);
  lo = __int2float_rn(r) * __uint_as_float(sb);
#else
  float scale;
  std::memcpy(&hi, &hb, sizeof hi);
  std::memcpy(&scale, &sb, sizeof scale);
  lo = (float)r * scale;
#endif
}

// Counting placement by cell: copies reach their cell's slots [s, e) in arrival order (per-cell atomic
// counters), so a cell's values (particle << 5 | image) arrive permuted.  The final slot of value v is s plus
// the number of smaller values of its cell: values are distinct (one per copy), so the slots are a
// permutation of [s, e) and the cell ends up in increasing particle index, the reference's serial order
// (a particle has at most one copy per cell) -- the order a stable sort by cell gives.
__host__ __device__ __forceinline__ int rank_in_cell(const uint32_t* __restrict__ vals, int s, int e, uint32_t v) {
  int r = 0;
  int k = s;
  for (; k + 4 <= e; k += 4) {
    r += (vals[k] < v) ? 1 : 0;
    r += (vals[k + 1] < v) ? 1 : 0;
    r += (vals[k + 2] < v) ? 1 : 0;
    r += (vals[k + 3] < v) ? 1 : 0;
  }
  for (; k < e; k++) r += (vals[k] < v) ? 1 : 0;
  return r;
}

// cell_start from the keys sorted by cell: copy t writes the starts of the cells between the previous
// copy's cell (exclusive) and its own (inclusive); t = n closes the list up to ncells.
__host__ __device__ __forceinline__ void cell_starts_at(const uint32_t* __restrict__ skeys, int t, int n, int ncells,
                                               int* __restrict__ cell_start) {
  const int lo = (t == 0) ? 0 : (int)skeys[t - 1] + 1;
  const int hi = (t == n) ? ncells : (int)skeys[t];
  for (int c = lo; c <= hi && c <= ncells; c++) cell_start[c] = t;
}

// Copy t of the sorted list: particle p, image k, in the cell `li` (local index of its system).
template <class T, int N>
__host__ __device__ __forceinline__ void gather_at(const DevGeom<T>& g, const T* __restrict__ wrapped, int t, int p, int k,
                                          int li, T* __restrict__ px, T* __restrict__ py, T* __restrict__ pz,
                                          float4* __restrict__ off, float4* __restrict__ xq,
                                          int* __restrict__ code, int* __restrict__ cell_flags, int cb) {
  T q[N];
#pragma unroll
  for (int d = 0; d < N; d++) {
    T w = wrapped[(int64_t)p * N + d];
    q[d] = (k == g.zero_code) ? w : xadd(w, g.shift[k][d]);
  }
  const int pc = (k == g.zero_code) ? p : -(p + 1);
  px[t] = q[0];
  py[t] = q[1];
  if (N == 3) pz[t] = q[N - 1];
  if constexpr (std::is_same<T, float>::value) {
    // Float32 handles test the coordinates themselves (no cell-relative offsets are read)
    xq[t] = make_float4((float)q[0], (float)q[1], N == 3 ? (float)q[N - 1] : 0.f, bits_as_float(pc));
  } else {
    int c[3];
    cart_of(li, g.nc, N, c);
    float o[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < N; d++) {
      // FP32 offset of the copy from its cell origin, all in float pairs: (qh + ql) - (oh + ol)
      float oh, ol, qh, ql;
      origin_ff(g.cbf_hi[d], g.cbf_lo[d], g.csf[d], g.csf_lo[d], c[d] - 1, oh, ol);
      float_pair((double)q[d], qh, ql);
      o[d] = (qh - oh) + (ql - ol);
    }
    off[t] = make_float4(o[0], o[1], o[2], bits_as_float(pc));
  }
  code[t] = pc;
  if (k == g.zero_code) cell_flags[cb + li] = 1;  // the cell holds a real particle
}

}  // namespace clm
