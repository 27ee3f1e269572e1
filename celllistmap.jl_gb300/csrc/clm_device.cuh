// Device-side definitions shared by the build and pair kernels.
//
// Bit-exactness: every multiply/add/divide/sqrt on the exact path goes through
// the *_rn intrinsics below, which the compiler never fuses into FMAs, so the
// device reproduces the reference's separately rounded Julia arithmetic
// (Julia does not contract a*b+c).  The FP32 prefilter in the pair kernels is
// free to use FMAs: it only decides which pairs get an exact re-test.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace clm {

// ---------------------------------------------------------------- exact arithmetic
// On the device the _rn intrinsics; on the host (the CPU tests compile the geometry helpers below with
// -ffp-contract=off) the plain IEEE operations, which round the same way.
#ifdef __CUDA_ARCH__
#define CLM_XOP(name, T, expr_dev, expr_host) \
  __host__ __device__ __forceinline__ T name(T a, T b) { return expr_dev; }
#else
#define CLM_XOP(name, T, expr_dev, expr_host) \
  __host__ __device__ __forceinline__ T name(T a, T b) { return expr_host; }
#endif
CLM_XOP(xadd, double, __dadd_rn(a, b), a + b)
CLM_XOP(xsub, double, __dsub_rn(a, b), a - b)
CLM_XOP(xmul, double, __dmul_rn(a, b), a * b)
CLM_XOP(xdiv, double, __ddiv_rn(a, b), a / b)
CLM_XOP(xadd, float, __fadd_rn(a, b), a + b)
CLM_XOP(xsub, float, __fsub_rn(a, b), a - b)
CLM_XOP(xmul, float, __fmul_rn(a, b), a * b)
CLM_XOP(xdiv, float, __fdiv_rn(a, b), a / b)
#undef CLM_XOP
#ifdef __CUDA_ARCH__
__host__ __device__ __forceinline__ double xfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__host__ __device__ __forceinline__ double xsqrt(double a) { return __dsqrt_rn(a); }
__host__ __device__ __forceinline__ float xsqrt(float a) { return __fsqrt_rn(a); }
template <class T> __host__ __device__ __forceinline__ T xfloor(T a) { return floor(a); }
template <class T> __host__ __device__ __forceinline__ T xabs(T a) { return fabs(a); }
#else
__host__ __device__ __forceinline__ double xfma(double a, double b, double c) { return std::fma(a, b, c); }
__host__ __device__ __forceinline__ double xsqrt(double a) { return std::sqrt(a); }
__host__ __device__ __forceinline__ float xsqrt(float a) { return std::sqrt(a); }
template <class T> __host__ __device__ __forceinline__ T xfloor(T a) { return std::floor(a); }
template <class T> __host__ __device__ __forceinline__ T xabs(T a) { return std::fabs(a); }
#endif

// ---------------------------------------------------------------- order keys
// The bit pattern of a float or double with the magnitude bits of negative values inverted, read as a signed
// integer: a <= b as numbers implies key(a) <= key(b) (-0 sorts just below +0; a NaN lies outside
// [key(-inf), key(+inf)]).  The image tests compare these keys on the integer pipe.
template <class T> struct OrderKey;
template <> struct OrderKey<double> { using type = long long; };
template <> struct OrderKey<float> { using type = int; };

__host__ __device__ __forceinline__ long long order_key(double v) {
#ifdef __CUDA_ARCH__
  const long long b = __double_as_longlong(v);
#else
  long long b;
  std::memcpy(&b, &v, sizeof b);
#endif
  return b ^ (long long)((unsigned long long)(b >> 63) >> 1);
}
__host__ __device__ __forceinline__ int order_key(float v) {
#ifdef __CUDA_ARCH__
  const int b = __float_as_int(v);
#else
  int b;
  std::memcpy(&b, &v, sizeof b);
#endif
  return b ^ (int)((unsigned)(b >> 31) >> 1);
}

// The bit pattern of a double, and equality of bit patterns (on the integer pipe).
__host__ __device__ __forceinline__ long long dbits(double v) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(v);
#else
  long long b;
  std::memcpy(&b, &v, sizeof b);
  return b;
#endif
}
__host__ __device__ __forceinline__ bool same_bits(double a, double b) { return dbits(a) == dbits(b); }
__host__ __device__ __forceinline__ bool same_bits(float a, float b) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(a) == __float_as_uint(b);
#else
  unsigned x, y;
  std::memcpy(&x, &a, sizeof x);
  std::memcpy(&y, &b, sizeof y);
  return x == y;
#endif
}

// RN(a / b) in double from y = RN(1 / b): q = q0 + (a - q0 b) y with q0 = RN(a y) (Markstein's correction
// step), accepted when its remainder r = RN(a - q b) proves it: r = 0 (a = q b exactly: with q and b normal and
// |b| 2^(E(q) - 53) normal, a - q b is a multiple of 2^-1074 and cannot round to 0 unless it is 0), or q is not
// a power of two and |r| < |b| 2^(E(q) - 53) (the exact |a - q b| is then below that bound, which is
// representable, so |a / b - q| is less than half the spacing of the doubles around q; a quotient of two
// doubles is never a midpoint).  Otherwise (powers of two, zero, subnormal or extreme exponents, inf or NaN)
// the IEEE division decides.  Four FP64 operations and integer checks instead of the division sequence.
__host__ __device__ __forceinline__ bool quot_fast(double a, double b, double y, double& q) {
  const double q0 = xmul(a, y);
  q = xfma(xfma(-q0, b, a), y, q0);
  const double r = xfma(-q, b, a);
  constexpr long long kMag = 0x7FFFFFFFFFFFFFFFLL, kFrac = 0x000FFFFFFFFFFFFFLL;
  const long long bq = dbits(q), bb = dbits(b) & kMag, br = dbits(r) & kMag;
  const int eq = (int)((bq >> 52) & 0x7ff), eb = (int)(bb >> 52), es = eb + eq - (1023 + 53);
  return eq > 0 && eq < 0x7ff && eb > 0 && es > 0 && es < 0x7ff &&
         (br == 0 || ((bq & kFrac) != 0 && br < bb + (long long)(eq - (1023 + 53)) * (1LL << 52)));
}
#ifdef __CUDA_ARCH__
// a call, so that the compiler cannot evaluate the division ahead of the branch in every warp
static __device__ __noinline__ double div_rn_call(double a, double b) { return __ddiv_rn(a, b); }
#endif
__host__ __device__ __forceinline__ double quot_rn(double a, double b, double y) {
  double q;
  if (quot_fast(a, b, y, q)) return q;
#ifdef __CUDA_ARCH__
  return div_rn_call(a, b);
#else
  return a / b;
#endif
}
__host__ __device__ __forceinline__ float quot_rn(float a, float b, float) { return xdiv(a, b); }

// ---------------------------------------------------------------- geometry on device
constexpr int kMaxDim = 3;

template <class T> struct DevGeom {
  int dim, kind, lcell;
  int nc[3];
  int ncells;
  T Min[3][3];    // input unit cell (wrap solve / product)
  T det_in;
  T inv_det;      // RN(1 / det_in) (quot_rn)
  T cof[3][3];    // cofactors of the 3D Cramer solve, p_i = RN((cof[i][0] x0 + cof[i][1] x1 + cof[i][2] x2) / det)
  T R[3][3];      // rotation after wrapping (identity unless triclinic)
  T Rinv[3][3];   // rotation back for pair coordinates
  T shift[27][3]; // aligned-cell translation of image code k (first index fastest)
  T cbmin[3], cbmax[3], cs[3];
  T inv_cs[3];          // RN(1 / cs) in the handle dtype (cell_of's quotient screen)
  T cutoff, cutoff_sqr;
  double margin_wide;   // projection margin when lcell > 1 (computed in double, as the reference does)
  float csf[3];         // cell sizes in FP32 for the prefilter (high part)
  float csf_lo[3];      // cell size - csf (low part of the float pair)
  float cbf_hi[3], cbf_lo[3];  // computing-box minimum as a float pair
  float thr_hi, thr_lo; // FP32 prefilter bounds on d2 (maybe-inside / surely-inside)
  int zero_code;        // image code of the zero shift (13 in 3D, 4 in 2D)
  int nimg;             // 3^dim
  int shape;            // kShapeUpper: input cell and cofactors zero below the diagonal; kShapeDiag: both
                        // diagonal and R the identity (3D periodic cells); else kShapeGeneral
  int img_tree;         // image-test pruning: 2 aligned cell exactly upper triangular (per dimension), 1 last
                        // row zero below the diagonal (per value of the last image index), 0 none
  // image k of a wrapped position p lies in the computing box along axis d, cbmin[d] <= RN(p[d] + shift[k][d])
  // < cbmax[d], exactly when img_lo[k][d] <= order_key(p[d]) < img_hi[k][d]
  typename OrderKey<T>::type img_lo[27][3], img_hi[27][3];
};

template <class T>
__host__ __device__ __forceinline__ bool image_in(const DevGeom<T>& g, int k, int d, typename OrderKey<T>::type pk) {
  return g.img_lo[k][d] <= pk && pk < g.img_hi[k][d];
}

__host__ __device__ __forceinline__ unsigned long long mag_bits(double v) {
  return (unsigned long long)dbits(v) & 0x7FFFFFFFFFFFFFFFull;
}
__host__ __device__ __forceinline__ unsigned long long mag_bits(float v) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(v) & 0x7FFFFFFFu;
#else
  unsigned b;
  std::memcpy(&b, &v, sizeof b);
  return b & 0x7FFFFFFFu;
#endif
}
template <class T> __host__ __device__ __forceinline__ bool is_zero_bits(T v) { return mag_bits(v) == 0; }
template <class T> __host__ __device__ __forceinline__ bool is_finite_bits(T v) {
  return mag_bits(v) < (sizeof(T) == 8 ? 0x7FF0000000000000ull : 0x7F800000ull);
}

// Cell shapes whose wrap skips exact-zero terms (DevGeom::shape; 3D only).  A left-to-right sum of separately
// rounded products whose dropped terms are signed zeros (a zero coefficient times a finite value) equals the
// sum of the other terms whenever that sum is not zero: a zero term leaves a nonzero partial sum as it is,
// and can only change the sign of a zero one, after which the next nonzero term gives the same value either
// way.  So the shaped wrap keeps its result when every input is finite and no shortened sum is zero, and
// otherwise the particle takes the full sums.
enum : int { kShapeGeneral = 0, kShapeUpper = 1, kShapeDiag = 2 };

template <class T, int SH>
__host__ __device__ __forceinline__ bool wrap_point_shaped(const DevGeom<T>& g, const T* x, T* out) {
  if (!(is_finite_bits(x[0]) && is_finite_bits(x[1]) && is_finite_bits(x[2]))) return false;
  const auto& c = g.cof;
  const auto& a = g.Min;
  T p[3];
  if constexpr (SH == kShapeDiag) {
    p[0] = xmul(c[0][0], x[0]);
    p[1] = xmul(c[1][1], x[1]);
    p[2] = xmul(c[2][2], x[2]);
  } else {
    p[0] = xadd(xadd(xmul(c[0][0], x[0]), xmul(c[0][1], x[1])), xmul(c[0][2], x[2]));
    p[1] = xadd(xmul(c[1][1], x[1]), xmul(c[1][2], x[2]));
    p[2] = xmul(c[2][2], x[2]);
  }
  if (is_zero_bits(p[0]) || is_zero_bits(p[1]) || is_zero_bits(p[2])) return false;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    p[i] = quot_rn(p[i], g.det_in, g.inv_det);
    p[i] = xsub(p[i], xfloor(p[i]));
    if (same_bits(p[i], T(1))) p[i] = T(0);
  }
  T w[3];
  if constexpr (SH == kShapeDiag) {
    w[0] = xmul(a[0][0], p[0]);
    w[1] = xmul(a[1][1], p[1]);
    w[2] = xmul(a[2][2], p[2]);
  } else {
    w[0] = xadd(xadd(xmul(a[0][0], p[0]), xmul(a[0][1], p[1])), xmul(a[0][2], p[2]));
    w[1] = xadd(xmul(a[1][1], p[1]), xmul(a[1][2], p[2]));
    w[2] = xmul(a[2][2], p[2]);
  }
  if (is_zero_bits(w[0]) || is_zero_bits(w[1]) || is_zero_bits(w[2])) return false;
  if constexpr (SH == kShapeDiag) {
    // R is the identity: 1 * w_i is w_i and the other two terms are zeros
#pragma unroll
    for (int i = 0; i < 3; i++) out[i] = w[i];
  } else {
#pragma unroll
    for (int i = 0; i < 3; i++) out[i] = xadd(xadd(xmul(g.R[i][0], w[0]), xmul(g.R[i][1], w[1])), xmul(g.R[i][2], w[2]));
  }
  return true;
}

// StaticArrays solve (Cramer form), then fastmod1, boundary -> 0, then M*p and R*(.).  SH: the cell's shape
// (kShapeUpper / kShapeDiag skip its exact-zero terms where that is exact, see wrap_point_shaped).
template <class T, int N, int SH = kShapeGeneral>
__host__ __device__ __forceinline__ void wrap_point(const DevGeom<T>& g, const T* x, T* out) {
  if constexpr (N == 3 && SH != kShapeGeneral) {
    if (wrap_point_shaped<T, SH>(g, x, out)) return;
  }
  T p[N];
  const auto& a = g.Min;
  if constexpr (N == 3) {
    // the cofactors (each RN(RN(a b) - RN(c d)), as the solve rounds them) come precomputed with the geometry
#pragma unroll
    for (int i = 0; i < 3; i++)
      p[i] = quot_rn(xadd(xadd(xmul(g.cof[i][0], x[0]), xmul(g.cof[i][1], x[1])), xmul(g.cof[i][2], x[2])),
                     g.det_in, g.inv_det);
  } else {
    p[0] = xdiv(xsub(xmul(a[1][1], x[0]), xmul(a[0][1], x[1])), g.det_in);
    p[1] = xdiv(xsub(xmul(a[0][0], x[1]), xmul(a[1][0], x[0])), g.det_in);
  }
#pragma unroll
  for (int i = 0; i < N; i++) {
    p[i] = xsub(p[i], xfloor(p[i]));
    if (same_bits(p[i], T(1))) p[i] = T(0);  // p == 1 (the only value equal to 1 is 1), on the integer pipe
  }
  T w[N];
#pragma unroll
  for (int i = 0; i < N; i++) {
    T s = xmul(a[i][0], p[0]);
#pragma unroll
    for (int k = 1; k < N; k++) s = xadd(s, xmul(a[i][k], p[k]));
    w[i] = s;
  }
#pragma unroll
  for (int i = 0; i < N; i++) {
    T s = xmul(g.R[i][0], w[0]);
#pragma unroll
    for (int k = 1; k < N; k++) s = xadd(s, xmul(g.R[i][k], w[k]));
    out[i] = s;
  }
}

// floor((x - xmin)/cell_size) + 1 with the border-case shift for real particles
// (src/internals/Box.jl:499-508, src/internals/CellLists.jl:956-967).  Returns
// the 0-based linear cell index, or -1 if the cell is outside the grid.
// Only floor(RN(a / cs)) is used, so it is taken from qa = RN(a * RN(1 / cs)) when qa is more than 4 units in
// the last place (u = 2^-24 or 2^-53 relative) from an integer: qa is within (2u + u^2)|a/cs| of the real
// quotient and RN(a / cs) within u of it, so no integer lies between qa and RN(a / cs) and both floors agree.
// Nearer an integer (a chance of a few in 10^5 per coordinate) the IEEE division decides.  The fractional
// parts qa - floor(qa) and floor(qa) + 1 - qa are exact or rounded by far less than the margin.
template <class T> __host__ __device__ __forceinline__ T cell_floor(T a, T cs, T inv_cs) {
  constexpr T u = std::is_same<T, double>::value ? T(1.1102230246251565e-16) : T(5.9604645e-08f);
  const T qa = xmul(a, inv_cs);
  const T fq = xfloor(qa);
  const T m = T(4) * u * (qa < T(0) ? -qa : qa);
  if (xsub(qa, fq) > m && xsub(xadd(fq, T(1)), qa) > m) return fq;
  return xfloor(xdiv(a, cs));
}

// floor(qa) from the bit pattern of qa = RN(a * RN(1 / cs)), when that is also floor(RN(a / cs)): qa in
// (0, 2^31) and at least 5 units in the last place of qa from every integer (which is more than the 4u|qa|
// margin of cell_floor: qa < 2^(e+1), so 4u|qa| < 4 ulp).  Returns false otherwise (qa <= 0, near an integer,
// huge, inf or NaN); cell_floor then decides.  Integer operations only, off the FP64 pipe for doubles.
template <class T> struct FloatBits;
template <> struct FloatBits<double> {
  using U = unsigned long long;
  static constexpr int kMant = 52, kBias = 1023;
};
template <> struct FloatBits<float> {
  using U = unsigned;
  static constexpr int kMant = 23, kBias = 127;
};
template <class T> __host__ __device__ __forceinline__ bool floor_quot_bits(T qa, int& fq) {
  using U = typename FloatBits<T>::U;
  constexpr int M = FloatBits<T>::kMant;
  U b;
#ifdef __CUDA_ARCH__
  if constexpr (sizeof(T) == 8) b = (U)__double_as_longlong(qa);
  else b = (U)__float_as_uint(qa);
#else
  std::memcpy(&b, &qa, sizeof b);
#endif
  const int e = (int)(b >> M) - FloatBits<T>::kBias;  // the sign bit makes e > 30 for negative qa
  if (e < -1) {  // 0 < qa < 1/2 (zero and -0 go to cell_floor)
    fq = 0;
    return b != 0 && (b >> (8 * sizeof(U) - 1)) == 0;
  }
  if (e > 30) return false;
  const int sh = M - e;  // bits of the fraction, 1 .. M + 1
  const U mant = (b & ((U(1) << M) - 1)) | (U(1) << M);
  const U one = U(1) << sh, frac = mant & (one - 1);
  fq = (int)(mant >> sh);
  return frac > 4 && one - frac > 4;
}

// cell_floor and its range test for the values floor_quot_bits leaves (a call on the device, so that the
// division it may take stays off the common path): floor(RN(a / cs)) if in [-1, nc), else INT_MIN.
template <class T>
#ifdef __CUDA_ARCH__
__device__ __noinline__
#else
inline
#endif
int floor_quot_call(T a, T cs, T inv_cs, int nc) {
  const T fq = cell_floor<T>(a, cs, inv_cs);
  return (fq >= T(-1) && fq < (T)nc) ? (int)fq : INT32_MIN;
}

template <class T, int N>
__host__ __device__ __forceinline__ int cell_of(const DevGeom<T>& g, const T* x, bool real) {
  int li = 0;
#pragma unroll
  for (int i = N - 1; i >= 0; i--) {
    // floor(RN(RN(x - cbmin) / cs)) from the bits of the reciprocal product where that decides it, else
    // cell_floor in the handle dtype (exact; cell indices are far below 2^24)
    const T a = xsub(x[i], g.cbmin[i]);
    int fq;
    if (!floor_quot_bits<T>(xmul(a, g.inv_cs[i]), fq)) fq = floor_quot_call<T>(a, g.cs[i], g.inv_cs[i], g.nc[i]);
    if (fq < -1 || fq >= g.nc[i]) return -1;
    int c = fq + 1;
    if (real) {
      if (c == g.lcell) c += 1;
      if (c == g.nc[i] - g.lcell + 1) c -= 1;
    }
    if (c < 1 || c > g.nc[i]) return -1;
    li = li * g.nc[i] + (c - 1);
  }
  return li;
}

__host__ __device__ __forceinline__ void cart_of(int li, const int* nc, int dim, int* c) {
  c[0] = li % nc[0] + 1;
  int r = li / nc[0];
  if (dim == 3) {
    c[1] = r % nc[1] + 1;
    c[2] = r / nc[1] + 1;
  } else {
    c[1] = r + 1;
    c[2] = 1;
  }
}

// cell_center (src/internals/Box.jl:517-525)
template <class T, int N>
__host__ __device__ __forceinline__ void cell_center(const DevGeom<T>& g, const int* c, T* ctr) {
#pragma unroll
  for (int i = 0; i < N; i++) ctr[i] = xsub(xadd(g.cbmin[i], xmul(g.cs[i], (T)c[i])), xmul(g.cs[i], T(0.5)));  // cs/2 exactly
}

// Offset of the k-th cell of the stencil around a cell, in the reference's enumeration order: the forward
// half stencil neighbor_cells_forward (CartesianIndices (1:l, -l:l, -l:l), then (0, 1:l, -l:l), then
// (0, 0, 1:l), first index fastest; 2D likewise) or all neighbours neighbor_cells (-l:l in every dimension,
// the cell itself left out), src/internals/Box.jl:436-474.
template <int LC = 0>
__host__ __device__ __forceinline__ void stencil_offset(bool forward, int l_rt, int dim, int k, int* o) {
  const int l = LC ? LC : l_rt;  // LC: lcell fixed at compile time (constant divisors)
  const int w = 2 * l + 1;
  o[2] = 0;
  if (forward) {
    if (dim == 3) {
      const int nA = l * w * w, nB = l * w;
      if (k < nA) {
        o[0] = 1 + k % l;
        int r = k / l;
        o[1] = r % w - l;
        o[2] = r / w - l;
      } else if (k < nA + nB) {
        int k2 = k - nA;
        o[0] = 0;
        o[1] = 1 + k2 % l;
        o[2] = k2 / l - l;
      } else {
        o[0] = 0;
        o[1] = 0;
        o[2] = 1 + (k - nA - nB);
      }
    } else {
      const int nA = l * w;
      if (k < nA) {
        o[0] = 1 + k % l;
        o[1] = k / l - l;
      } else {
        o[0] = 0;
        o[1] = 1 + (k - nA);
      }
    }
  } else {
    int total = (dim == 3) ? w * w * w : w * w;
    int center = (total - 1) / 2;
    int kk = (k < center) ? k : k + 1;
    o[0] = kk % w - l;
    o[1] = (kk / w) % w - l;
    if (dim == 3) o[2] = kk / (w * w) - l;
  }
}

// Self pairs in triclinic cells, visited once per pair of cells.  The reference visits, from every cell
// holding a real particle, all its neighbour cells, and keeps the pairs (i, j) with i real and
// index_i < index_j (src/internals/self.jl:106-135,164-184, vicinal_cells.jl:48-75).  Here the pair of cells
// (A, B) is visited once: from A when B lies in A's forward half stencil, or when B lies in A's backward half
// and holds no real particle (no work item starts from B).  A visited pair of copies is then the reference's
// pair exactly when the copy with the lower particle index is real: that copy is the reference's i, the other
// its j.  Entry k (0-based) of the neighbour list of this visit: k < nf the forward half stencil in the
// reference's order, nf <= k < 2 nf the same offsets negated (the backward half), nf = ((2 lcell + 1)^dim - 1)/2.
template <int LC = 0>
__host__ __device__ __forceinline__ void sym_stencil_offset(int l_rt, int dim, int nf, int k, int* o, bool* back) {
  *back = k >= nf;
  stencil_offset<LC>(true, l_rt, dim, *back ? k - nf : k, o);
  if (*back) {
    o[0] = -o[0];
    o[1] = -o[1];
    o[2] = -o[2];
  }
}

// Which visits of a candidate pair the map keeps (src/internals/self.jl:143-184, cross.jl:111-129), for a
// particle copy i (slot ii of its cell) and a candidate copy j (slot slot_j; `same`: the same cell).
// Self pairs: orthorhombic cells keep a pair once (j after i in the same cell; any cell of the forward half
// stencil) when one of the copies is real; triclinic cells (visited once per pair of cells, see
// sym_stencil_offset) keep a pair once (j after i in the same cell) when the copy of the lower particle
// index is real; non-periodic systems have no images.  Cross pairs in orthorhombic cells: the particle copy
// must be real for a candidate of its own cell, and one of the two copies for a candidate of another cell;
// triclinic and non-periodic cross pairs keep every visit.
__host__ __device__ __forceinline__ bool pair_rule(bool cross, bool tri, bool nonper, bool same, int slot_j, int ii,
                                                   bool real_i, bool real_j, int idx_i, int idx_j) {
  bool cand = true;
  if (!cross) {
    if (tri) cand = (!same || slot_j > ii) && idx_i != idx_j && ((idx_i < idx_j) ? real_i : real_j);
    else if (same) cand = (slot_j > ii) && (nonper || real_i || real_j);
    else cand = nonper || real_i || real_j;
  } else {
    if (!tri && !nonper) cand = same ? real_i : (real_i || real_j);
  }
  return cand;
}

// pair_rule as the pair kernel applies it, in three parts.  In the FP32 distance pass: a pair of two images
// is dropped (the AND of the two particle codes, image = negative code, is negative), and in the cell itself
// the slots same_cell_dropped names are masked out per round.  In the hit queue: a triclinic self pair of a
// real copy and an image is kept when the copy of the lower index is real (sym_mixed_keeps).  Together
// these equal pair_rule (checked over every case by the CPU tests).
__host__ __device__ __forceinline__ bool same_cell_dropped(bool cross, bool tri, bool nonper, int slot_j, int ii,
                                                           bool real_i) {
  if (!cross) return slot_j <= ii;  // self pairs: each pair of the cell once, from its earlier slot
  return !tri && !nonper && !real_i;  // cross pairs, orthorhombic: the particle copy must be real
}
__host__ __device__ __forceinline__ bool sym_mixed_keeps(int code_i, int code_j) {
  const int idx_i = code_i >= 0 ? code_i : ~code_i, idx_j = code_j >= 0 ? code_j : ~code_j;
  return (idx_i < idx_j) ? code_i >= 0 : code_j >= 0;
}
__host__ __device__ __forceinline__ bool pair_rule_parts(bool cross, bool tri, bool nonper, bool same, int slot_j,
                                                         int ii, int code_i, int code_j) {
  if ((code_i & code_j) < 0) return false;
  if (same && same_cell_dropped(cross, tri, nonper, slot_j, ii, code_i >= 0)) return false;
  if (!cross && tri && (code_i ^ code_j) < 0) return sym_mixed_keeps(code_i, code_j);
  return true;
}

template <class T, int N>
__host__ __device__ __forceinline__ T exact_dot_rel(const T* x, const T* c, const T* u) {
  T s = xmul(xsub(x[0], c[0]), u[0]);
#pragma unroll
  for (int d = 1; d < N; d++) s = xadd(s, xmul(xsub(x[d], c[d]), u[d]));
  return s;
}

// The reference's projection filter for a pair seen from cell `from` (center cf) towards cell `to`
// (center ct): the particle of `to` must satisfy |proj| <= margin and |proj_to - proj_from| <= cutoff
// (src/internals/vicinal_cells.jl:4-75, auxiliary_functions.jl:66-111).
template <class T, int N>
__host__ __device__ bool projection_pass(const DevGeom<T>& g, const T* cf, const T* ct, const T* x_from,
                                         const T* x_to) {
  T dc[3] = {0, 0, 0};
#pragma unroll
  for (int d = 0; d < N; d++) dc[d] = xsub(ct[d], cf[d]);
  T s2 = xmul(dc[0], dc[0]);
#pragma unroll
  for (int d = 1; d < N; d++) s2 = xadd(s2, xmul(dc[d], dc[d]));
  T dcn = xsqrt(s2);
  T u[3] = {0, 0, 0};
#pragma unroll
  for (int d = 0; d < N; d++) u[d] = xdiv(dc[d], dcn);
  T pt = exact_dot_rel<T, N>(x_to, cf, u);
  bool keep = (g.lcell == 1) ? (xabs(pt) <= xadd(g.cutoff, xdiv(dcn, T(2)))) : ((double)xabs(pt) <= g.margin_wide);
  if (!keep) return false;
  T pf = exact_dot_rel<T, N>(x_from, cf, u);
  return xabs(xsub(pt, pf)) <= g.cutoff;
}

// Radial histogram bins (test/examples/pairwise_velocities.jl:17-24): the index of the first of the
// nbins + 1 ascending edges that is >= r (searchsortedfirst - 1 gives the bin: r on an edge goes to the
// lower bin, r <= edges[0] to none, r > edges[nbins] to none).
template <class E> __host__ __device__ __forceinline__ int first_edge_at_or_above(const E* edges, int nbins, E r) {
  int lo = 0, hi = nbins + 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (edges[mid] >= r) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// FP32 distance rf within 2^-12 (relative) of one of the two edges around it (lo from
// first_edge_at_or_above): the split form then decides the bin from the exact distance.
__host__ __device__ __forceinline__ bool near_edge(const float* edges, int nbins, int lo, float rf) {
  const float tol = rf * 2.44140625e-4f;
  return (lo <= nbins && xabs(edges[lo] - rf) <= tol) || (lo >= 1 && xabs(edges[lo - 1] - rf) <= tol);
}

// Device error bits (OR-ed into the handle's error word).
enum DevError : int {
  DERR_NAN = 1,
  DERR_CELL_RANGE = 2,
  DERR_COPY_OVERFLOW = 4,
  DERR_NL_OVERFLOW = 8,
  DERR_SCAN = 16,  // a single-pass scan gave up waiting for the prefix of an earlier tile
  DERR_STAGE = 32, // the pair kernel gave up waiting for the bulk copies of a staging window
  DERR_TILE_OVERFLOW = 64,  // a tile of the counting build had more copies than its staging slots
};

}  // namespace clm
