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
__host__ __device__ __forceinline__ double xsqrt(double a) { return __dsqrt_rn(a); }
__host__ __device__ __forceinline__ float xsqrt(float a) { return __fsqrt_rn(a); }
template <class T> __host__ __device__ __forceinline__ T xfloor(T a) { return floor(a); }
template <class T> __host__ __device__ __forceinline__ T xabs(T a) { return fabs(a); }
#else
__host__ __device__ __forceinline__ double xsqrt(double a) { return std::sqrt(a); }
__host__ __device__ __forceinline__ float xsqrt(float a) { return std::sqrt(a); }
template <class T> __host__ __device__ __forceinline__ T xfloor(T a) { return std::floor(a); }
template <class T> __host__ __device__ __forceinline__ T xabs(T a) { return std::fabs(a); }
#endif

// ---------------------------------------------------------------- geometry on device
constexpr int kMaxDim = 3;

template <class T> struct DevGeom {
  int dim, kind, lcell;
  int nc[3];
  int ncells;
  T Min[3][3];    // input unit cell (wrap solve / product)
  T det_in;
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
  int img_tree;         // image-test pruning: 2 aligned cell exactly upper triangular (per dimension), 1 last
                        // row zero below the diagonal (per value of the last image index), 0 none
};

// StaticArrays solve (Cramer form), then fastmod1, boundary -> 0, then M*p and R*(.)
template <class T, int N>
__host__ __device__ __forceinline__ void wrap_point(const DevGeom<T>& g, const T* x, T* out) {
  T p[N];
  const auto& a = g.Min;
  if constexpr (N == 3) {
    p[0] = xdiv(xadd(xadd(xmul(xsub(xmul(a[1][1], a[2][2]), xmul(a[1][2], a[2][1])), x[0]),
                          xmul(xsub(xmul(a[0][2], a[2][1]), xmul(a[0][1], a[2][2])), x[1])),
                     xmul(xsub(xmul(a[0][1], a[1][2]), xmul(a[0][2], a[1][1])), x[2])),
                g.det_in);
    p[1] = xdiv(xadd(xadd(xmul(xsub(xmul(a[1][2], a[2][0]), xmul(a[1][0], a[2][2])), x[0]),
                          xmul(xsub(xmul(a[0][0], a[2][2]), xmul(a[0][2], a[2][0])), x[1])),
                     xmul(xsub(xmul(a[0][2], a[1][0]), xmul(a[0][0], a[1][2])), x[2])),
                g.det_in);
    p[2] = xdiv(xadd(xadd(xmul(xsub(xmul(a[1][0], a[2][1]), xmul(a[1][1], a[2][0])), x[0]),
                          xmul(xsub(xmul(a[0][1], a[2][0]), xmul(a[0][0], a[2][1])), x[1])),
                     xmul(xsub(xmul(a[0][0], a[1][1]), xmul(a[0][1], a[1][0])), x[2])),
                g.det_in);
  } else {
    p[0] = xdiv(xsub(xmul(a[1][1], x[0]), xmul(a[0][1], x[1])), g.det_in);
    p[1] = xdiv(xsub(xmul(a[0][0], x[1]), xmul(a[1][0], x[0])), g.det_in);
  }
#pragma unroll
  for (int i = 0; i < N; i++) {
    p[i] = xsub(p[i], xfloor(p[i]));
    if (p[i] == T(1)) p[i] = T(0);
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

template <class T, int N>
__host__ __device__ __forceinline__ bool in_box(const DevGeom<T>& g, const T* x) {
  bool ok = true;
#pragma unroll
  for (int i = 0; i < N; i++) ok = ok && (g.cbmin[i] <= x[i]) && (x[i] < g.cbmax[i]);
  return ok;
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

template <class T, int N>
__host__ __device__ __forceinline__ int cell_of(const DevGeom<T>& g, const T* x, bool real) {
  int li = 0;
#pragma unroll
  for (int i = N - 1; i >= 0; i--) {
    // floor in the handle dtype (exact; cell indices are far below 2^24), which keeps Float32 builds off
    // GB300's slow FP64 pipe
    const T fq = cell_floor<T>(xsub(x[i], g.cbmin[i]), g.cs[i], g.inv_cs[i]);
    if (!(fq >= T(-1) && fq < (T)g.nc[i])) return -1;
    int c = (int)fq + 1;
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
