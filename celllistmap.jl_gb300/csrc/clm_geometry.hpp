// Host-side box geometry of the cutoff-pair engine: the O(1) part of
// CellListMap.jl's `Box` (src/internals/Box.jl:191-270), computed in the
// handle's dtype with the reference's operation order so that the device
// kernels see the same cell sizes, computing box and rotation.
//
//   Box construction        src/internals/Box.jl:240-270
//   number/size of cells    src/internals/Box.jl:209-220
//   unit-cell check         src/internals/Box.jl:579-636
//   cell alignment          src/internals/CellOperations.jl:377-423 (3D), 353-375 (2D)
//   cell limits / vertices  src/internals/CellOperations.jl:431-479
//   non-periodic box        src/internals/Box.jl:38, 374-377
//   StaticArrays det/inv/\  (3x3 and 2x2 closed forms; products are left-folded sums)
//
// The host compiler must not contract a*b+c (built with -ffp-contract=off).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace clm {

enum Kind { ORTHO = 0, TRICLINIC = 1, NONPERIODIC = 2 };

template <class T> struct Geometry {
  int dim = 3, kind = ORTHO, lcell = 1;
  T Min[3][3] = {};   // input unit cell, [row][col]
  T Mal[3][3] = {};   // aligned unit cell
  T R[3][3] = {};     // rotation applied after wrapping
  T Rinv[3][3] = {};  // inverse rotation (pair coordinates are rotated back with it)
  T det_in = 0;       // det(Min), divisor of the wrap solve
  int64_t nc[3] = {1, 1, 1};
  T cs[3] = {};       // cell sizes
  T cbmin[3] = {}, cbmax[3] = {};
  T origin[3] = {};
  T cutoff = 0, cutoff_sqr = 0;
  int64_t ncells() const {
    int64_t p = 1;
    for (int i = 0; i < dim; i++) p *= nc[i];
    return p;
  }
};

namespace geo {

template <class T> inline T jmin(T a, T b) { return a < b ? a : (b < a ? b : (std::signbit(a) ? a : b)); }
template <class T> inline T jmax(T a, T b) { return a > b ? a : (b > a ? b : (std::signbit(a) ? b : a)); }

// norm of a column of a static matrix: squares in T, sum in double (generic_norm2)
template <class T> T colnorm(const T* v, int n) {
  T mx = 0;
  for (int i = 0; i < n; i++) mx = jmax(mx, (T)std::fabs(v[i]));
  if (mx == 0 || std::isinf(mx)) return mx;
  double s = 0;
  for (int i = 0; i < n; i++) {
    T sq = v[i] * v[i];
    s = (i == 0) ? (double)sq : s + (double)sq;
  }
  return (T)std::sqrt(s);
}

template <class T> inline T dot(const T* a, const T* b, int n) {
  T s = a[0] * b[0];
  for (int i = 1; i < n; i++) s = s + a[i] * b[i];
  return s;
}

template <class T> inline void cross(const T* a, const T* b, T* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

template <class T> void mul(const T A[3][3], const T B[3][3], T C[3][3], int n) {
  T tmp[3][3];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T s = A[i][0] * B[0][j];
      for (int k = 1; k < n; k++) s = s + A[i][k] * B[k][j];
      tmp[i][j] = s;
    }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) C[i][j] = tmp[i][j];
}

template <class T> void identity(T A[3][3], int n) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) A[i][j] = (i == j && i < n) ? T(1) : T(0);
}

template <class T> void column(const T A[3][3], int c, T* v, int n) {
  for (int i = 0; i < n; i++) v[i] = A[i][c];
}

template <class T> T det(const T A[3][3], int n) {
  if (n == 2) return A[0][0] * A[1][1] - A[0][1] * A[1][0];
  T c0[3], c1[3], c2[3], cr[3];
  column(A, 0, c0, 3);
  column(A, 1, c1, 3);
  column(A, 2, c2, 3);
  cross(c1, c2, cr);
  return dot(c0, cr, 3);
}

template <class T> void inverse(const T A[3][3], T B[3][3], int n) {
  if (n == 2) {
    T d = det(A, 2);
    B[0][0] = A[1][1] / d;
    B[1][0] = (-A[1][0]) / d;
    B[0][1] = (-A[0][1]) / d;
    B[1][1] = A[0][0] / d;
    return;
  }
  T x0[3], x1[3], x2[3], y0[3], y1[3], y2[3];
  column(A, 0, x0, 3);
  column(A, 1, x1, 3);
  column(A, 2, x2, 3);
  cross(x1, x2, y0);
  T d = dot(x0, y0, 3);
  for (int i = 0; i < 3; i++) {
    x0[i] = x0[i] / d;
    y0[i] = y0[i] / d;
  }
  cross(x2, x0, y1);
  cross(x0, x1, y2);
  for (int i = 0; i < 3; i++) {
    B[0][i] = y0[i];
    B[1][i] = y1[i];
    B[2][i] = y2[i];
  }
}

// align_cell: longest lattice vector along x, (a,b) plane normal to z.
template <class T> void align3(const T M[3][3], T out[3][3], T Rot[3][3]) {
  T m[3][3];
  std::memcpy(m, M, sizeof(m));
  T sq[3];
  for (int c = 0; c < 3; c++) sq[c] = (m[0][c] * m[0][c] + m[1][c] * m[1][c]) + m[2][c] * m[2][c];
  static const int order[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  int lead = 0;
  for (auto& o : order)
    if (sq[o[0]] >= sq[o[1]] && sq[o[1]] >= sq[o[2]]) {
      lead = o[0];
      break;
    }
  T a[3];
  column(m, lead, a, 3);
  T na = colnorm(a, 3);
  T u[3] = {a[0] / na, a[1] / na, a[2] / na};
  T v[3] = {T(0), u[2], -u[1]};
  T vv = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
  T R1[3][3];
  identity(R1, 3);
  if (vv != 0) {
    T K[3][3] = {{T(0), -v[2], v[1]}, {v[2], T(0), -v[0]}, {-v[1], v[0], T(0)}};
    T K2[3][3];
    mul(K, K, K2, 3);
    T s = T(1) / (T(1) + u[0]);
    T I[3][3];
    identity(I, 3);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) R1[i][j] = (I[i][j] + K[i][j]) + K2[i][j] * s;
  }
  mul(R1, m, m, 3);
  T bx = m[0][1], by = m[1][1], bz = m[2][1];
  T R2[3][3];
  identity(R2, 3);
  T yz = by * by + bz * bz;
  if (yz != 0) {
    T s2 = (m[0][1] * m[0][1] + m[1][1] * m[1][1]) + m[2][1] * m[2][1];
    T b = std::sqrt(s2 - bx * bx);
    T sn = ((-bz) * b) / yz;
    T cn = std::sqrt(T(1) - sn * sn);
    R2[1][1] = cn;
    R2[1][2] = -sn;
    R2[2][1] = sn;
    R2[2][2] = cn;
  }
  mul(R2, m, out, 3);
  mul(R2, R1, Rot, 3);
}

template <class T> void align2(const T M[3][3], T out[3][3], T Rot[3][3]) {
  T a[2] = {M[0][0], M[1][0]}, b[2] = {M[0][1], M[1][1]};
  if (colnorm(b, 2) > colnorm(a, 2)) {
    a[0] = b[0];
    a[1] = b[1];
  }
  identity(Rot, 2);
  std::memcpy(out, M, sizeof(T) * 9);
  if (a[1] == 0) return;
  T na = colnorm(a, 2);
  T sn = (-na) / ((a[0] * a[0]) / a[1] + a[1]);
  T cn = ((-a[0]) * sn) / a[1];
  Rot[0][0] = cn;
  Rot[0][1] = -sn;
  Rot[1][0] = sn;
  Rot[1][1] = cn;
  mul(Rot, M, out, 2);
}

// distance between opposite cell planes must exceed twice the cutoff
template <class T> bool planes_ok(const T m[3][3], int n, T cutoff) {
  T two = T(2) * cutoff;
  if (n == 3) {
    T a[3], b[3], c[3];
    column(m, 0, a, 3);
    column(m, 1, b, 3);
    column(m, 2, c, 3);
    auto proj = [&](const T* p, const T* q, const T* r) {
      T w[3];
      cross(p, q, w);
      T nw = colnorm(w, 3);
      for (int i = 0; i < 3; i++) w[i] = w[i] / nw;
      return dot(r, w, 3);
    };
    T ap = proj(b, c, a), cp = proj(a, b, c), bp = proj(c, a, b);
    return !(ap <= two || bp <= two || cp <= two);
  }
  T a[2] = {m[0][0], m[1][0]}, b[2] = {m[0][1], m[1][1]};
  T na = colnorm(a, 2);
  T ia[2] = {a[0] / na, a[1] / na};
  T t = dot(b, ia, 2);
  T bp = std::sqrt((b[0] * b[0] + b[1] * b[1]) - t * t);
  T nb = colnorm(b, 2);
  T ib[2] = {b[0] / nb, b[1] / nb};
  T s = dot(a, ib, 2);
  T ap = std::sqrt((a[0] * a[0] + a[1] * a[1]) - s * s);
  return !(ap <= two || bp <= two);
}

template <class T> void limits(const T m[3][3], int n, T* lo, T* hi) {
  T v[8][3];
  int nv = (n == 3) ? 8 : 4;
  for (int i = 0; i < n; i++) {
    T a = m[i][0], b = m[i][1];
    v[0][i] = 0;
    v[1][i] = a;
    v[2][i] = a + b;
    v[3][i] = b;
    if (n == 3) {
      T c = m[i][2];
      v[4][i] = a + c;
      v[5][i] = c;
      v[6][i] = b + c;
      v[7][i] = (a + b) + c;
    }
  }
  for (int i = 0; i < n; i++) lo[i] = hi[i] = v[0][i];
  for (int k = 1; k < nv; k++)
    for (int i = 0; i < n; i++) {
      lo[i] = jmin(lo[i], v[k][i]);
      hi[i] = jmax(hi[i], v[k][i]);
    }
}

}  // namespace geo

// Returns 0 on success or a clm_status code.  `M` is the input unit cell
// [row][col] in T (for NONPERIODIC the caller passes the padded limits box and
// its origin, see nonperiodic_cell()).
template <class T>
int make_geometry(Geometry<T>& g, int dim, int kind, const T M[3][3], T cutoff, int lcell, const T* origin) {
  if (lcell < 1) return 10;
  g.dim = dim;
  g.kind = kind;
  g.lcell = lcell;
  g.cutoff = cutoff;
  std::memset(g.Min, 0, sizeof(g.Min));
  for (int i = 0; i < dim; i++)
    for (int j = 0; j < dim; j++) g.Min[i][j] = M[i][j];
  for (int i = 0; i < 3; i++) g.origin[i] = (origin && i < dim) ? origin[i] : T(0);
  if (kind == TRICLINIC) {
    if (dim == 3) geo::align3(g.Min, g.Mal, g.R);
    else geo::align2(g.Min, g.Mal, g.R);
  } else {
    std::memcpy(g.Mal, g.Min, sizeof(g.Min));
    geo::identity(g.R, dim);
  }
  if (!geo::planes_ok(g.Mal, dim, cutoff)) return 2;
  T lo[3], hi[3];
  geo::limits(g.Mal, dim, lo, hi);
  T step = cutoff / T(lcell);
  for (int i = 0; i < dim; i++) {
    T q = (hi[i] - lo[i]) / step;
    int64_t n0;
    if (kind == TRICLINIC) {
      n0 = (int64_t)std::ceil(q);
      g.cs[i] = step;
    } else {
      n0 = (int64_t)std::floor(q);
      g.cs[i] = (hi[i] - lo[i]) / T(n0);
    }
    g.nc[i] = n0 + 2 * lcell + 1;
    T pad = T(lcell) * g.cs[i];
    g.cbmin[i] = (lo[i] + g.origin[i]) - pad;
    g.cbmax[i] = (hi[i] + g.origin[i]) + pad;
  }
  for (int i = dim; i < 3; i++) {
    g.nc[i] = 1;
    g.cs[i] = 0;
  }
  g.cutoff_sqr = cutoff * cutoff;
  geo::inverse(g.R, g.Rinv, dim);
  g.det_in = geo::det(g.Min, dim);
  return 0;
}

// Padded box of a non-periodic system from the particle limits:
// sides = (max - min) + 210*cutoff/100, origin = min (src/internals/Box.jl:38).
template <class T> void nonperiodic_cell(int dim, const T* lo, const T* hi, T cutoff, T M[3][3], T* origin) {
  T pad = (T(210) * cutoff) / T(100);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) M[i][j] = 0;
  for (int i = 0; i < dim; i++) {
    M[i][i] = (hi[i] - lo[i]) + pad;
    origin[i] = lo[i];
  }
}

// Bound on the error of the FP32 pair distance of the split form (Float64 handles): the offsets of the
// copies from their cell origins (at most a cell side, within 2^-23 relative), the cell displacement added
// to the candidate's offset (at most lcell cells, the FP32 cell side within 2^-24), and the subtraction give
// each component an absolute error below (3 lcell + 5) cell_side 2^-24, the distance below sqrt(dim) times
// that, plus its own few-ulp rounding.
template <class T> double split_distance_error(const Geometry<T>& g) {
  double cs = 0.0;
  for (int i = 0; i < g.dim; i++) cs = std::max(cs, (double)g.cs[i]);
  return std::sqrt((double)g.dim) * (3.0 * g.lcell + 5.0) * cs * std::ldexp(1.0, -24);
}

// The split-form radial histogram decides bins from that FP32 distance and re-decides exactly within 2^-12
// (relative) of an edge, which covers the error for every edge above split_distance_error * 2^12.  True when
// all positive edges are above it (the bins then equal the exact form's).  An edge at 0 only separates
// pairs at distance 0, which the FP32 distance also gives as 0 for copies of the same cell.
template <class T> bool split_bins_exact(const Geometry<T>& g, const double* edges, int nedges) {
  const double rmin = split_distance_error(g) * 4096.0;
  for (int k = 0; k < nedges; k++)
    if (edges[k] > 0.0 && edges[k] < rmin) return false;
  return true;
}

}  // namespace clm
