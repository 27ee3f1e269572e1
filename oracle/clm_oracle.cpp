// CPU restatement of CellListMap.jl's cutoff-pair engine.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA library is
// checked against, and the CPU baseline that bench.py times.  Nothing in the
// shipped library links, loads or calls it.
//
// It follows the reference's serial code path operation by operation (same
// formulas, same evaluation order, no FMA contraction: build with
// -ffp-contract=off), for Float32 and Float64, 2D and 3D, orthorhombic,
// triclinic and non-periodic boxes:
//   box geometry      src/internals/Box.jl:191-270, 209-220, 577-636
//   cell alignment    src/internals/CellOperations.jl:337-442
//   wrapping          src/internals/CellOperations.jl:30, 56-66, 91-94
//   ghost images      src/internals/Box.jl:536-566, CellOperations.jl:138-139
//   serial build      src/internals/CellLists.jl:940-1057
//   non-periodic path src/internals/NonPeriodicCells.jl:63-70, 281-352
//   self map          src/internals/self.jl:50-63, 106-184
//   cross map         src/internals/cross.jl:30-129
//   projection cull   src/internals/vicinal_cells.jl:4-75,
//                     src/internals/auxiliary_functions.jl:66-111
//   naive oracle      test/modules/Testing.jl:62-104 (wrap_relative_to,
//                     CellOperations.jl:102-127)
// Operator semantics follow the reference's examples:
//   neighbour list    src/internals/neighborlist.jl:67-76
//   forces            test/examples/gravitational_force.jl:37-44
//   min distance      test/examples/nearest_neighbor.jl:9-16,43
//   radial histogram  test/examples/pairwise_velocities.jl:17-24
//
// Third-party arithmetic that the reference takes from StaticArrays.jl
// (not vendored, compat 1.9.15): `M \ x` for 2x2/3x3 static matrices is the
// Cramer/adjugate solve divided by det(M) (det = dot(col1, cross(col2, col3)));
// matrix products are left-folded sums of products; SVector `norm` is
// sqrt of the left-folded sum of squares.  Column views of a static matrix go
// through LinearAlgebra's generic_norm2 (sum accumulated in Float64).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <array>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

typedef struct {
  int32_t dtype;   // 0 = Float32, 1 = Float64
  int32_t dim;     // 2 or 3
  int32_t kind;    // 0 orthorhombic, 1 triclinic, 2 non-periodic
  int32_t lcell;
  double cutoff;
  double M[9];     // input unit cell, column-major dim x dim (columns = lattice vectors)
} orc_spec;

typedef struct {
  int64_t nc[3];
  double cell_size[3];
  double cbmin[3];
  double cbmax[3];
  double origin[3];
  double Min[9];
  double Mal[9];
  double R[9];
  double Rinv[9];
  double cutoff;
  double cutoff_sqr;
} orc_boxinfo;

typedef struct {
  int32_t op;
  int32_t nthreads;
  int32_t compensated;
  int32_t ntypes;
  const int32_t* types_x;
  const int32_t* types_y;
  double p[8];
  const double* eps_table;
  const double* sig_table;
  const double* vel_x;
  const double* vel_y;
  const double* bins;
  int32_t nbins;
  int32_t pad_;
  const double* weights_x;  // WEIGHTED_INV_D: per-particle weights (masses, charges) of x and y
  const double* weights_y;
} orc_op;

typedef struct {
  int64_t nl_cap;
  int64_t nl_n;
  int64_t* nl_i;
  int64_t* nl_j;
  double* nl_d;
  double scalar;
  int64_t count;
  double* forces_x;
  double* forces_y;
  int64_t min_i;
  int64_t min_j;
  double min_d;
  int64_t* hist_count;
  double* hist_sum;
  double adj[32];  // LJ adjoint: virial W (9, row-major), dU/deps (classes), dU/dsigma (classes)
} orc_result;

}  // extern "C"

namespace {

enum { KIND_ORTHO = 0, KIND_TRI = 1, KIND_NONPER = 2 };
enum {
  OP_NL = 1, OP_COUNT = 2, OP_SUM_D2 = 3, OP_SUM_D = 4, OP_SUM_INV_D = 5,
  OP_SOFT_ENERGY = 6, OP_SOFT_FORCES = 7, OP_LJ_ENERGY = 8, OP_LJ_FORCES = 9,
  OP_MINDIST = 10, OP_RHIST = 11, OP_INV_D_FORCES = 12, OP_LJ_ADJOINT = 13, OP_WEIGHTED_INV_D = 14
};
enum {
  ERR_OK = 0, ERR_ARG = 1, ERR_CELL_TOO_SMALL = 2, ERR_NAN = 3, ERR_DIM = 4,
  ERR_CAPACITY = 6, ERR_LCELL = 10
};

// Julia's min/max on floats prefer -0.0 / +0.0 respectively (no NaNs here).
inline int orc_max_threads_impl() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

template <class T> inline T jmin(T a, T b) {
  if (a < b) return a;
  if (b < a) return b;
  return std::signbit(a) ? a : b;
}
template <class T> inline T jmax(T a, T b) {
  if (a > b) return a;
  if (b > a) return b;
  return std::signbit(a) ? b : a;
}

// LinearAlgebra.generic_norm2 on a column view: squares rounded in T, summed
// in Float64, sqrt in Float64, converted back to T.
template <class T, int N> T gnorm2(const T* v) {
  T mx = 0;
  for (int i = 0; i < N; i++) mx = jmax(mx, (T)std::fabs(v[i]));
  if (mx == 0 || std::isinf(mx)) return mx;
  double s = (double)(T)(v[0] * v[0]);
  for (int i = 1; i < N; i++) s = s + (double)(T)(v[i] * v[i]);
  return (T)std::sqrt(s);
}

// StaticArrays norm of an SVector: sqrt(left-folded sum of squares) in T.
template <class T, int N> inline T snorm(const T* v) {
  T s = v[0] * v[0];
  for (int i = 1; i < N; i++) s = s + v[i] * v[i];
  return std::sqrt(s);
}

template <class T, int N> struct Mat {
  T a[N][N];  // a[row][col]
};

template <class T, int N> Mat<T, N> eye() {
  Mat<T, N> m;
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) m.a[i][j] = (i == j) ? T(1) : T(0);
  return m;
}

template <class T, int N> Mat<T, N> matmul(const Mat<T, N>& A, const Mat<T, N>& B) {
  Mat<T, N> C;
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      T s = A.a[i][0] * B.a[0][j];
      for (int k = 1; k < N; k++) s = s + A.a[i][k] * B.a[k][j];
      C.a[i][j] = s;
    }
  return C;
}

template <class T, int N> inline void matvec(const Mat<T, N>& A, const T* x, T* y) {
  for (int i = 0; i < N; i++) {
    T s = A.a[i][0] * x[0];
    for (int k = 1; k < N; k++) s = s + A.a[i][k] * x[k];
    y[i] = s;
  }
}

template <class T> inline void cross3(const T* a, const T* b, T* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

template <class T, int N> inline T dotN(const T* a, const T* b) {
  T s = a[0] * b[0];
  for (int i = 1; i < N; i++) s = s + a[i] * b[i];
  return s;
}

// StaticArrays det
template <class T> T det(const Mat<T, 3>& A) {
  T x1[3] = {A.a[0][1], A.a[1][1], A.a[2][1]};
  T x2[3] = {A.a[0][2], A.a[1][2], A.a[2][2]};
  T x0[3] = {A.a[0][0], A.a[1][0], A.a[2][0]};
  T c[3];
  cross3(x1, x2, c);
  return dotN<T, 3>(x0, c);
}
template <class T> T det(const Mat<T, 2>& A) {
  return A.a[0][0] * A.a[1][1] - A.a[0][1] * A.a[1][0];
}

// StaticArrays `a \ b` (Cramer form) for 3x3 and 2x2.
template <class T> inline void solve(const Mat<T, 3>& m, T d, const T* b, T* p) {
  const auto& a = m.a;
  p[0] = (((a[1][1] * a[2][2] - a[1][2] * a[2][1]) * b[0] + (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * b[1]) +
          (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * b[2]) / d;
  p[1] = (((a[1][2] * a[2][0] - a[1][0] * a[2][2]) * b[0] + (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * b[1]) +
          (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * b[2]) / d;
  p[2] = (((a[1][0] * a[2][1] - a[1][1] * a[2][0]) * b[0] + (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * b[1]) +
          (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * b[2]) / d;
}
template <class T> inline void solve(const Mat<T, 2>& m, T d, const T* b, T* p) {
  const auto& a = m.a;
  p[0] = (a[1][1] * b[0] - a[0][1] * b[1]) / d;
  p[1] = (a[0][0] * b[1] - a[1][0] * b[0]) / d;
}

// StaticArrays inv for 3x3 and 2x2.
template <class T> Mat<T, 3> inv(const Mat<T, 3>& A) {
  T x0[3] = {A.a[0][0], A.a[1][0], A.a[2][0]};
  T x1[3] = {A.a[0][1], A.a[1][1], A.a[2][1]};
  T x2[3] = {A.a[0][2], A.a[1][2], A.a[2][2]};
  T y0[3], y1[3], y2[3];
  cross3(x1, x2, y0);
  T d = dotN<T, 3>(x0, y0);
  for (int i = 0; i < 3; i++) { x0[i] = x0[i] / d; y0[i] = y0[i] / d; }
  cross3(x2, x0, y1);
  cross3(x0, x1, y2);
  Mat<T, 3> B;
  for (int i = 0; i < 3; i++) { B.a[0][i] = y0[i]; B.a[1][i] = y1[i]; B.a[2][i] = y2[i]; }
  return B;
}
template <class T> Mat<T, 2> inv(const Mat<T, 2>& A) {
  T d = det(A);
  Mat<T, 2> B;
  B.a[0][0] = A.a[1][1] / d;
  B.a[1][0] = (-A.a[1][0]) / d;
  B.a[0][1] = (-A.a[0][1]) / d;
  B.a[1][1] = A.a[0][0] / d;
  return B;
}

// align_cell (CellOperations.jl:377-423)
template <class T> void align(const Mat<T, 3>& m0, Mat<T, 3>& mout, Mat<T, 3>& R) {
  Mat<T, 3> m = m0;
  T n[3];
  for (int c = 0; c < 3; c++) n[c] = (m.a[0][c] * m.a[0][c] + m.a[1][c] * m.a[1][c]) + m.a[2][c] * m.a[2][c];
  static const int comb[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  int ia = 0;
  for (int q = 0; q < 6; q++) {
    int i = comb[q][0], j = comb[q][1], k = comb[q][2];
    if (n[i] >= n[j] && n[j] >= n[k]) { ia = i; break; }
  }
  T a[3] = {m.a[0][ia], m.a[1][ia], m.a[2][ia]};
  T na = gnorm2<T, 3>(a);
  T a1[3] = {a[0] / na, a[1] / na, a[2] / na};
  T v[3] = {T(0), a1[2], -a1[1]};
  T sv = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
  Mat<T, 3> R1 = eye<T, 3>();
  if (!(sv == 0)) {
    Mat<T, 3> vs;
    vs.a[0][0] = 0;     vs.a[0][1] = -v[2]; vs.a[0][2] = v[1];
    vs.a[1][0] = v[2];  vs.a[1][1] = 0;     vs.a[1][2] = -v[0];
    vs.a[2][0] = -v[1]; vs.a[2][1] = v[0];  vs.a[2][2] = 0;
    Mat<T, 3> vs2 = matmul(vs, vs);
    T s = T(1) / (T(1) + a1[0]);
    Mat<T, 3> I = eye<T, 3>();
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) R1.a[i][j] = (I.a[i][j] + vs.a[i][j]) + vs2.a[i][j] * s;
  }
  m = matmul(R1, m);
  T x = m.a[0][1], y = m.a[1][1], z = m.a[2][1];
  Mat<T, 3> R2 = eye<T, 3>();
  T yz = y * y + z * z;
  if (!(yz == 0)) {
    T s2 = (m.a[0][1] * m.a[0][1] + m.a[1][1] * m.a[1][1]) + m.a[2][1] * m.a[2][1];
    T b = std::sqrt(s2 - x * x);
    T sinT = ((-z) * b) / yz;
    T cosT = std::sqrt(T(1) - sinT * sinT);
    R2.a[1][1] = cosT; R2.a[1][2] = -sinT;
    R2.a[2][1] = sinT; R2.a[2][2] = cosT;
  }
  mout = matmul(R2, m);
  R = matmul(R2, R1);
}

template <class T> void align(const Mat<T, 2>& m0, Mat<T, 2>& mout, Mat<T, 2>& R) {
  Mat<T, 2> m = m0;
  T a[2] = {m.a[0][0], m.a[1][0]};
  T b[2] = {m.a[0][1], m.a[1][1]};
  if (gnorm2<T, 2>(b) > gnorm2<T, 2>(a)) { a[0] = b[0]; a[1] = b[1]; }
  if (a[1] == 0) {
    R = eye<T, 2>();
    mout = m;
    return;
  }
  T na = gnorm2<T, 2>(a);
  T sinT = (-na) / ((a[0] * a[0]) / a[1] + a[1]);
  T cosT = ((-a[0]) * sinT) / a[1];
  R.a[0][0] = cosT; R.a[0][1] = -sinT;
  R.a[1][0] = sinT; R.a[1][1] = cosT;
  mout = matmul(R, m);
}

// check_unit_cell (Box.jl:579-636)
template <class T> bool check_cell(const Mat<T, 3>& m, T cutoff) {
  T a[3], b[3], c[3];
  for (int i = 0; i < 3; i++) { a[i] = m.a[i][0]; b[i] = m.a[i][1]; c[i] = m.a[i][2]; }
  T bc[3], ab[3], ca[3];
  cross3(b, c, bc);
  T nbc = gnorm2<T, 3>(bc);
  for (int i = 0; i < 3; i++) bc[i] = bc[i] / nbc;
  T aproj = dotN<T, 3>(a, bc);
  cross3(a, b, ab);
  T nab = gnorm2<T, 3>(ab);
  for (int i = 0; i < 3; i++) ab[i] = ab[i] / nab;
  T cproj = dotN<T, 3>(c, ab);
  cross3(c, a, ca);
  T nca = gnorm2<T, 3>(ca);
  for (int i = 0; i < 3; i++) ca[i] = ca[i] / nca;
  T bproj = dotN<T, 3>(b, ca);
  T two = T(2) * cutoff;
  return !((aproj <= two) || (bproj <= two) || (cproj <= two));
}
template <class T> bool check_cell(const Mat<T, 2>& m, T cutoff) {
  T a[2] = {m.a[0][0], m.a[1][0]};
  T b[2] = {m.a[0][1], m.a[1][1]};
  T na = gnorm2<T, 2>(a);
  T iv[2] = {a[0] / na, a[1] / na};
  T db = dotN<T, 2>(b, iv);
  T bproj = std::sqrt((b[0] * b[0] + b[1] * b[1]) - db * db);
  T nb = gnorm2<T, 2>(b);
  T jv[2] = {b[0] / nb, b[1] / nb};
  T da = dotN<T, 2>(a, jv);
  T aproj = std::sqrt((a[0] * a[0] + a[1] * a[1]) - da * da);
  T two = T(2) * cutoff;
  return !((aproj <= two) || (bproj <= two));
}

// cell_limits over the 2^N vertices (CellOperations.jl:431-479)
template <class T> void cell_limits(const Mat<T, 3>& m, T* xmin, T* xmax) {
  T a[3], b[3], c[3];
  for (int i = 0; i < 3; i++) { a[i] = m.a[i][0]; b[i] = m.a[i][1]; c[i] = m.a[i][2]; }
  T v[8][3];
  for (int i = 0; i < 3; i++) {
    v[0][i] = 0; v[1][i] = a[i]; v[2][i] = a[i] + b[i]; v[3][i] = b[i];
    v[4][i] = a[i] + c[i]; v[5][i] = c[i]; v[6][i] = b[i] + c[i]; v[7][i] = (a[i] + b[i]) + c[i];
  }
  for (int i = 0; i < 3; i++) { xmin[i] = v[0][i]; xmax[i] = v[0][i]; }
  for (int k = 1; k < 8; k++)
    for (int i = 0; i < 3; i++) { xmin[i] = jmin(xmin[i], v[k][i]); xmax[i] = jmax(xmax[i], v[k][i]); }
}
template <class T> void cell_limits(const Mat<T, 2>& m, T* xmin, T* xmax) {
  T a[2] = {m.a[0][0], m.a[1][0]};
  T b[2] = {m.a[0][1], m.a[1][1]};
  T v[4][2];
  for (int i = 0; i < 2; i++) { v[0][i] = 0; v[1][i] = a[i]; v[2][i] = a[i] + b[i]; v[3][i] = b[i]; }
  for (int i = 0; i < 2; i++) { xmin[i] = v[0][i]; xmax[i] = v[0][i]; }
  for (int k = 1; k < 4; k++)
    for (int i = 0; i < 2; i++) { xmin[i] = jmin(xmin[i], v[k][i]); xmax[i] = jmax(xmax[i], v[k][i]); }
}

template <class T, int N> struct Box {
  int kind = 0, lcell = 1;
  Mat<T, N> Min, Mal, R, Rinv;
  int64_t nc[N];
  T cutoff, cutoff_sqr;
  T cbmin[N], cbmax[N], cs[N], origin[N];
  T det_in;  // det of the input cell, used by the wrap solve
  int64_t ncells() const {
    int64_t p = 1;
    for (int i = 0; i < N; i++) p *= nc[i];
    return p;
  }
};

template <class T, int N>
int make_box(const orc_spec* s, const T* x, int64_t nx, const T* y, int64_t ny, Box<T, N>& B) {
  if (s->lcell < 1) return ERR_LCELL;
  B.kind = s->kind;
  B.lcell = s->lcell;
  B.cutoff = (T)s->cutoff;
  for (int i = 0; i < N; i++) B.origin[i] = 0;
  if (s->kind == KIND_NONPER) {
    // limits(x[,y]) (CellOperations.jl:262-324) -> Box(Limits) (Box.jl:374-377)
    T mn[N], mx[N];
    for (int i = 0; i < N; i++) { mn[i] = std::numeric_limits<T>::max(); mx[i] = -std::numeric_limits<T>::max(); }
    bool any = false;
    auto upd = [&](const T* v, int64_t n) {
      for (int64_t p = 0; p < n; p++) {
        any = true;
        for (int i = 0; i < N; i++) { mn[i] = jmin(mn[i], v[p * N + i]); mx[i] = jmax(mx[i], v[p * N + i]); }
      }
    };
    // Julia: xmin starts at typemax (Inf) and xmax at typemin (-Inf); with at
    // least one particle the result is the same as starting from +/-max.
    upd(x, nx);
    T ymn[N], ymx[N];
    if (y) {
      T xmn[N], xmx[N];
      for (int i = 0; i < N; i++) { xmn[i] = mn[i]; xmx[i] = mx[i]; }
      for (int i = 0; i < N; i++) { mn[i] = std::numeric_limits<T>::max(); mx[i] = -std::numeric_limits<T>::max(); }
      bool anyx = any;
      any = false;
      upd(y, ny);
      bool anyy = any;
      for (int i = 0; i < N; i++) {
        ymn[i] = anyy ? mn[i] : T(0); ymx[i] = anyy ? mx[i] : T(0);
        T a0 = anyx ? xmn[i] : T(0), a1 = anyx ? xmx[i] : T(0);
        mn[i] = jmin(a0, ymn[i]);
        mx[i] = jmax(a1, ymx[i]);
      }
    } else if (!any) {
      for (int i = 0; i < N; i++) { mn[i] = 0; mx[i] = 0; }
    }
    T pad = (T(210) * B.cutoff) / T(100);
    for (int i = 0; i < N; i++)
      for (int j = 0; j < N; j++) B.Min.a[i][j] = (i == j) ? ((mx[i] - mn[i]) + pad) : T(0);
    for (int i = 0; i < N; i++) B.origin[i] = mn[i];
  } else {
    for (int i = 0; i < N; i++)
      for (int j = 0; j < N; j++) B.Min.a[i][j] = (T)s->M[j * N + i];
  }
  if (s->kind == KIND_TRI) {
    align(B.Min, B.Mal, B.R);
  } else {
    B.Mal = B.Min;
    B.R = eye<T, N>();
  }
  if (!check_cell(B.Mal, B.cutoff)) return ERR_CELL_TOO_SMALL;
  T xmin[N], xmax[N];
  cell_limits(B.Mal, xmin, xmax);
  T cl = B.cutoff / T(B.lcell);
  for (int i = 0; i < N; i++) {
    T q = (xmax[i] - xmin[i]) / cl;
    int64_t n0;
    if (s->kind == KIND_TRI) {
      n0 = (int64_t)std::ceil(q);
      B.cs[i] = cl;
    } else {
      n0 = (int64_t)std::floor(q);
      B.cs[i] = (xmax[i] - xmin[i]) / T(n0);
    }
    B.nc[i] = n0 + 2 * B.lcell + 1;
    T lc = T(B.lcell) * B.cs[i];
    B.cbmin[i] = (xmin[i] + B.origin[i]) - lc;
    B.cbmax[i] = (xmax[i] + B.origin[i]) + lc;
  }
  B.cutoff_sqr = B.cutoff * B.cutoff;
  B.Rinv = inv(B.R);
  B.det_in = det(B.Min);
  return ERR_OK;
}

template <class T, int N> struct Particle {
  int64_t index;
  bool real;
  T x[N];
};

// Read-only view of the particles of one cell.
template <class P> struct Span {
  const P* b = nullptr;
  int64_t n = 0;
  const P* begin() const { return b; }
  const P* end() const { return b + n; }
  size_t size() const { return (size_t)n; }
  bool empty() const { return n == 0; }
  const P& operator[](int64_t i) const { return b[i]; }
};

// The cell list in one flat array: the copies of cell c (linear index, x fastest) are
// parts[start[c] .. start[c+1]), in the order the reference's serial build appends them
// (particle index order; a particle's real copy, then its images in image order).
template <class T, int N> struct CellList {
  const Box<T, N>* box;
  int64_t n_real = 0, n_particles = 0;
  std::vector<Particle<T, N>> parts;
  std::vector<int64_t> start;                // ncells + 1
  std::vector<int64_t> real_cells;           // linear indices of the cells holding real particles, ascending
  Span<Particle<T, N>> cell(int64_t li) const {
    Span<Particle<T, N>> sp;
    sp.b = parts.data() + start[(size_t)li];
    sp.n = start[(size_t)li + 1] - start[(size_t)li];
    return sp;
  }
};

template <class T, int N> inline void wrap_to_first(const Box<T, N>& B, const T* x, T* out) {
  T p[N];
  solve(B.Min, B.det_in, x, p);
  for (int i = 0; i < N; i++) {
    p[i] = p[i] - std::floor(p[i]);
    if (p[i] == T(1)) p[i] = T(0);
  }
  T w[N];
  matvec(B.Min, p, w);
  matvec(B.R, w, out);
}

template <class T, int N> inline void particle_cell(const Box<T, N>& B, const T* x, int64_t* c) {
  for (int i = 0; i < N; i++) c[i] = (int64_t)std::floor((x[i] - B.cbmin[i]) / B.cs[i]) + 1;
}

template <class T, int N> inline int64_t linear_index(const Box<T, N>& B, const int64_t* c) {
  int64_t li = 0;
  for (int i = N - 1; i >= 0; i--) li = li * B.nc[i] + (c[i] - 1);
  return li;
}

template <class T, int N> inline void cell_center(const Box<T, N>& B, const int64_t* c, T* ctr) {
  for (int i = 0; i < N; i++) ctr[i] = (B.cbmin[i] + B.cs[i] * T(c[i])) - B.cs[i] / T(2);
}

template <class T, int N> void cart_from_linear(const Box<T, N>& B, int64_t li, int64_t* c) {
  for (int i = 0; i < N; i++) { c[i] = li % B.nc[i] + 1; li /= B.nc[i]; }
}

// Cell of a copy: particle_cell (Box.jl:499-508) with real_particle_border_case (CellLists.jl:956-967)
// for real copies.
template <class T, int N> inline int64_t copy_cell(const Box<T, N>& B, const T* x, bool real) {
  int64_t c[N];
  particle_cell(B, x, c);
  if (real) {
    for (int i = 0; i < N; i++) {
      if (c[i] == B.lcell) c[i] += 1;
      if (c[i] == B.nc[i] - B.lcell + 1) c[i] -= 1;
    }
  }
  return linear_index(B, c);
}

template <class T, int N> inline bool in_computing_box(const Box<T, N>& B, const T* x) {
  for (int i = 0; i < N; i++)
    if (!(B.cbmin[i] <= x[i] && x[i] < B.cbmax[i])) return false;
  return true;
}

// UpdateCellList! (CellLists.jl:727-927, 940-1057): the copies of every particle (wrap_to_first, then
// replicate_particle! over Iterators.product(-1:1, ...) with the first index fastest) are generated in
// parallel into particle order, then placed by a stable counting sort on the cell, which reproduces the
// serial append order of the reference inside every cell.
template <class T, int N>
void build(CellList<T, N>& cl, const Box<T, N>& B, const T* x, int64_t n, int nthreads = 1) {
  cl.box = &B;
  cl.n_real = n;
  const int64_t ncells = B.ncells();
  int nimg = 1;
  for (int i = 0; i < N; i++) nimg *= 3;
  const int zero = (nimg - 1) / 2;
  T shift[27][N];
  for (int k = 0; k < nimg; k++) {
    int sv[N];
    int kk = k;
    for (int i = 0; i < N; i++) { sv[i] = kk % 3 - 1; kk /= 3; }
    for (int i = 0; i < N; i++) {
      T acc = B.Mal.a[i][0] * T(sv[0]);
      for (int j = 1; j < N; j++) acc = acc + B.Mal.a[i][j] * T(sv[j]);
      shift[k][i] = acc;
    }
  }
  const bool nonper = (B.kind == KIND_NONPER);
  std::vector<T> w((size_t)(n * N));
  std::vector<uint32_t> mask((size_t)n);
  std::vector<int64_t> off((size_t)n + 1, 0);
  int nth = nthreads > 0 ? nthreads : 1;
#ifndef _OPENMP
  nth = 1;
#endif
#ifdef _OPENMP
#pragma omp parallel for num_threads(nth) schedule(static)
#endif
  for (int64_t ip = 0; ip < n; ip++) {
    T* p = w.data() + ip * N;
    if (nonper) {
      for (int i = 0; i < N; i++) p[i] = x[ip * N + i];
      mask[(size_t)ip] = 0;
      off[(size_t)ip + 1] = 1;
      continue;
    }
    wrap_to_first(B, x + ip * N, p);
    uint32_t m = 0;
    int cnt = 1;
    for (int k = 0; k < nimg; k++) {
      if (k == zero) continue;
      T g[N];
      for (int i = 0; i < N; i++) g[i] = p[i] + shift[k][i];
      if (in_computing_box(B, g)) { m |= 1u << k; cnt++; }
    }
    mask[(size_t)ip] = m;
    off[(size_t)ip + 1] = cnt;
  }
  for (int64_t ip = 0; ip < n; ip++) off[(size_t)ip + 1] += off[(size_t)ip];
  const int64_t nc = off[(size_t)n];
  std::vector<Particle<T, N>> tmp((size_t)nc);
  std::vector<int64_t> cellof((size_t)nc);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nth) schedule(static)
#endif
  for (int64_t ip = 0; ip < n; ip++) {
    const T* p = w.data() + ip * N;
    int64_t at = off[(size_t)ip];
    Particle<T, N>& r = tmp[(size_t)at];
    r.index = ip;
    r.real = true;
    for (int i = 0; i < N; i++) r.x[i] = p[i];
    cellof[(size_t)at] = copy_cell(B, p, true);
    at++;
    uint32_t m = mask[(size_t)ip];
    for (int k = 0; k < nimg; k++) {
      if (!(m & (1u << k))) continue;
      Particle<T, N>& q = tmp[(size_t)at];
      q.index = ip;
      q.real = false;
      for (int i = 0; i < N; i++) q.x[i] = p[i] + shift[k][i];
      cellof[(size_t)at] = copy_cell(B, q.x, false);
      at++;
    }
  }
  // stable counting sort by cell
  cl.start.assign((size_t)ncells + 1, 0);
  std::vector<char> has_real((size_t)ncells, 0);
  for (int64_t t = 0; t < nc; t++) {
    cl.start[(size_t)cellof[(size_t)t] + 1]++;
    if (tmp[(size_t)t].real) has_real[(size_t)cellof[(size_t)t]] = 1;
  }
  for (int64_t c = 0; c < ncells; c++) cl.start[(size_t)c + 1] += cl.start[(size_t)c];
  std::vector<int64_t> fill(cl.start.begin(), cl.start.end() - 1);
  cl.parts.resize((size_t)nc);
  for (int64_t t = 0; t < nc; t++) cl.parts[(size_t)fill[(size_t)cellof[(size_t)t]]++] = tmp[(size_t)t];
  cl.n_particles = nc;
  cl.real_cells.clear();
  for (int64_t c = 0; c < ncells; c++)
    if (has_real[(size_t)c]) cl.real_cells.push_back(c);
}

// ----------------------------------------------------------------------------
// Operators.  Pair values are evaluated in double from the T-precision pair
// (for T = double this is the reference's own arithmetic).
// ----------------------------------------------------------------------------
struct Acc {  // Neumaier-compensated or plain double accumulator
  double s = 0, c = 0;
  bool comp = true;
  inline void add(double v) {
    if (!comp) { s += v; return; }
    double t = s + v;
    if (std::fabs(s) >= std::fabs(v)) c += (s - t) + v; else c += (v - t) + s;
    s = t;
  }
  double value() const { return s + c; }
};

// Per-thread force sums: compensated accumulators, or plain doubles (the reference's per-batch output
// copies) when compensation is off.
struct FSum {
  bool comp = true;
  std::vector<Acc> a;
  std::vector<double> p;
  void assign(size_t n, bool c) {
    comp = c;
    if (c) {
      Acc z;
      a.assign(n, z);
      p.clear();
    } else {
      p.assign(n, 0.0);
      a.clear();
    }
  }
  inline void add(size_t q, double v) {
    if (comp) a[q].add(v);
    else p[q] += v;
  }
  double value(size_t q) const { return comp ? a[q].value() : p[q]; }
  bool empty() const { return a.empty() && p.empty(); }
};

struct Local {
  bool used = false;  // set by the thread that owns it
  std::vector<int64_t> ni, nj;
  std::vector<double> nd;
  Acc energy;
  int64_t count = 0;
  FSum fx, fy;   // per particle per component
  double min_d = std::numeric_limits<double>::infinity();
  int64_t min_i = -1, min_j = -1;
  std::vector<int64_t> hc;
  std::vector<Acc> hs;
  Acc adj[15];
};

template <class T, int N> struct OpCtx {
  const orc_op* op;
  bool cross;
  int64_t nx, ny;
  T bins_T[1024];
};

template <class T, int N>
__attribute__((always_inline)) inline void apply_op(const OpCtx<T, N>& ctx, Local& L, int64_t i, int64_t j, const T* xi, const T* xj, T d2,
                     const Mat<T, N>* rinv = nullptr) {
  const orc_op* op = ctx.op;
  const int code = op->op;
  if (code == OP_COUNT) { L.count++; return; }
  if (code == OP_NL) {
    L.ni.push_back(i); L.nj.push_back(j); L.nd.push_back((double)std::sqrt(d2));
    return;
  }
  double dv[N];
  for (int k = 0; k < N; k++) dv[k] = (double)xi[k] - (double)xj[k];
  double dd2;
  if (sizeof(T) == sizeof(double)) dd2 = (double)d2;
  else { dd2 = dv[0] * dv[0]; for (int k = 1; k < N; k++) dd2 = dd2 + dv[k] * dv[k]; }
  if (rinv) {
    double r[N];
    for (int a = 0; a < N; a++) {
      double acc = 0;
      for (int k = 0; k < N; k++) acc += (double)rinv->a[a][k] * dv[k];
      r[a] = acc;
    }
    for (int a = 0; a < N; a++) dv[a] = r[a];
  }
  double dd = std::sqrt(dd2);
  switch (code) {
    case OP_SUM_D2: L.energy.add(dd2); break;
    case OP_SUM_D: L.energy.add(dd); break;
    case OP_SUM_INV_D: L.energy.add(1.0 / dd); break;
    case OP_MINDIST: {
      double dT = (double)std::sqrt(d2);
      if (dT < L.min_d) { L.min_d = dT; L.min_i = i; L.min_j = j; }
      break;
    }
    case OP_SOFT_ENERGY:
    case OP_SOFT_FORCES: {
      double c = op->p[0];
      double u = (c - dd) * (c - dd);
      L.energy.add(u);
      if (code == OP_SOFT_FORCES) {
        double dudr = -2.0 * (c - dd);
        double g = dudr / dd;
        for (int k = 0; k < N; k++) {
          double df = g * dv[k];
          L.fx.add((size_t)(i * N + k), -df);
          if (ctx.cross) L.fy.add((size_t)(j * N + k), df); else L.fx.add((size_t)(j * N + k), df);
        }
      }
      break;
    }
    case OP_LJ_ENERGY:
    case OP_LJ_FORCES:
    case OP_LJ_ADJOINT: {
      double eps = op->p[0], sig = op->p[1];
      if (op->ntypes > 0) {
        int ti = op->types_x[i];
        int tj = ctx.cross ? op->types_y[j] : op->types_x[j];
        eps = op->eps_table[ti * op->ntypes + tj];
        sig = op->sig_table[ti * op->ntypes + tj];
      }
      double c12 = op->p[2], c6 = op->p[3];
      double sr2 = (sig * sig) / dd2;
      double sr6 = sr2 * sr2 * sr2;
      double sr12 = sr6 * sr6;
      L.energy.add(eps * (c12 * sr12 - c6 * sr6));
      if (code == OP_LJ_ADJOINT) {
        // adjoint of U: virial W = sum g dx dx^T with g = u'(r)/r; dU/deps and dU/dsigma per type pair
        double g = eps * (-12.0 * c12 * sr12 + 6.0 * c6 * sr6) / dd2;
        for (int a = 0; a < N; a++)
          for (int b = 0; b < N; b++) L.adj[a * 3 + b].add(g * dv[a] * dv[b]);
        int cls = 0;
        if (op->ntypes > 0) {
          int ti = op->types_x[i];
          int tj = ctx.cross ? op->types_y[j] : op->types_x[j];
          int a = ti < tj ? ti : tj, b = ti < tj ? tj : ti;
          cls = a * op->ntypes - a * (a - 1) / 2 + (b - a);  // upper triangle, row-major
        }
        L.adj[9 + cls].add(c12 * sr12 - c6 * sr6);
        L.adj[12 + cls].add(eps * (12.0 * c12 * sr12 - 6.0 * c6 * sr6) / sig);
      }
      if (code == OP_LJ_FORCES || code == OP_LJ_ADJOINT) {
        double g = eps * (-12.0 * c12 * sr12 + 6.0 * c6 * sr6) / dd2;  // (du/dr)/r
        for (int k = 0; k < N; k++) {
          double df = g * dv[k];
          L.fx.add((size_t)(i * N + k), -df);
          if (ctx.cross) L.fy.add((size_t)(j * N + k), df); else L.fx.add((size_t)(j * N + k), df);
        }
      }
      break;
    }
    case OP_WEIGHTED_INV_D: {
      // u -= c w_i w_j / d (test/examples/gravitational_potential.jl:30-33, c = 9.8, w = mass);
      // df = ((c w_i w_j) / d2 / d) (x - y), f[i] -= df, f[j] += df (gravitational_force.jl:37-46)
      const double wi = op->weights_x[i];
      const double wj = ctx.cross ? op->weights_y[j] : op->weights_x[j];
      const double cw = op->p[0] * wi * wj;
      L.energy.add(-(cw / dd));
      const double g = cw / dd2 / dd;
      for (int k = 0; k < N; k++) {
        double df = g * dv[k];
        L.fx.add((size_t)(i * N + k), -df);
        if (ctx.cross) L.fy.add((size_t)(j * N + k), df); else L.fx.add((size_t)(j * N + k), df);
      }
      break;
    }
    case OP_INV_D_FORCES: {
      // energy += 1/d; forces accumulate the gradient (single_set_compound.md:79-86)
      L.energy.add(1.0 / dd);
      double g = 1.0 / dd2 / dd;
      for (int k = 0; k < N; k++) {
        double df = g * (-dv[k]);  // (1/d2)*(1/d)*(y - x)
        L.fx.add((size_t)(i * N + k), df);
        if (ctx.cross) L.fy.add((size_t)(j * N + k), -df); else L.fx.add((size_t)(j * N + k), -df);
      }
      break;
    }
    case OP_RHIST: {
      T r = std::sqrt(d2);
      int nb = op->nbins;
      // searchsortedfirst(bins, r) - 1 (1-based) -> 0-based bin = first e with bins[e] >= r, minus 1
      int e = (int)(std::lower_bound(ctx.bins_T, ctx.bins_T + nb + 1, r) - ctx.bins_T);
      int b = e - 1;
      if (b < 0 || b >= nb) break;
      L.hc[b]++;
      const double* vx = op->vel_x;
      const double* vy = ctx.cross ? op->vel_y : op->vel_x;
      double dot = 0;
      for (int k = 0; k < N; k++) {
        double dvv = vx[i * N + k] - vy[j * N + k];
        dot = (k == 0) ? dvv * dv[k] : dot + dvv * dv[k];
      }
      L.hs[b].add(dot / (double)r);
      break;
    }
    default: break;
  }
}

// ----------------------------------------------------------------------------
// Map (serial structure of self.jl / cross.jl / vicinal_cells.jl)
// ----------------------------------------------------------------------------
// Per-thread scratch: the projected particles of a vicinal cell (project_particles!), the candidates'
// coordinates as separate arrays, one row of squared distances, pass flags and the passing positions.
// The inner loops first compute the squared distances of one particle to all its candidates and the
// tests in a branch-free pass (each d2 is computed exactly as dist2 computes it), then visit the
// candidates that passed every test in their original order: the pairs found, their order and their d2
// are those of the plain loop.
template <class T, int N> struct Scratch {
  std::vector<Particle<T, N>> pp;
  std::vector<T> ppx;
  std::vector<T> c[N];
  std::vector<T> d2;
  std::vector<unsigned char> ok;
  std::vector<int32_t> sel;
  void coords_of(const Particle<T, N>* p, int64_t n) {
    for (int k = 0; k < N; k++) c[k].resize((size_t)n);
    for (int64_t q = 0; q < n; q++)
      for (int k = 0; k < N; k++) c[k][(size_t)q] = p[q].x[k];
    if ((int64_t)d2.size() < n) {
      d2.resize((size_t)n);
      ok.resize((size_t)n);
      sel.resize((size_t)n);
    }
  }
};

// d2 of x to the candidates q in [q0, q1) (coordinates by component), same operation order as dist2
template <class T, int N>
inline void d2_row(const T* x, const std::vector<T>* c, int64_t q0, int64_t q1, T* out) {
  const T x0 = x[0];
  const T* c0 = c[0].data();
  for (int64_t q = q0; q < q1; q++) out[q] = (x0 - c0[q]) * (x0 - c0[q]);
  for (int k = 1; k < N; k++) {
    const T xk = x[k];
    const T* ck = c[k].data();
    for (int64_t q = q0; q < q1; q++) out[q] = out[q] + (xk - ck[q]) * (xk - ck[q]);
  }
}

template <class T, int N> struct Mapper {
  const Box<T, N>& B;
  const OpCtx<T, N>& ctx;
  bool tri, nonper;
  Mapper(const Box<T, N>& b, const OpCtx<T, N>& c) : B(b), ctx(c) {
    tri = (B.kind == KIND_TRI);
    nonper = (B.kind == KIND_NONPER);
  }

  // Pair values are evaluated in double: for triclinic cells the difference of the
  // (rotated) copies is rotated back with the inverse rotation in double, so that
  // Float32 inputs are checked against an FP64 evaluation rather than against the
  // Float32 rotation of pair.x/pair.y (self.jl:178).
  inline void emit(Local& L, const Particle<T, N>& pi, const Particle<T, N>& pj, T d2) const {
    apply_op(ctx, L, pi.index, pj.index, pi.x, pj.x, d2, tri ? &B.Rinv : nullptr);
  }

  static inline T dist2(const T* a, const T* b) {
    T s = (a[0] - b[0]) * (a[0] - b[0]);
    for (int k = 1; k < N; k++) s = s + (a[k] - b[k]) * (a[k] - b[k]);
    return s;
  }

  // same-cell, self
  void current_self(Local& L, const Span<Particle<T, N>>& cell, Scratch<T, N>& S) const {
    const int64_t n = (int64_t)cell.size();
    S.coords_of(cell.b, n);
    T* d2 = S.d2.data();
    if (!tri) {
      for (int64_t a = 0; a + 1 < n; a++) {
        const auto& pi = cell[a];
        d2_row<T, N>(pi.x, S.c, a + 1, n, d2);
        for (int64_t b = a + 1; b < n; b++) {
          if (!(d2[b] <= B.cutoff_sqr)) continue;
          const auto& pj = cell[b];
          if (!nonper && !(pi.real || pj.real)) continue;
          emit(L, pi, pj, d2[b]);
        }
      }
    } else {
      for (int64_t a = 0; a < n; a++) {
        const auto& pi = cell[a];
        if (!pi.real) continue;
        d2_row<T, N>(pi.x, S.c, 0, n, d2);
        for (int64_t b = 0; b < n; b++) {
          if (!(d2[b] <= B.cutoff_sqr)) continue;
          const auto& pj = cell[b];
          if (pi.index >= pj.index) continue;
          emit(L, pi, pj, d2[b]);
        }
      }
    }
  }

  // same-cell, cross
  void current_cross(Local& L, const Span<Particle<T, N>>& ci, const Span<Particle<T, N>>& cj,
                     Scratch<T, N>& S) const {
    const int64_t n = (int64_t)cj.size();
    S.coords_of(cj.b, n);
    T* d2 = S.d2.data();
    for (const auto& pi : ci) {
      if (!nonper && !pi.real) continue;
      d2_row<T, N>(pi.x, S.c, 0, n, d2);
      for (int64_t b = 0; b < n; b++)
        if (d2[b] <= B.cutoff_sqr) emit(L, pi, cj[b], d2[b]);
    }
  }

  // vicinal cells with projection culling; skip = index rule for triclinic self
  void vicinal(Local& L, const Span<Particle<T, N>>& ci, const int64_t* cci, const Span<Particle<T, N>>& cj,
               const int64_t* ccj, bool skip, Scratch<T, N>& S) const {
    std::vector<Particle<T, N>>& pp = S.pp;
    std::vector<T>& ppx = S.ppx;
    T ctr_i[N], ctr_j[N], dc[N];
    cell_center(B, cci, ctr_i);
    cell_center(B, ccj, ctr_j);
    for (int k = 0; k < N; k++) dc[k] = ctr_j[k] - ctr_i[k];
    T dcn = snorm<T, N>(dc);
    for (int k = 0; k < N; k++) dc[k] = dc[k] / dcn;
    // project_particles! (auxiliary_functions.jl:66-111)
    double margin_d;
    T margin_T;
    bool margin_is_T = (B.lcell == 1);
    if (margin_is_T) margin_T = B.cutoff + dcn / T(2);
    else margin_d = (double)B.cutoff * (1.0 + std::sqrt((double)N) / 2.0);
    pp.clear();
    ppx.clear();
    for (const auto& pj : cj) {
      T v[N];
      for (int k = 0; k < N; k++) v[k] = pj.x[k] - ctr_i[k];
      T xp = dotN<T, N>(v, dc);
      bool keep = margin_is_T ? (std::fabs(xp) <= margin_T) : ((double)std::fabs(xp) <= margin_d);
      if (keep) { pp.push_back(pj); ppx.push_back(xp); }
    }
    if (pp.empty()) return;
    const int64_t np = (int64_t)pp.size();
    S.coords_of(pp.data(), np);
    T* d2 = S.d2.data();
    unsigned char* ok = S.ok.data();
    const T* px = ppx.data();
    for (const auto& pi : ci) {
      if (tri && !pi.real) continue;
      T v[N];
      for (int k = 0; k < N; k++) v[k] = pi.x[k] - ctr_i[k];
      T xpi = dotN<T, N>(v, dc);
      // d2 (as dist2 computes it), partition! (|xproj_j - xproj_i| <= cutoff) and the cutoff test, in one
      // branch-free pass
      const T* c0 = S.c[0].data();
      const T* c1 = S.c[1].data();
      const T* c2 = S.c[N - 1].data();
      const T x0 = pi.x[0], x1 = pi.x[1], x2 = pi.x[N - 1];
      const T cut = B.cutoff, cut2 = B.cutoff_sqr;
      for (int64_t q = 0; q < np; q++) {
        T e = (x0 - c0[q]) * (x0 - c0[q]);
        e = e + (x1 - c1[q]) * (x1 - c1[q]);
        if (N == 3) e = e + (x2 - c2[q]) * (x2 - c2[q]);
        d2[q] = e;
        ok[q] = (unsigned char)((std::fabs(px[q] - xpi) <= cut) & (e <= cut2));
      }
      // the candidates that passed, in their order (branch-free compaction)
      int32_t* sel = S.sel.data();
      int64_t m = 0;
      for (int64_t q = 0; q < np; q++) {
        sel[m] = (int32_t)q;
        m += ok[q];
      }
      for (int64_t t = 0; t < m; t++) {
        const int64_t q = sel[t];
        const auto& pj = pp[(size_t)q];
        if (tri) {
          if (skip && pi.index >= pj.index) continue;
        } else if (!nonper) {
          if (!(pi.real || pj.real)) continue;
        }
        emit(L, pi, pj, d2[q]);
      }
    }
  }
};

template <class T, int N> void stencil(const Box<T, N>& B, bool forward, std::vector<std::array<int64_t, 3>>& out) {
  out.clear();
  int64_t l = B.lcell;
  if (forward) {
    if (N == 3) {
      for (int64_t z = -l; z <= l; z++)
        for (int64_t y = -l; y <= l; y++)
          for (int64_t x = 1; x <= l; x++) out.push_back({x, y, z});
      for (int64_t z = -l; z <= l; z++)
        for (int64_t y = 1; y <= l; y++) out.push_back({0, y, z});
      for (int64_t z = 1; z <= l; z++) out.push_back({0, 0, z});
    } else {
      for (int64_t y = -l; y <= l; y++)
        for (int64_t x = 1; x <= l; x++) out.push_back({x, y, 0});
      for (int64_t y = 1; y <= l; y++) out.push_back({0, y, 0});
    }
  } else {
    int64_t zl = (N == 3) ? l : 0;
    for (int64_t z = -zl; z <= zl; z++)
      for (int64_t y = -l; y <= l; y++)
        for (int64_t x = -l; x <= l; x++) {
          if (x == 0 && y == 0 && z == 0) continue;
          out.push_back({x, y, z});
        }
  }
}

template <class T, int N> void alloc_local(Local& L, const orc_op* op, int64_t nx, int64_t ny, bool cross) {
  L.energy.comp = op->compensated != 0;
  for (auto& a : L.adj) a.comp = op->compensated != 0;
  if (op->op == OP_SOFT_FORCES || op->op == OP_LJ_FORCES || op->op == OP_INV_D_FORCES || op->op == OP_LJ_ADJOINT ||
      op->op == OP_WEIGHTED_INV_D) {
    L.fx.assign((size_t)(nx * N), op->compensated != 0);
    if (cross) L.fy.assign((size_t)(ny * N), op->compensated != 0);
  }
  if (op->op == OP_RHIST) {
    Acc z; z.comp = op->compensated != 0;
    L.hc.assign((size_t)op->nbins, 0);
    L.hs.assign((size_t)op->nbins, z);
  }
}

template <class T, int N>
int run_map(const orc_spec* s, const T* x, int64_t nx, const T* y, int64_t ny, const orc_op* op, orc_result* res) {
  for (int64_t i = 0; i < nx * N; i++) if (std::isnan(x[i])) return ERR_NAN;
  if (y) for (int64_t i = 0; i < ny * N; i++) if (std::isnan(y[i])) return ERR_NAN;
  Box<T, N> B;
  int st = make_box<T, N>(s, x, nx, y, ny, B);
  if (st) return st;
  const bool cross = (y != nullptr);
  CellList<T, N> clx, cly;
  build(clx, B, x, nx, op->nthreads);
  if (cross) build(cly, B, y, ny, op->nthreads);
  OpCtx<T, N> ctx;
  ctx.op = op;
  ctx.cross = cross;
  ctx.nx = nx;
  ctx.ny = ny;
  if (op->op == OP_RHIST) {
    if (op->nbins < 1 || op->nbins > 1000) return ERR_ARG;
    for (int b = 0; b <= op->nbins; b++) ctx.bins_T[b] = (T)op->bins[b];
  }
  Mapper<T, N> mp(B, ctx);
  std::vector<std::array<int64_t, 3>> st_fw, st_all;
  stencil(B, true, st_fw);
  stencil(B, false, st_all);
  const bool tri = (B.kind == KIND_TRI);
  int nth = op->nthreads > 0 ? op->nthreads : 1;
#ifndef _OPENMP
  nth = 1;
#endif
  std::vector<Local> locals((size_t)nth);
  const int64_t nreal = (int64_t)clx.real_cells.size();
#ifdef _OPENMP
#pragma omp parallel num_threads(nth)
#endif
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    Local& L = locals[(size_t)tid];
    alloc_local<T, N>(L, op, nx, ny, cross);  // each thread fills its own sums (in parallel)
    L.used = true;
    Scratch<T, N> scr;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 8)
#endif
    for (int64_t r = 0; r < nreal; r++) {
      const int64_t li = clx.real_cells[(size_t)r];
      const auto cell = clx.cell(li);
      int64_t cc[N];
      cart_from_linear(B, li, cc);
      if (!cross) {
        mp.current_self(L, cell, scr);
        const auto& sten = (tri ? st_all : st_fw);
        for (const auto& o : sten) {
          int64_t cj[N];
          for (int k = 0; k < N; k++) cj[k] = cc[k] + o[k];
          const auto other = clx.cell(linear_index(B, cj));
          if (other.empty()) continue;
          mp.vicinal(L, cell, cc, other, cj, true, scr);
        }
      } else {
        const auto same = cly.cell(li);
        if (!same.empty()) mp.current_cross(L, cell, same, scr);
        for (const auto& o : st_all) {
          int64_t cj[N];
          for (int k = 0; k < N; k++) cj[k] = cc[k] + o[k];
          const auto other = cly.cell(linear_index(B, cj));
          if (other.empty()) continue;
          mp.vicinal(L, cell, cc, other, cj, false, scr);
        }
      }
    }
  }
  // reduce_output!
  Acc e; e.comp = op->compensated != 0;
  int64_t cnt = 0;
  res->nl_n = 0;
  res->min_d = std::numeric_limits<double>::infinity();
  res->min_i = -1;
  res->min_j = -1;
  for (auto& L : locals) {
    e.add(L.energy.value());
    cnt += L.count;
    if (op->op == OP_NL) {
      for (size_t q = 0; q < L.ni.size(); q++) {
        if (res->nl_n < res->nl_cap) {
          res->nl_i[res->nl_n] = L.ni[q];
          res->nl_j[res->nl_n] = L.nj[q];
          res->nl_d[res->nl_n] = L.nd[q];
        }
        res->nl_n++;
      }
    }
    if (L.min_d <= res->min_d && L.min_i >= 0) {
      if (L.min_d < res->min_d || res->min_i < 0) { res->min_d = L.min_d; res->min_i = L.min_i; res->min_j = L.min_j; }
    }
  }
  res->scalar = e.value();
  res->count = cnt;
  for (int k = 0; k < 15; k++) {
    Acc a; a.comp = op->compensated != 0;
    for (auto& L : locals) a.add(L.adj[k].value());
    res->adj[k] = a.value();
  }
  std::vector<const Local*> used;
  for (auto& L : locals)
    if (L.used) used.push_back(&L);
  if (!used.empty() && !used[0]->fx.empty()) {
    // element-wise sum of the threads' copies in thread order (parallel over elements)
    const int64_t mx = nx * N, my = (cross && res->forces_y) ? ny * N : 0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nth) schedule(static)
#endif
    for (int64_t q = 0; q < mx + my; q++) {
      Acc a; a.comp = op->compensated != 0;
      if (q < mx) {
        for (const Local* L : used) a.add(L->fx.value((size_t)q));
        res->forces_x[q] = a.value();
      } else {
        for (const Local* L : used) a.add(L->fy.value((size_t)(q - mx)));
        res->forces_y[q - mx] = a.value();
      }
    }
  }
  if (op->op == OP_RHIST) {
    for (int b = 0; b < op->nbins; b++) {
      int64_t c = 0;
      Acc a; a.comp = op->compensated != 0;
      for (auto& L : locals) {
        if (!L.used) continue;
        c += L.hc[(size_t)b];
        a.add(L.hs[(size_t)b].value());
      }
      res->hist_count[b] = c;
      res->hist_sum[b] = a.value();
    }
  }
  if (op->op == OP_NL && res->nl_n > res->nl_cap) return ERR_CAPACITY;
  return ERR_OK;
}

// Naive O(N^2) minimum-image oracle (test/modules/Testing.jl:62-104)
template <class T> inline T jmod1(T x) {
  T r = std::fmod(x, T(1));
  if (r == 0) return std::copysign(r, T(1));
  if ((r > 0) != (T(1) > 0)) return r + T(1);
  return r;
}

template <class T, int N>
inline void wrap_relative(const Box<T, N>& B, const T* x, const T* xref, T* out) {
  T xf[N], rf[N];
  solve(B.Min, B.det_in, x, xf);
  solve(B.Min, B.det_in, xref, rf);
  for (int i = 0; i < N; i++) {
    xf[i] = xf[i] - std::floor(xf[i]); if (xf[i] == T(1)) xf[i] = 0;
    rf[i] = rf[i] - std::floor(rf[i]); if (rf[i] == T(1)) rf[i] = 0;
  }
  T xw[N];
  for (int i = 0; i < N; i++) {
    T w = jmod1(xf[i] - rf[i]);
    if (w >= T(1) / T(2)) w = w - T(1);
    xw[i] = w + rf[i];
  }
  T dlt[N], md[N];
  for (int i = 0; i < N; i++) dlt[i] = xw[i] - rf[i];
  matvec(B.Min, dlt, md);
  for (int i = 0; i < N; i++) out[i] = md[i] + xref[i];
}

template <class T, int N>
int run_naive(const orc_spec* s, const T* x, int64_t nx, const T* y, int64_t ny, const orc_op* op, orc_result* res) {
  Box<T, N> B;
  int st = make_box<T, N>(s, x, nx, y, ny, B);
  if (st) return st;
  const bool cross = (y != nullptr);
  OpCtx<T, N> ctx;
  ctx.op = op;
  ctx.cross = cross;
  ctx.nx = nx;
  ctx.ny = ny;
  if (op->op == OP_RHIST)
    for (int b = 0; b <= op->nbins; b++) ctx.bins_T[b] = (T)op->bins[b];
  Local L;
  alloc_local<T, N>(L, op, nx, ny, cross);
  for (int64_t i = 0; i < nx; i++) {
    const T* xi = x + i * N;
    int64_t j0 = cross ? 0 : i + 1;
    int64_t jn = cross ? ny : nx;
    for (int64_t j = j0; j < jn; j++) {
      const T* xj = (cross ? y : x) + j * N;
      T w[N];
      wrap_relative(B, xj, xi, w);
      T d2 = (xi[0] - w[0]) * (xi[0] - w[0]);
      for (int k = 1; k < N; k++) d2 = d2 + (xi[k] - w[k]) * (xi[k] - w[k]);
      if (d2 <= B.cutoff_sqr) apply_op(ctx, L, i, j, xi, w, d2);
    }
  }
  res->scalar = L.energy.value();
  res->count = L.count;
  for (int k = 0; k < 15; k++) res->adj[k] = L.adj[k].value();
  res->nl_n = (int64_t)L.ni.size();
  for (size_t q = 0; q < L.ni.size() && (int64_t)q < res->nl_cap; q++) {
    res->nl_i[q] = L.ni[q]; res->nl_j[q] = L.nj[q]; res->nl_d[q] = L.nd[q];
  }
  res->min_d = L.min_d; res->min_i = L.min_i; res->min_j = L.min_j;
  if (!L.fx.empty()) {
    for (int64_t q = 0; q < nx * N; q++) res->forces_x[q] = L.fx.value((size_t)q);
    if (cross && res->forces_y)
      for (int64_t q = 0; q < ny * N; q++) res->forces_y[q] = L.fy.value((size_t)q);
  }
  if (op->op == OP_RHIST)
    for (int b = 0; b < op->nbins; b++) { res->hist_count[b] = L.hc[(size_t)b]; res->hist_sum[b] = L.hs[(size_t)b].value(); }
  if (op->op == OP_NL && res->nl_n > res->nl_cap) return ERR_CAPACITY;
  return ERR_OK;
}

template <class T, int N>
int run_box(const orc_spec* s, const T* x, int64_t nx, const T* y, int64_t ny, orc_boxinfo* out) {
  Box<T, N> B;
  int st = make_box<T, N>(s, x, nx, y, ny, B);
  if (st) return st;
  std::memset(out, 0, sizeof(*out));
  for (int i = 0; i < N; i++) {
    out->nc[i] = B.nc[i];
    out->cell_size[i] = (double)B.cs[i];
    out->cbmin[i] = (double)B.cbmin[i];
    out->cbmax[i] = (double)B.cbmax[i];
    out->origin[i] = (double)B.origin[i];
    for (int j = 0; j < N; j++) {
      out->Min[j * N + i] = (double)B.Min.a[i][j];
      out->Mal[j * N + i] = (double)B.Mal.a[i][j];
      out->R[j * N + i] = (double)B.R.a[i][j];
      out->Rinv[j * N + i] = (double)B.Rinv.a[i][j];
    }
  }
  out->cutoff = (double)B.cutoff;
  out->cutoff_sqr = (double)B.cutoff_sqr;
  return ERR_OK;
}

template <class T, int N>
int run_celllist(const orc_spec* s, const T* x, int64_t n, int64_t* n_copies, int64_t* n_cells_real, int64_t cap,
                 int64_t* cell, int64_t* idx, int8_t* real, double* coords) {
  Box<T, N> B;
  int st = make_box<T, N>(s, x, n, nullptr, 0, B);
  if (st) return st;
  CellList<T, N> cl;
  build(cl, B, x, n, orc_max_threads_impl());
  *n_copies = cl.n_particles;
  *n_cells_real = (int64_t)cl.real_cells.size();
  if (!cell) return ERR_OK;
  if (cap < cl.n_particles) return ERR_CAPACITY;
  // cell linear-index order, particles in the reference's in-cell order
  const int64_t ncells = B.ncells();
  for (int64_t c = 0; c < ncells; c++) {
    for (int64_t k = cl.start[(size_t)c]; k < cl.start[(size_t)c + 1]; k++) {
      const auto& p = cl.parts[(size_t)k];
      cell[k] = c;
      idx[k] = p.index;
      real[k] = p.real ? 1 : 0;
      for (int d = 0; d < N; d++) coords[k * N + d] = (double)p.x[d];
    }
  }
  return ERR_OK;
}


template <class T, int N>
int box_tramp(const orc_spec* s, const void* x, int64_t nx, const void* y, int64_t ny, orc_boxinfo* out) {
  return run_box<T, N>(s, (const T*)x, nx, (const T*)y, ny, out);
}
template <class T, int N>
int map_tramp(const orc_spec* s, const void* x, int64_t nx, const void* y, int64_t ny, const orc_op* op, orc_result* r) {
  return run_map<T, N>(s, (const T*)x, nx, (const T*)y, ny, op, r);
}
template <class T, int N>
int naive_tramp(const orc_spec* s, const void* x, int64_t nx, const void* y, int64_t ny, const orc_op* op, orc_result* r) {
  return run_naive<T, N>(s, (const T*)x, nx, (const T*)y, ny, op, r);
}
template <class T, int N>
int cl_tramp(const orc_spec* s, const void* x, int64_t n, int64_t* nc, int64_t* ncr, int64_t cap, int64_t* cell,
                    int64_t* idx, int8_t* real, double* coords) {
  return run_celllist<T, N>(s, (const T*)x, n, nc, ncr, cap, cell, idx, real, coords);
}

}  // namespace

#define ORC_DISPATCH(FN, s, ...)                                                    \
  do {                                                                              \
    if (!(s) || ((s)->dim != 2 && (s)->dim != 3) || ((s)->dtype != 0 && (s)->dtype != 1)) return ERR_ARG; \
    if ((s)->dtype == 1) {                                                          \
      if ((s)->dim == 3) return FN<double, 3>(s, __VA_ARGS__);                      \
      return FN<double, 2>(s, __VA_ARGS__);                                         \
    } else {                                                                        \
      if ((s)->dim == 3) return FN<float, 3>(s, __VA_ARGS__);                       \
      return FN<float, 2>(s, __VA_ARGS__);                                          \
    }                                                                               \
  } while (0)

extern "C" {

int orc_box(const orc_spec* s, const void* x, int64_t nx, const void* y, int64_t ny, orc_boxinfo* out) {
  ORC_DISPATCH(box_tramp, s, x, nx, y, ny, out);
}

int orc_map(const orc_spec* s, const void* x, int64_t nx, const void* y, int64_t ny, const orc_op* op, orc_result* r) {
  ORC_DISPATCH(map_tramp, s, x, nx, y, ny, op, r);
}

int orc_naive(const orc_spec* s, const void* x, int64_t nx, const void* y, int64_t ny, const orc_op* op, orc_result* r) {
  ORC_DISPATCH(naive_tramp, s, x, nx, y, ny, op, r);
}

int orc_celllist(const orc_spec* s, const void* x, int64_t n, int64_t* n_copies, int64_t* n_cells_real, int64_t cap,
                 int64_t* cell, int64_t* idx, int8_t* real, double* coords) {
  ORC_DISPATCH(cl_tramp, s, x, n, n_copies, n_cells_real, cap, cell, idx, real, coords);
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
