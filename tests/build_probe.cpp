// Test infrastructure: runs the cell-list build steps of the library (csrc/clm_build_steps.cuh: the geometry
// copy the kernels receive, K1 wrap_count_at, K2 emit_at, K4 gather_at) on the host, one particle or copy at a
// time, so that the CPU tests can compare the copies, their cells and their coordinates with the oracle's
// serial cell list without a GPU.  The exclusive scan and the radix sort between the steps are replaced by
// their contracts (copy offsets in particle order; a stable sort of the copies by cell).  Built by
// tests/test_build_steps.py with g++ -ffp-contract=off, as the library's host code is.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

#include "clm_build_steps.cuh"

namespace {
template <class T, int N>
int run(int kind, const double* Mcol, double cutoff, int lcell, const double* xin, int n, int64_t cap,
        int64_t* n_copies, int64_t* n_real_cells, int64_t* cell, int64_t* idx, int8_t* real, double* coords,
        int* err_out) {
  std::vector<T> x((size_t)n * N), wrapped((size_t)n * N);
  for (size_t k = 0; k < x.size(); k++) x[k] = (T)xin[k];
  T M[3][3] = {}, origin[3] = {0, 0, 0};
  if (kind == clm::NONPERIODIC) {
    // the limits box of the particles, as the library's set_limits + nonperiodic_cell make it
    T lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int i = 0; i < n; i++)
      for (int k = 0; k < N; k++) {
        const T v = x[(size_t)i * N + k];
        lo[k] = i ? clm::geo::jmin(lo[k], v) : v;
        hi[k] = i ? clm::geo::jmax(hi[k], v) : v;
      }
    clm::nonperiodic_cell<T>(N, lo, hi, (T)cutoff, M, origin);
  } else {
    for (int i = 0; i < N; i++)
      for (int j = 0; j < N; j++) {
        T v = (T)Mcol[j * N + i];
        if (kind == clm::ORTHO && i != j) v = 0;
        M[i][j] = v;
      }
  }
  clm::Geometry<T> g;
  const int st = clm::make_geometry<T>(g, N, kind, M, (T)cutoff, lcell, kind == clm::NONPERIODIC ? origin : nullptr);
  if (st) return st;
  clm::DevGeom<T> d;
  clm::fill_devgeom<T>(g, 1, d);
  std::vector<uint32_t> mask((size_t)n);
  std::vector<int> ncopy((size_t)n), off((size_t)n + 1, 0);
  int err = 0;
  for (int i = 0; i < n; i++)
    if (!clm::wrap_count_at<T, N>(d, x.data(), i, wrapped.data(), mask.data(), ncopy.data())) err |= clm::DERR_NAN;
  for (int i = 0; i < n; i++) off[(size_t)i + 1] = off[(size_t)i] + ncopy[(size_t)i];
  const int total = off[(size_t)n];
  std::vector<uint32_t> keys((size_t)total), vals((size_t)total);
  for (int i = 0; i < n; i++)
    clm::emit_at<T, N>(d, 0, wrapped.data(), mask.data(), ncopy.data(), off.data(), i, total, keys.data(),
                       vals.data(), &err);
  // the radix sort's contract: copies ordered by cell, stable (particle order inside a cell)
  std::vector<int> perm((size_t)total);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return keys[(size_t)a] < keys[(size_t)b]; });
  std::vector<uint32_t> skeys((size_t)total), svals((size_t)total);
  for (int t = 0; t < total; t++) {
    skeys[(size_t)t] = keys[(size_t)perm[(size_t)t]];
    svals[(size_t)t] = vals[(size_t)perm[(size_t)t]];
  }
  const int ncells = d.ncells;
  std::vector<T> px((size_t)total + 1), py((size_t)total + 1), pz((size_t)total + 1);
  std::vector<float4> foff((size_t)total + 1), xq((size_t)total + 1);
  std::vector<int> code((size_t)total + 1), flags((size_t)ncells + 1, 0), start((size_t)ncells + 1, -1);
  for (int t = 0; t <= total; t++) {
    clm::cell_starts_at(skeys.data(), t, total, ncells, start.data());
    if (t == total) break;
    const int p = (int)(svals[(size_t)t] >> 5), k = (int)(svals[(size_t)t] & 31u);
    clm::gather_at<T, N>(d, wrapped.data(), t, p, k, (int)skeys[(size_t)t], px.data(), py.data(), pz.data(),
                         foff.data(), xq.data(), code.data(), flags.data(), 0);
  }
  *err_out = err;
  *n_copies = total;
  *n_real_cells = 0;
  for (int c = 0; c < ncells; c++) *n_real_cells += flags[(size_t)c] ? 1 : 0;
  // cell_start must bracket each cell's copies
  for (int c = 0; c < ncells; c++)
    if (start[(size_t)c] < 0 || start[(size_t)c] > start[(size_t)c + 1]) return 99;
  for (int t = 0; t < total; t++)
    if (start[skeys[(size_t)t]] > t || start[skeys[(size_t)t] + 1] <= t) return 98;
  if (!cell) return 0;
  if (cap < total) return 97;
  for (int t = 0; t < total; t++) {
    const int pc = code[(size_t)t];
    cell[t] = skeys[(size_t)t];
    idx[t] = pc >= 0 ? pc : -(pc + 1);
    real[t] = pc >= 0 ? 1 : 0;
    coords[(size_t)t * N + 0] = (double)px[(size_t)t];
    coords[(size_t)t * N + 1] = (double)py[(size_t)t];
    if (N == 3) coords[(size_t)t * N + 2] = (double)pz[(size_t)t];
  }
  return 0;
}
}  // namespace

extern "C" int build_probe(int f64, int dim, int kind, const double* Mcol, double cutoff, int lcell, const double* x,
                           int n, int64_t cap, int64_t* n_copies, int64_t* n_real_cells, int64_t* cell, int64_t* idx,
                           int8_t* real, double* coords, int* err) {
  if (dim == 3)
    return f64 ? run<double, 3>(kind, Mcol, cutoff, lcell, x, n, cap, n_copies, n_real_cells, cell, idx, real,
                                coords, err)
               : run<float, 3>(kind, Mcol, cutoff, lcell, x, n, cap, n_copies, n_real_cells, cell, idx, real, coords,
                               err);
  return f64 ? run<double, 2>(kind, Mcol, cutoff, lcell, x, n, cap, n_copies, n_real_cells, cell, idx, real, coords,
                              err)
             : run<float, 2>(kind, Mcol, cutoff, lcell, x, n, cap, n_copies, n_real_cells, cell, idx, real, coords,
                             err);
}

// The k-th offset of the pair kernel's stencil (runtime lcell, or lcell = 1 fixed at compile time).
extern "C" void stencil_probe(int forward, int lcell, int fixed1, int dim, int k, int* o) {
  if (fixed1) clm::stencil_offset<1>(forward != 0, lcell, dim, k, o);
  else clm::stencil_offset(forward != 0, lcell, dim, k, o);
}
