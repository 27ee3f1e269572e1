// Test infrastructure: runs the library's device-code decisions on the host, so that the CPU tests can
// compare them with the oracle without a GPU (built by tests/test_build_steps.py with g++
// -ffp-contract=off, as the library's host code is):
//   build_probe        the cell-list build steps (csrc/clm_build_steps.cuh: the geometry copy the kernels
//                      receive, K1 wrap_count_at, K2 emit_at, K4 gather_at) one particle or copy at a time,
//                      with the copy-offset scan replaced by its contract (offsets in particle order) and the
//                      counting placement emulated (arrival ranks in a scrambled order, cell starts, each
//                      copy's final slot from rank_in_cell), which must give the stable sort by cell;
//   stencil_probe      the pair kernel's stencil enumeration; cell_probe its cell index (border case);
//   band_probe         the condition under which the pair kernel skips the projection filter;
//   map_nl_probe,      the self and x-y pair maps emulated from the kernel's pieces (stencil, pair_rule,
//   map_cross_probe    exact test, band, projection filter, FP32 distance pass);
//   split_error_probe, the split form's FP32 distance error against its bound, the histogram guard, the
//   split_bins_probe,  bin search and the exact re-decision window, and the split form's histogram
//   bin_probe,         counts composed over every x-y pair.
//   near_edge_probe, split_hist_probe
//   map_nl_visits_probe the self-pair map's candidate visits that reach the hit queue, and its pairs;
//   noalloc_slots_probe the per-block slots of the allocation-free entry point's scratch;
//   cell_floor_probe   the cell index's floor from the reciprocal product against the IEEE quotient's.
//   image_key_probe    the image tests on order keys against the sums and compares they stand for.
//   first_key_probe    the image-test thresholds on arbitrary shifts and bounds.
//   quot_probe         the wrap solve's checked reciprocal quotient against the IEEE division.
//   cell_index_probe   the cell index's floor from the bits of the reciprocal product, with its range test.
//   float_pair_probe   the gather's float pair of a double from its bits against the two conversions.
//   wrap_shape_probe   the wrap that skips a cell's exact-zero terms against the general wrap.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <vector>

#include "clm_build_steps.cuh"
#include "clm_internal.hpp"

namespace {

template <class T, int N> struct HostList {
  clm::DevGeom<T> d;
  int err = 0;
  int total = 0;
  std::vector<uint32_t> skeys;  // cell of each copy, in cell order
  std::vector<T> px, py, pz;    // coordinates of each copy
  std::vector<int> code, flags, start;
  T x(int t, int k) const { return k == 0 ? px[(size_t)t] : (k == 1 ? py[(size_t)t] : pz[(size_t)t]); }
};

// Geometry and cell list of one set, as clm_set_box + clm_build make them; returns a clm status (or 9x for a
// broken cell-start table).
template <class T, int N>
int build_host(int kind, const double* Mcol, double cutoff, int lcell, const double* xin, int n, HostList<T, N>& L,
               const double* other = nullptr, int n_other = 0) {
  std::vector<T> x((size_t)n * N), wrapped((size_t)n * N);
  for (size_t k = 0; k < x.size(); k++) x[k] = (T)xin[k];
  T M[3][3] = {}, origin[3] = {0, 0, 0};
  if (kind == clm::NONPERIODIC) {
    // the limits box of the particles (of both sets for x-y pairs: `other`), as the library's set_limits +
    // nonperiodic_cell make it
    T lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int i = 0; i < n + n_other; i++)
      for (int k = 0; k < N; k++) {
        const T v = i < n ? x[(size_t)i * N + k] : (T)other[(size_t)(i - n) * N + k];
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
  clm::DevGeom<T>& d = L.d;
  clm::fill_devgeom<T>(g, 1, d);
  std::vector<uint32_t> mask((size_t)n);
  std::vector<int> ncopy((size_t)n), off((size_t)n + 1, 0);
  for (int i = 0; i < n; i++)
    if (!clm::wrap_count_at<T, N>(d, x.data(), i, wrapped.data(), mask.data(), ncopy.data())) L.err |= clm::DERR_NAN;
  for (int i = 0; i < n; i++) off[(size_t)i + 1] = off[(size_t)i] + ncopy[(size_t)i];
  const int total = off[(size_t)n];
  std::vector<uint32_t> keys((size_t)total), vals((size_t)total);
  for (int i = 0; i < n; i++)
    clm::emit_at<T, N>(d, 0, wrapped.data(), mask.data(), ncopy.data(), off.data(), i, total, keys.data(),
                       vals.data(), &L.err);
  const int ncells = d.ncells;
  // the counting build of one system: copies take their cell's slots in an arrival order the device leaves
  // open (emulated by a fixed scramble of the copies), the cell starts are the scan of the counts, and each
  // copy moves to its cell's start plus its rank by value in the cell (rank_in_cell)
  std::vector<int> cnt((size_t)ncells + 1, 0), arrival((size_t)total), order((size_t)total);
  std::iota(order.begin(), order.end(), 0);
  uint64_t rs = 0x9e3779b97f4a7c15ull;
  for (int t = total - 1; t > 0; t--) {
    rs = rs * 6364136223846793005ull + 1442695040888963407ull;
    std::swap(order[(size_t)t], order[(size_t)((rs >> 33) % (uint64_t)(t + 1))]);
  }
  for (int q : order) arrival[(size_t)q] = cnt[keys[(size_t)q]]++;
  std::vector<int> cstart((size_t)ncells + 1, 0);
  for (int c = 0; c < ncells; c++) cstart[(size_t)c + 1] = cstart[(size_t)c] + cnt[(size_t)c];
  std::vector<uint32_t> pk((size_t)total), pv((size_t)total), svals((size_t)total);
  for (int t = 0; t < total; t++) {
    const int pos = cstart[keys[(size_t)t]] + arrival[(size_t)t];
    pk[(size_t)pos] = keys[(size_t)t];
    pv[(size_t)pos] = vals[(size_t)t];
  }
  L.skeys.resize((size_t)total);
  for (int q = 0; q < total; q++) {
    const uint32_t c = pk[(size_t)q];
    const int t = cstart[c] + clm::rank_in_cell(pv.data(), cstart[c], cstart[c + 1], pv[(size_t)q]);
    L.skeys[(size_t)t] = c;
    svals[(size_t)t] = pv[(size_t)q];
  }
  // which is the contract of a stable sort by cell (particle order inside a cell)
  std::vector<int> perm((size_t)total);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return keys[(size_t)a] < keys[(size_t)b]; });
  for (int t = 0; t < total; t++)
    if (L.skeys[(size_t)t] != keys[(size_t)perm[(size_t)t]] || svals[(size_t)t] != vals[(size_t)perm[(size_t)t]])
      return 97;
  L.total = total;
  L.px.assign((size_t)total + 1, T(0));
  L.py.assign((size_t)total + 1, T(0));
  L.pz.assign((size_t)total + 1, T(0));
  std::vector<float4> foff((size_t)total + 1), xq((size_t)total + 1);
  L.code.assign((size_t)total + 1, 0);
  L.flags.assign((size_t)ncells + 1, 0);
  L.start.assign((size_t)ncells + 1, -1);
  for (int t = 0; t <= total; t++) {
    clm::cell_starts_at(L.skeys.data(), t, total, ncells, L.start.data());
    if (t == total) break;
    const int p = (int)(svals[(size_t)t] >> 5), k = (int)(svals[(size_t)t] & 31u);
    clm::gather_at<T, N>(d, wrapped.data(), t, p, k, (int)L.skeys[(size_t)t], L.px.data(), L.py.data(),
                         L.pz.data(), foff.data(), xq.data(), L.code.data(), L.flags.data(), 0);
  }
  // cell_start must bracket each cell's copies
  for (int c = 0; c < ncells; c++)
    if (L.start[(size_t)c] < 0 || L.start[(size_t)c] > L.start[(size_t)c + 1]) return 99;
  for (int t = 0; t < total; t++)
    if (L.start[L.skeys[(size_t)t]] > t || L.start[L.skeys[(size_t)t] + 1] <= t) return 98;
  for (int c = 0; c <= ncells; c++)
    if (L.start[(size_t)c] != cstart[(size_t)c]) return 96;  // the cell scan's starts
  return 0;
}

// FP32 prefilter coordinates of a cell list's copies for Float64 handles, as the gather writes them: the
// FP32 offset of each copy from its cell origin, in float pairs.
template <class T, int N> std::vector<float4> fp32_offsets(const HostList<T, N>& L) {
  const clm::DevGeom<T>& g = L.d;
  std::vector<float4> foff((size_t)L.total + 1);
  if (sizeof(T) == 8) {
    for (int t = 0; t < L.total; t++) {
      int c[3];
      clm::cart_of((int)L.skeys[(size_t)t], g.nc, N, c);
      float o[3] = {0.f, 0.f, 0.f};
      for (int d = 0; d < N; d++) {
        float oh, ol;
        clm::origin_ff(g.cbf_hi[d], g.cbf_lo[d], g.csf[d], g.csf_lo[d], c[d] - 1, oh, ol);
        const float qh = (float)L.x(t, d);
        const float ql = (float)(L.x(t, d) - (T)qh);
        o[d] = (qh - oh) + (ql - ol);
      }
      foff[(size_t)t] = make_float4(o[0], o[1], o[2], 0.f);
    }
  }
  return foff;
}

// The FP32 distance pass of the kernel for copy a of list La against copy b of list Lb in a cell displaced
// by o: true when it keeps the pair (d2 - thr_hi < 0) with the displacement shift of the offsets both
// fused and unfused.
template <class T, int N>
bool fp32_keeps(const HostList<T, N>& La, const std::vector<float4>& fa, int a, const HostList<T, N>& Lb,
                const std::vector<float4>& fb, int b, const int* o) {
  const clm::DevGeom<T>& g = La.d;
  for (int fused = 0; fused < 2; fused++) {
    float p[3] = {0.f, 0.f, 0.f}, q[3] = {0.f, 0.f, 0.f};
    for (int k = 0; k < N; k++) {
      if (sizeof(T) == 4) {
        p[k] = (float)La.x(a, k);
        q[k] = (float)Lb.x(b, k);
      } else {
        const float offk = k == 0 ? fb[(size_t)b].x : (k == 1 ? fb[(size_t)b].y : fb[(size_t)b].z);
        const float sh = (float)o[k];
        q[k] = fused ? std::fmaf(g.csf[k], sh, offk) : offk + g.csf[k] * sh;
        p[k] = k == 0 ? fa[(size_t)a].x : (k == 1 ? fa[(size_t)a].y : fa[(size_t)a].z);
      }
    }
    const float fx = p[0] - q[0], fy = p[1] - q[1], fz = p[2] - q[2];
    const float ef = std::fmaf(fz, fz, std::fmaf(fy, fy, std::fmaf(fx, fx, -g.thr_hi)));
    if (!(ef < 0.f)) return false;
  }
  return true;
}

// The split form's FP32 squared distance (Float64 handles) of copy a against copy b in a cell displaced by o,
// with the displacement shift of the candidate's offset fused or not.
template <class T, int N>
float fp32_d2(const std::vector<float4>& fa, int a, const std::vector<float4>& fb, int b, const float* csf,
              const int* o, bool fused) {
  float e = 0.f;
  for (int k = 0; k < N; k++) {
    const float pa = k == 0 ? fa[(size_t)a].x : (k == 1 ? fa[(size_t)a].y : fa[(size_t)a].z);
    const float pb = k == 0 ? fb[(size_t)b].x : (k == 1 ? fb[(size_t)b].y : fb[(size_t)b].z);
    const float q = fused ? std::fmaf(csf[k], (float)o[k], pb) : pb + csf[k] * (float)o[k];
    const float dk = pa - q;
    e = std::fmaf(dk, dk, e);
  }
  return e;
}

template <class T, int N>
int run(int kind, const double* Mcol, double cutoff, int lcell, const double* xin, int n, int64_t cap,
        int64_t* n_copies, int64_t* n_real_cells, int64_t* cell, int64_t* idx, int8_t* real, double* coords,
        int* err_out) {
  HostList<T, N> L;
  const int st = build_host<T, N>(kind, Mcol, cutoff, lcell, xin, n, L);
  if (st) return st;
  *err_out = L.err;
  *n_copies = L.total;
  *n_real_cells = 0;
  for (int c = 0; c < L.d.ncells; c++) *n_real_cells += L.flags[(size_t)c] ? 1 : 0;
  if (!cell) return 0;
  if (cap < L.total) return 97;
  for (int t = 0; t < L.total; t++) {
    const int pc = L.code[(size_t)t];
    cell[t] = L.skeys[(size_t)t];
    idx[t] = pc >= 0 ? pc : -(pc + 1);
    real[t] = pc >= 0 ? 1 : 0;
    for (int k = 0; k < N; k++) coords[(size_t)t * N + k] = (double)L.x(t, k);
  }
  return 0;
}

// Over every pair (real copy a of a cell, copy b of another cell of the full stencil): the pair kernel
// accepts a pair without the projection filter when its exact d2 is at most the band bound thr_lo (or, for
// Float32 handles, when the FP32 distance test of the kernel, fma(dz,dz,fma(dy,dy,dx*dx)) on the
// coordinates, is).  Counts such pairs for which the exact d2 exceeds the cutoff or the reference's filter
// (projection_pass) would reject the pair: out = {pairs within the cutoff, pairs accepted by the shortcut,
// pairs in the band (filter evaluated), band pairs the filter rejects, violations}.
template <class T, int N>
int band(int kind, const double* Mcol, double cutoff, int lcell, const double* xin, int n, int64_t* out) {
  HostList<T, N> L;
  const int st = build_host<T, N>(kind, Mcol, cutoff, lcell, xin, n, L);
  if (st) return st;
  const clm::DevGeom<T>& g = L.d;
  const T thr = (T)g.thr_lo;
  const std::vector<float4> fo = fp32_offsets(L);
  const int w = 2 * g.lcell + 1;
  const int nst = (N == 3) ? w * w * w - 1 : w * w - 1;
  for (int k = 0; k < 5; k++) out[k] = 0;
  for (int ci_lin = 0; ci_lin < g.ncells; ci_lin++) {
    if (!L.flags[(size_t)ci_lin]) continue;
    int ci[3];
    clm::cart_of(ci_lin, g.nc, N, ci);
    T ctr_i[3] = {0, 0, 0};
    clm::cell_center<T, N>(g, ci, ctr_i);
    for (int s = 0; s < nst; s++) {
      int o[3];
      clm::stencil_offset(false, g.lcell, N, s, o);
      const int cj[3] = {ci[0] + o[0], ci[1] + o[1], N == 3 ? ci[2] + o[2] : 1};
      bool inside = true;
      for (int k = 0; k < N; k++) inside = inside && cj[k] >= 1 && cj[k] <= g.nc[k];
      if (!inside) continue;
      const int cj_lin = (N == 3) ? (cj[0] - 1) + g.nc[0] * ((cj[1] - 1) + g.nc[1] * (cj[2] - 1))
                                  : (cj[0] - 1) + g.nc[0] * (cj[1] - 1);
      T ctr_j[3] = {0, 0, 0};
      clm::cell_center<T, N>(g, cj, ctr_j);
      for (int a = L.start[(size_t)ci_lin]; a < L.start[(size_t)ci_lin + 1]; a++) {
        if (L.code[(size_t)a] < 0) continue;  // the particle side is a real copy
        T xa[3];
        for (int k = 0; k < N; k++) xa[k] = L.x(a, k);
        for (int b = L.start[(size_t)cj_lin]; b < L.start[(size_t)cj_lin + 1]; b++) {
          T xb[3], dx[3];
          for (int k = 0; k < N; k++) {
            xb[k] = L.x(b, k);
            dx[k] = clm::xsub(xa[k], xb[k]);
          }
          T d2 = clm::xmul(dx[0], dx[0]);  // the exact d2, in the reference's order
          for (int k = 1; k < N; k++) d2 = clm::xadd(d2, clm::xmul(dx[k], dx[k]));
          bool shortcut = d2 <= thr;
          if constexpr (sizeof(T) == 8) {
            // the split form accepts a pair whose FP32 offset distance is below thr_lo (either rounding)
            for (int fused = 0; fused < 2; fused++)
              if (fp32_d2<T, N>(fo, a, fo, b, g.csf, o, fused != 0) <= g.thr_lo) shortcut = true;
          }
          if constexpr (sizeof(T) == 4) {
            const float fx = xa[0] - xb[0], fy = xa[1] - xb[1], fz = (N == 3) ? xa[N - 1] - xb[N - 1] : 0.f;
            const float d2f = std::fmaf(fz, fz, std::fmaf(fy, fy, fx * fx));
            if (d2f <= g.thr_lo) shortcut = true;
          }
          const bool within = d2 <= g.cutoff_sqr;
          out[0] += within ? 1 : 0;
          if (shortcut) {
            out[1]++;
            if (!within || !clm::projection_pass<T, N>(g, ctr_i, ctr_j, xa, xb)) out[4]++;
          } else if (within) {
            out[2]++;
            if (!clm::projection_pass<T, N>(g, ctr_i, ctr_j, xa, xb)) out[3]++;
          }
        }
      }
    }
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

extern "C" int band_probe(int f64, int dim, int kind, const double* Mcol, double cutoff, int lcell, const double* x,
                          int n, int64_t* out) {
  if (dim == 3)
    return f64 ? band<double, 3>(kind, Mcol, cutoff, lcell, x, n, out)
               : band<float, 3>(kind, Mcol, cutoff, lcell, x, n, out);
  return f64 ? band<double, 2>(kind, Mcol, cutoff, lcell, x, n, out)
             : band<float, 2>(kind, Mcol, cutoff, lcell, x, n, out);
}

// The k-th offset of the pair kernel's stencil (runtime lcell, or lcell = 1 fixed at compile time).
extern "C" void stencil_probe(int forward, int lcell, int fixed1, int dim, int k, int* o) {
  if (fixed1) clm::stencil_offset<1>(forward != 0, lcell, dim, k, o);
  else clm::stencil_offset(forward != 0, lcell, dim, k, o);
}

// The library's cell of one point (cell_of, with the border-case shift when `real`), as 1-based cartesian
// indices; returns the linear index or -1, or a clm status (> 0 is returned as -2 - status).
extern "C" int cell_probe(int dim, int kind, const double* Mcol, double cutoff, int lcell, const double* x, int real,
                          int* cart, int* nc) {
  double M[3][3] = {};
  for (int i = 0; i < dim; i++)
    for (int j = 0; j < dim; j++) M[i][j] = (kind == clm::ORTHO && i != j) ? 0.0 : Mcol[j * dim + i];
  clm::Geometry<double> g;
  const int st = clm::make_geometry<double>(g, dim, kind, M, cutoff, lcell, nullptr);
  if (st) return -2 - st;
  clm::DevGeom<double> d;
  clm::fill_devgeom<double>(g, 1, d);
  for (int k = 0; k < 3; k++) nc[k] = d.nc[k];
  const int li = (dim == 3) ? clm::cell_of<double, 3>(d, x, real != 0) : clm::cell_of<double, 2>(d, x, real != 0);
  if (li >= 0) clm::cart_of(li, d.nc, dim, cart);
  return li;
}

namespace {
// The self-pair map of the pair kernel, emulated on the host from the library's own pieces: the cells with
// real particles, every copy of such a cell as the particle side, stencil entry 0 (the cell itself) then
// the forward half stencil (orthorhombic, non-periodic) or, in triclinic cells, the forward half and the
// cells of the backward half that hold no real particle (sym_stencil_offset), the kernel's pair rule, the
// exact test in the input dtype and, for pairs in the band d2 > thr_lo of another cell, the projection
// filter seen from the cell of the reference's i (the copy of the lower index in triclinic cells).  The FP32
// distance pass of the kernel is evaluated too, with the cell-displacement shift of the offsets both fused
// and unfused: a pair the exact test accepts but the FP32 pass would drop is counted in *lost.  *visits
// (when given) receives the number of candidate visits the FP32 pass could let through: copies pairs within
// the cutoff before the pair rule, excluding pairs of two images (which the kernel drops in that pass).
template <class T, int N>
int64_t map_nl(int kind, const double* Mcol, double cutoff, int lcell, const double* xin, int n, int64_t cap,
               int64_t* pi_out, int64_t* pj_out, double* d_out, int64_t* lost, int* st_out, int64_t* visits = nullptr) {
  HostList<T, N> L;
  *st_out = build_host<T, N>(kind, Mcol, cutoff, lcell, xin, n, L);
  if (*st_out) return -1;
  const clm::DevGeom<T>& g = L.d;
  const bool tri = g.kind == clm::TRICLINIC, nonper = g.kind == clm::NONPERIODIC;
  const int w = 2 * g.lcell + 1;
  const int wN = (N == 3) ? w * w * w : w * w;
  const int nf = (wN - 1) / 2;
  const int nent = nf * (tri ? 2 : 1) + 1;
  const T band = (T)g.thr_lo;
  const std::vector<float4> foff = fp32_offsets(L);
  int64_t np = 0;
  *lost = 0;
  if (visits) *visits = 0;
  for (int ci_lin = 0; ci_lin < g.ncells; ci_lin++) {
    if (!L.flags[(size_t)ci_lin]) continue;
    int ci[3];
    clm::cart_of(ci_lin, g.nc, N, ci);
    T ctr_i[3] = {0, 0, 0};
    clm::cell_center<T, N>(g, ci, ctr_i);
    const int si = L.start[(size_t)ci_lin], ni = L.start[(size_t)ci_lin + 1] - si;
    for (int ii = 0; ii < ni; ii++) {
      const int a = si + ii;
      const int code_i = L.code[(size_t)a];
      const bool real_i = code_i >= 0;
      const int idx_i = real_i ? code_i : -code_i - 1;
      T xa[3];
      for (int k = 0; k < N; k++) xa[k] = L.x(a, k);
      for (int e = 0; e < nent; e++) {
        int o[3] = {0, 0, 0};
        bool back = false;
        if (e > 0) clm::sym_stencil_offset(g.lcell, N, nf, e - 1, o, &back);
        const int cj[3] = {ci[0] + o[0], ci[1] + o[1], N == 3 ? ci[2] + o[2] : 1};
        bool inside = true;
        for (int k = 0; k < N; k++) inside = inside && cj[k] >= 1 && cj[k] <= g.nc[k];
        if (!inside) continue;
        const int cj_lin = (N == 3) ? (cj[0] - 1) + g.nc[0] * ((cj[1] - 1) + g.nc[1] * (cj[2] - 1))
                                    : (cj[0] - 1) + g.nc[0] * (cj[1] - 1);
        if (back && L.flags[(size_t)cj_lin]) continue;  // that pair of cells is visited from the other cell
        const int sj = L.start[(size_t)cj_lin], nj = L.start[(size_t)cj_lin + 1] - sj;
        T ctr_j[3] = {0, 0, 0};
        if (e > 0) clm::cell_center<T, N>(g, cj, ctr_j);
        for (int jj = 0; jj < nj; jj++) {
          const int b = sj + jj;
          const int code_j = L.code[(size_t)b];
          const bool real_j = code_j >= 0;
          const int idx_j = real_j ? code_j : -code_j - 1;
          T xb[3], dx[3];
          for (int k = 0; k < N; k++) {
            xb[k] = L.x(b, k);
            dx[k] = clm::xsub(xa[k], xb[k]);
          }
          T d2 = clm::xmul(dx[0], dx[0]);
          for (int k = 1; k < N; k++) d2 = clm::xadd(d2, clm::xmul(dx[k], dx[k]));
          if (visits && d2 <= g.cutoff_sqr && (e > 0 || jj > ii) && (real_i || real_j)) (*visits)++;
          if (!clm::pair_rule(false, tri, nonper, e == 0, jj, ii, real_i, real_j, idx_i, idx_j)) continue;
          // the reference's i: the particle copy, or in triclinic cells the copy of the lower index
          const bool swap = tri && idx_j < idx_i;
          bool hit = d2 <= g.cutoff_sqr;
          if (hit && d2 > band && e > 0)
            hit = swap ? clm::projection_pass<T, N>(g, ctr_j, ctr_i, xb, xa) : clm::projection_pass<T, N>(g, ctr_i, ctr_j, xa, xb);
          if (!hit) continue;
          // the FP32 distance pass must keep this pair, whichever way the shift rounds
          if (!fp32_keeps(L, foff, a, L, foff, b, o)) (*lost)++;
          if (np < cap) {
            pi_out[np] = swap ? idx_j : idx_i;
            pj_out[np] = swap ? idx_i : idx_j;
            d_out[np] = (double)clm::xsqrt(d2);
          }
          np++;
        }
      }
    }
  }
  return np;
}
}  // namespace

extern "C" int64_t map_nl_probe(int f64, int dim, int kind, const double* Mcol, double cutoff, int lcell,
                                const double* x, int n, int64_t cap, int64_t* pi, int64_t* pj, double* d,
                                int64_t* lost, int* st) {
  if (dim == 3)
    return f64 ? map_nl<double, 3>(kind, Mcol, cutoff, lcell, x, n, cap, pi, pj, d, lost, st)
               : map_nl<float, 3>(kind, Mcol, cutoff, lcell, x, n, cap, pi, pj, d, lost, st);
  return f64 ? map_nl<double, 2>(kind, Mcol, cutoff, lcell, x, n, cap, pi, pj, d, lost, st)
             : map_nl<float, 2>(kind, Mcol, cutoff, lcell, x, n, cap, pi, pj, d, lost, st);
}

namespace {
// The x-y (cross) map of the pair kernel emulated on the host: the cells with real x
// particles, every x copy of such a cell as the particle side (real copies only in triclinic cells), the y
// copies of the cell itself and of all its neighbours as candidates, the kernel's pair rule, the exact test,
// the band and the projection filter; the FP32 pass is checked as for self pairs.
template <class T, int N>
int64_t map_cross(int kind, const double* Mcol, double cutoff, int lcell, const double* xin, int nx,
                  const double* yin, int ny, int64_t cap, int64_t* pi_out, int64_t* pj_out, double* d_out,
                  int64_t* lost, int* st_out) {
  HostList<T, N> X, Y;  // one geometry for both sets (non-periodic: the limits of both)
  *st_out = build_host<T, N>(kind, Mcol, cutoff, lcell, xin, nx, X, yin, ny);
  if (!*st_out) *st_out = build_host<T, N>(kind, Mcol, cutoff, lcell, yin, ny, Y, xin, nx);
  if (*st_out) return -1;
  const clm::DevGeom<T>& g = X.d;
  const bool tri = g.kind == clm::TRICLINIC;
  const int w = 2 * g.lcell + 1;
  const int nent = ((N == 3) ? w * w * w : w * w);  // the cell itself, then all neighbours
  const T band = (T)g.thr_lo;
  const std::vector<float4> fx = fp32_offsets(X), fy = fp32_offsets(Y);
  int64_t np = 0;
  *lost = 0;
  for (int ci_lin = 0; ci_lin < g.ncells; ci_lin++) {
    if (!X.flags[(size_t)ci_lin]) continue;
    int ci[3];
    clm::cart_of(ci_lin, g.nc, N, ci);
    T ctr_i[3] = {0, 0, 0};
    clm::cell_center<T, N>(g, ci, ctr_i);
    const int si = X.start[(size_t)ci_lin], ni = X.start[(size_t)ci_lin + 1] - si;
    for (int ii = 0; ii < ni; ii++) {
      const int a = si + ii;
      const int code_i = X.code[(size_t)a];
      const bool real_i = code_i >= 0;
      const int idx_i = real_i ? code_i : -code_i - 1;
      if (tri && !real_i) continue;
      T xa[3];
      for (int k = 0; k < N; k++) xa[k] = X.x(a, k);
      for (int e = 0; e < nent; e++) {
        int o[3] = {0, 0, 0};
        if (e > 0) clm::stencil_offset(false, g.lcell, N, e - 1, o);
        const int cj[3] = {ci[0] + o[0], ci[1] + o[1], N == 3 ? ci[2] + o[2] : 1};
        bool inside = true;
        for (int k = 0; k < N; k++) inside = inside && cj[k] >= 1 && cj[k] <= g.nc[k];
        if (!inside) continue;
        const int cj_lin = (N == 3) ? (cj[0] - 1) + g.nc[0] * ((cj[1] - 1) + g.nc[1] * (cj[2] - 1))
                                    : (cj[0] - 1) + g.nc[0] * (cj[1] - 1);
        const int sj = Y.start[(size_t)cj_lin], nj = Y.start[(size_t)cj_lin + 1] - sj;
        T ctr_j[3] = {0, 0, 0};
        if (e > 0) clm::cell_center<T, N>(g, cj, ctr_j);
        for (int jj = 0; jj < nj; jj++) {
          const int b = sj + jj;
          const int code_j = Y.code[(size_t)b];
          const bool real_j = code_j >= 0;
          const int idx_j = real_j ? code_j : -code_j - 1;
          if (!clm::pair_rule(true, tri, g.kind == clm::NONPERIODIC, e == 0, jj, ii, real_i, real_j, idx_i, idx_j))
            continue;
          T xb[3], dx[3];
          for (int k = 0; k < N; k++) {
            xb[k] = Y.x(b, k);
            dx[k] = clm::xsub(xa[k], xb[k]);
          }
          T d2 = clm::xmul(dx[0], dx[0]);
          for (int k = 1; k < N; k++) d2 = clm::xadd(d2, clm::xmul(dx[k], dx[k]));
          bool hit = d2 <= g.cutoff_sqr;
          if (hit && d2 > band && e > 0) hit = clm::projection_pass<T, N>(g, ctr_i, ctr_j, xa, xb);
          if (!hit) continue;
          if (!fp32_keeps(X, fx, a, Y, fy, b, o)) (*lost)++;
          if (np < cap) {
            pi_out[np] = idx_i;
            pj_out[np] = idx_j;
            d_out[np] = (double)clm::xsqrt(d2);
          }
          np++;
        }
      }
    }
  }
  return np;
}
}  // namespace

extern "C" int64_t map_cross_probe(int f64, int dim, int kind, const double* Mcol, double cutoff, int lcell,
                                   const double* x, int nx, const double* y, int ny, int64_t cap, int64_t* pi,
                                   int64_t* pj, double* d, int64_t* lost, int* st) {
  if (dim == 3)
    return f64 ? map_cross<double, 3>(kind, Mcol, cutoff, lcell, x, nx, y, ny, cap, pi, pj, d, lost, st)
               : map_cross<float, 3>(kind, Mcol, cutoff, lcell, x, nx, y, ny, cap, pi, pj, d, lost, st);
  return f64 ? map_cross<double, 2>(kind, Mcol, cutoff, lcell, x, nx, y, ny, cap, pi, pj, d, lost, st)
             : map_cross<float, 2>(kind, Mcol, cutoff, lcell, x, nx, y, ny, cap, pi, pj, d, lost, st);
}

// Largest |r_fp32 - r| over the pairs within the cutoff (real copy of a cell against every copy of the
// full stencil), divided by the library's bound split_distance_error: r_fp32 is the split form's FP32
// distance of cell-relative offsets (shift fused and unfused), r the exact distance.  Float64 handles.
extern "C" int split_error_probe(int dim, int kind, const double* Mcol, double cutoff, int lcell, const double* x,
                                 int n, double* worst) {
  auto run = [&](auto tag) -> int {
    constexpr int N = decltype(tag)::value;
    HostList<double, N> L;
    const int st = build_host<double, N>(kind, Mcol, cutoff, lcell, x, n, L);
    if (st) return st;
    const clm::DevGeom<double>& g = L.d;
    clm::Geometry<double> geo;  // the bound needs the cell sides and lcell only
    geo.dim = N;
    geo.lcell = g.lcell;
    for (int k = 0; k < 3; k++) geo.cs[k] = k < N ? g.cs[k] : 0.0;
    const double bound = clm::split_distance_error(geo);
    const std::vector<float4> fo = fp32_offsets(L);
    const int w = 2 * g.lcell + 1, nst = (N == 3) ? w * w * w : w * w;  // entry 0: the cell itself
    *worst = 0.0;
    for (int ci_lin = 0; ci_lin < g.ncells; ci_lin++) {
      if (!L.flags[(size_t)ci_lin]) continue;
      int ci[3];
      clm::cart_of(ci_lin, g.nc, N, ci);
      for (int s = 0; s < nst; s++) {
        int o[3] = {0, 0, 0};
        if (s > 0) clm::stencil_offset(false, g.lcell, N, s - 1, o);
        const int cj[3] = {ci[0] + o[0], ci[1] + o[1], N == 3 ? ci[2] + o[2] : 1};
        bool inside = true;
        for (int k = 0; k < N; k++) inside = inside && cj[k] >= 1 && cj[k] <= g.nc[k];
        if (!inside) continue;
        const int cj_lin = (N == 3) ? (cj[0] - 1) + g.nc[0] * ((cj[1] - 1) + g.nc[1] * (cj[2] - 1))
                                    : (cj[0] - 1) + g.nc[0] * (cj[1] - 1);
        for (int a = L.start[(size_t)ci_lin]; a < L.start[(size_t)ci_lin + 1]; a++) {
          if (L.code[(size_t)a] < 0) continue;
          for (int b = L.start[(size_t)cj_lin]; b < L.start[(size_t)cj_lin + 1]; b++) {
            double d2 = 0.0;
            for (int k = 0; k < N; k++) d2 += (L.x(a, k) - L.x(b, k)) * (L.x(a, k) - L.x(b, k));
            if (d2 > g.cutoff_sqr || b == a) continue;
            for (int fused = 0; fused < 2; fused++) {
              const float e = fp32_d2<double, N>(fo, a, fo, b, g.csf, o, fused != 0);
              const double err = std::fabs((double)std::sqrt(e) - std::sqrt(d2));
              *worst = std::max(*worst, err / bound);
            }
          }
        }
      }
    }
    return 0;
  };
  return dim == 3 ? run(std::integral_constant<int, 3>()) : run(std::integral_constant<int, 2>());
}

// The library's guard for split-form histograms: 1 when every positive edge is above the split form's
// distance error window (split_bins_exact); *rmin receives that smallest safe edge.
extern "C" int split_bins_probe(int dim, int kind, const double* Mcol, double cutoff, int lcell, const double* edges,
                                int nedges, double* rmin) {
  double M[3][3] = {};
  for (int i = 0; i < dim; i++)
    for (int j = 0; j < dim; j++) M[i][j] = (kind == clm::ORTHO && i != j) ? 0.0 : Mcol[j * dim + i];
  clm::Geometry<double> g;
  const int st = clm::make_geometry<double>(g, dim, kind, M, cutoff, lcell, nullptr);
  if (st) return -st;
  *rmin = clm::split_distance_error(g) * 4096.0;
  return clm::split_bins_exact(g, edges, nedges) ? 1 : 0;
}

// The pair kernel's histogram bin search (first_edge_at_or_above, on Float64 edges) and the split form's
// exact re-decision window (near_edge, on FP32 edges).
extern "C" int bin_probe(const double* edges, int nbins, double r) {
  return clm::first_edge_at_or_above(edges, nbins, r);
}
extern "C" int near_edge_probe(const float* edges, int nbins, float rf, int* lo) {
  *lo = clm::first_edge_at_or_above(edges, nbins, rf);
  return clm::near_edge(edges, nbins, *lo, rf) ? 1 : 0;
}

// Histogram counts of the x-y pairs the way the split form bins them (Float64 handles): a pair the FP32
// pass accepts outright (FP32 distance below the band) takes its bin from that FP32 distance unless the
// re-decision window applies; every other pair (and windowed ones) from the exact distance.  counts has
// nbins entries; returns the number of binned pairs, or -1 with *st set.
extern "C" int64_t split_hist_probe(int dim, int kind, const double* Mcol, double cutoff, int lcell, const double* x,
                                    int nx, const double* y, int ny, const double* edges, int nbins, int64_t* counts,
                                    int* st) {
  auto run = [&](auto tag) -> int64_t {
    constexpr int N = decltype(tag)::value;
    HostList<double, N> X, Y;
    *st = build_host<double, N>(kind, Mcol, cutoff, lcell, x, nx, X, y, ny);
    if (!*st) *st = build_host<double, N>(kind, Mcol, cutoff, lcell, y, ny, Y, x, nx);
    if (*st) return -1;
    const clm::DevGeom<double>& g = X.d;
    std::vector<float> ef((size_t)nbins + 1);
    for (int k = 0; k <= nbins; k++) ef[(size_t)k] = (float)edges[k];
    const std::vector<float4> fx = fp32_offsets(X), fy = fp32_offsets(Y);
    const bool tri = g.kind == clm::TRICLINIC, nonper = g.kind == clm::NONPERIODIC;
    const int w = 2 * g.lcell + 1, nent = (N == 3) ? w * w * w : w * w;
    for (int k = 0; k < nbins; k++) counts[k] = 0;
    int64_t binned = 0;
    for (int ci_lin = 0; ci_lin < g.ncells; ci_lin++) {
      if (!X.flags[(size_t)ci_lin]) continue;
      int ci[3];
      clm::cart_of(ci_lin, g.nc, N, ci);
      double ctr_i[3] = {0, 0, 0};
      clm::cell_center<double, N>(g, ci, ctr_i);
      for (int a = X.start[(size_t)ci_lin]; a < X.start[(size_t)ci_lin + 1]; a++) {
        const int ii = a - X.start[(size_t)ci_lin];
        const int code_i = X.code[(size_t)a];
        const bool real_i = code_i >= 0;
        if (tri && !real_i) continue;
        double xa[3];
        for (int k = 0; k < N; k++) xa[k] = X.x(a, k);
        for (int e = 0; e < nent; e++) {
          int o[3] = {0, 0, 0};
          if (e > 0) clm::stencil_offset(false, g.lcell, N, e - 1, o);
          const int cj[3] = {ci[0] + o[0], ci[1] + o[1], N == 3 ? ci[2] + o[2] : 1};
          bool inside = true;
          for (int k = 0; k < N; k++) inside = inside && cj[k] >= 1 && cj[k] <= g.nc[k];
          if (!inside) continue;
          const int cj_lin = (N == 3) ? (cj[0] - 1) + g.nc[0] * ((cj[1] - 1) + g.nc[1] * (cj[2] - 1))
                                      : (cj[0] - 1) + g.nc[0] * (cj[1] - 1);
          double ctr_j[3] = {0, 0, 0};
          if (e > 0) clm::cell_center<double, N>(g, cj, ctr_j);
          for (int b = Y.start[(size_t)cj_lin]; b < Y.start[(size_t)cj_lin + 1]; b++) {
            const int jj = b - Y.start[(size_t)cj_lin];
            const int code_j = Y.code[(size_t)b];
            if (!clm::pair_rule(true, tri, nonper, e == 0, jj, ii, real_i, code_j >= 0, 0, 0)) continue;
            double xb[3], d2 = 0.0;
            for (int k = 0; k < N; k++) xb[k] = Y.x(b, k);
            for (int k = 0; k < N; k++) d2 = clm::xadd(d2, clm::xmul(clm::xsub(xa[k], xb[k]), clm::xsub(xa[k], xb[k])));
            const float d2f = fp32_d2<double, N>(fx, a, fy, b, g.csf, o, true);
            const bool sure = d2f <= g.thr_lo;
            bool hit = sure || d2 <= g.cutoff_sqr;
            if (hit && !sure && d2 > (double)g.thr_lo && e > 0) hit = clm::projection_pass<double, N>(g, ctr_i, ctr_j, xa, xb);
            if (!hit) continue;
            int bin;
            const float rf = std::sqrt(d2f);
            const int lo = clm::first_edge_at_or_above(ef.data(), nbins, rf);
            if (sure && !clm::near_edge(ef.data(), nbins, lo, rf)) bin = lo - 1;
            else bin = clm::first_edge_at_or_above(edges, nbins, clm::xsqrt(d2)) - 1;
            if (bin >= 0 && bin < nbins) {
              counts[bin]++;
              binned++;
            }
          }
        }
      }
    }
    return binned;
  };
  return dim == 3 ? run(std::integral_constant<int, 3>()) : run(std::integral_constant<int, 2>());
}

// The self-pair map's candidate visits that pass the FP32 pass's image test (see map_nl), and its pairs.
extern "C" int64_t map_nl_visits_probe(int f64, int dim, int kind, const double* Mcol, double cutoff, int lcell,
                                       const double* x, int n, int64_t* visits, int* st) {
  int64_t lost = 0;
  if (dim == 3)
    return f64 ? map_nl<double, 3>(kind, Mcol, cutoff, lcell, x, n, 0, nullptr, nullptr, nullptr, &lost, st, visits)
               : map_nl<float, 3>(kind, Mcol, cutoff, lcell, x, n, 0, nullptr, nullptr, nullptr, &lost, st, visits);
  return f64 ? map_nl<double, 2>(kind, Mcol, cutoff, lcell, x, n, 0, nullptr, nullptr, nullptr, &lost, st, visits)
             : map_nl<float, 2>(kind, Mcol, cutoff, lcell, x, n, 0, nullptr, nullptr, nullptr, &lost, st, visits);
}

// Per-block slots of the allocation-free entry point's scratch (clm_internal.hpp noalloc_block_slots).
extern "C" long long noalloc_slots_probe(long long scratch_bytes, int tsize) {
  return (long long)clm::noalloc_block_slots((size_t)scratch_bytes, (size_t)tsize);
}

// pair_rule and its three parts as the pair kernel applies them (clm_device.cuh), for one case.
extern "C" int pair_rule_probe(int cross, int tri, int nonper, int same, int slot_j, int ii, int code_i, int code_j,
                               int* parts) {
  const int idx_i = code_i >= 0 ? code_i : ~code_i, idx_j = code_j >= 0 ? code_j : ~code_j;
  *parts = clm::pair_rule_parts(cross != 0, tri != 0, nonper != 0, same != 0, slot_j, ii, code_i, code_j) ? 1 : 0;
  return clm::pair_rule(cross != 0, tri != 0, nonper != 0, same != 0, slot_j, ii, code_i >= 0, code_j >= 0, idx_i,
                        idx_j)
             ? 1
             : 0;
}

// cell_floor (the cell index's floor of (x - xmin) / cs from a product with RN(1 / cs), the IEEE division near
// integers) against floor of the IEEE quotient, for n numerators; returns the number of disagreements.
extern "C" int64_t cell_floor_probe(int f64, const double* a, int64_t n, double cs) {
  int64_t bad = 0;
  for (int64_t t = 0; t < n; t++) {
    if (f64) {
      const double c = cs, inv = 1.0 / c, x = a[t];
      if (clm::cell_floor<double>(x, c, inv) != std::floor(x / c)) bad++;
    } else {
      const float c = (float)cs, inv = 1.0f / c, x = (float)a[t];
      if (clm::cell_floor<float>(x, c, inv) != std::floor(x / c)) bad++;
    }
  }
  return bad;
}

namespace {
// The image tests of one geometry on order keys (image_in) against the tests they stand for,
// cbmin <= RN(v + shift) < cbmax, for every image and axis: at the n values given, at the 7 keys around each
// of the two thresholds, and at +-0, +-inf and NaN.  Returns the number of disagreements, or -2 - status.
template <class T>
int64_t image_keys(int dim, int kind, const double* Mcol, double cutoff, int lcell, const double* v, int64_t n) {
  T M[3][3] = {};
  for (int i = 0; i < dim; i++)
    for (int j = 0; j < dim; j++) M[i][j] = (kind == clm::ORTHO && i != j) ? T(0) : (T)Mcol[j * dim + i];
  clm::Geometry<T> g;
  const int st = clm::make_geometry<T>(g, dim, kind, M, (T)cutoff, lcell, nullptr);
  if (st) return -2 - st;
  clm::DevGeom<T> d;
  clm::fill_devgeom<T>(g, 1, d);
  using K = typename clm::OrderKey<T>::type;
  const T inf = std::numeric_limits<T>::infinity();
  int64_t bad = 0;
  std::vector<T> vals;
  for (int k = 0; k < d.nimg; k++)
    for (int a = 0; a < dim; a++) {
      vals.clear();
      for (int64_t t = 0; t < n; t++) vals.push_back((T)v[t]);
      for (const K th : {d.img_lo[k][a], d.img_hi[k][a]})
        for (int j = -3; j <= 3; j++) vals.push_back(clm::from_order_key<T>(th + j));
      for (const T s : {T(0), -T(0), inf, -inf, std::numeric_limits<T>::quiet_NaN()}) vals.push_back(s);
      for (const T x : vals) {
        const T q = x + d.shift[k][a];
        const bool want = d.cbmin[a] <= q && q < d.cbmax[a];
        if (clm::image_in<T>(d, k, a, clm::order_key(x)) != want) bad++;
      }
    }
  return bad;
}
}  // namespace

extern "C" int64_t image_key_probe(int f64, int dim, int kind, const double* Mcol, double cutoff, int lcell,
                                   const double* v, int64_t n) {
  return f64 ? image_keys<double>(dim, kind, Mcol, cutoff, lcell, v, n)
             : image_keys<float>(dim, kind, Mcol, cutoff, lcell, v, n);
}

// quot_rn (the wrap solve's division from RN(1 / b) with a checked correction step) against the IEEE quotient
// a / b, bit for bit (NaN against NaN), for n pairs; returns the number of disagreements and, in *fallbacks,
// how many pairs took the IEEE division.
extern "C" int64_t quot_probe(const double* a, const double* b, int64_t n, int64_t* fallbacks) {
  int64_t bad = 0, fb = 0;
  for (int64_t t = 0; t < n; t++) {
    const double y = 1.0 / b[t], q = clm::quot_rn(a[t], b[t], y), want = a[t] / b[t];
    if (std::isnan(want) ? !std::isnan(q) : clm::dbits(q) != clm::dbits(want)) bad++;
    double qf;
    if (!clm::quot_fast(a[t], b[t], y, qf)) fb++;
  }
  *fallbacks = fb;
  return bad;
}

namespace {
template <class T> int64_t cell_index_t(const double* av, int64_t n, double csd, int nc, int64_t* fast) {
  const T cs = (T)csd, inv = T(1) / cs;
  int64_t bad = 0, nf = 0;
  for (int64_t t = 0; t < n; t++) {
    const T a = (T)av[t];
    const T q = std::floor(a / cs);
    const int want = (q >= T(-1) && q < (T)nc) ? (int)q : INT32_MIN;
    int fq;
    const bool f = clm::floor_quot_bits<T>(a * inv, fq);
    if (f) {
      nf++;
      if (fq >= nc) fq = INT32_MIN;
    } else {
      fq = clm::floor_quot_call<T>(a, cs, inv, nc);
    }
    if (fq != want) bad++;
  }
  *fast = nf;
  return bad;
}
}  // namespace

// The cell index's floor as cell_of takes it (floor_quot_bits on the reciprocal product, else
// floor_quot_call) against the IEEE floor(a / cs) with its range test [-1, nc), for n numerators; returns
// the number of disagreements and, in *fast, how many the bit screen decided.
extern "C" int64_t cell_index_probe(int f64, const double* a, int64_t n, double cs, int nc, int64_t* fast) {
  return f64 ? cell_index_t<double>(a, n, cs, nc, fast) : cell_index_t<float>(a, n, cs, nc, fast);
}

// float_pair (the gather's float pair of a double from its bits) against the two conversions it stands for,
// hi = (float)q and lo = (float)(q - (double)hi), bit for bit (NaN against NaN), for n values; returns the
// number of disagreements.
extern "C" int64_t float_pair_probe(const double* q, int64_t n) {
  int64_t bad = 0;
  for (int64_t t = 0; t < n; t++) {
    float hi, lo;
    clm::float_pair(q[t], hi, lo);
    const float wh = (float)q[t], wl = (float)(q[t] - (double)wh);
    uint32_t a, b, c, d;
    std::memcpy(&a, &hi, 4);
    std::memcpy(&b, &wh, 4);
    std::memcpy(&c, &lo, 4);
    std::memcpy(&d, &wl, 4);
    const bool ok_hi = std::isnan(wh) ? std::isnan(hi) : a == b;
    const bool ok_lo = std::isnan(wl) ? std::isnan(lo) : c == d;
    if (!ok_hi || !ok_lo) bad++;
  }
  return bad;
}

// The shaped wrap (wrap_point with the cell's shape: exact-zero terms skipped, the full sums where that might
// not be exact) against the general wrap, bit for bit, for n points of one 3D periodic geometry; returns
// the number of disagreements (NaN against NaN), -1 if the geometry has the general shape, or -2 - status.
// *shape receives the geometry's shape.
extern "C" int64_t wrap_shape_probe(int kind, const double* Mcol, double cutoff, const double* x, int64_t n,
                                    int* shape) {
  double M[3][3] = {};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) M[i][j] = (kind == clm::ORTHO && i != j) ? 0.0 : Mcol[j * 3 + i];
  clm::Geometry<double> g;
  const int st = clm::make_geometry<double>(g, 3, kind, M, cutoff, 1, nullptr);
  if (st) return -2 - st;
  clm::DevGeom<double> d;
  clm::fill_devgeom<double>(g, 1, d);
  *shape = d.shape;
  if (d.shape == clm::kShapeGeneral) return -1;
  int64_t bad = 0;
  for (int64_t t = 0; t < n; t++) {
    double a[3], b[3];
    clm::wrap_point<double, 3>(d, x + 3 * t, a);
    if (d.shape == clm::kShapeDiag) clm::wrap_point<double, 3, clm::kShapeDiag>(d, x + 3 * t, b);
    else clm::wrap_point<double, 3, clm::kShapeUpper>(d, x + 3 * t, b);
    for (int k = 0; k < 3; k++)
      if (std::isnan(a[k]) ? !std::isnan(b[k]) : clm::dbits(a[k]) != clm::dbits(b[k])) {
        bad++;
        break;
      }
  }
  return bad;
}

// first_key_at_least (the image tests' thresholds) on arbitrary (s, b): the returned key q must pass,
// RN(value(q) + s) >= b, and the key below it must not (unless q is key(-inf)), in the handle dtype; returns
// the number of violations.
extern "C" int64_t first_key_probe(int f64, const double* s, const double* b, int64_t n) {
  int64_t bad = 0;
  for (int64_t t = 0; t < n; t++) {
    if (f64) {
      const double ss = s[t], bb = b[t];
      const long long q = clm::first_key_at_least<double>(ss, bb);
      const bool at = clm::from_order_key<double>(q) + ss >= bb;
      const bool below = q > clm::order_key(-std::numeric_limits<double>::infinity()) &&
                         clm::from_order_key<double>(q - 1) + ss >= bb;
      if (!at || below) bad++;
    } else {
      const float ss = (float)s[t], bb = (float)b[t];
      const int q = clm::first_key_at_least<float>(ss, bb);
      const bool at = clm::from_order_key<float>(q) + ss >= bb;
      const bool below = q > clm::order_key(-std::numeric_limits<float>::infinity()) &&
                         clm::from_order_key<float>(q - 1) + ss >= bb;
      if (!at || below) bad++;
    }
  }
  return bad;
}
