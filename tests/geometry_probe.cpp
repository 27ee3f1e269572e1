// Test infrastructure: exposes the library's host-side box geometry (csrc/clm_geometry.hpp, the code
// clm_set_box runs) through a C entry point so that the CPU tests can compare it with the oracle's
// restatement without a GPU.  Built by tests/test_geometry.py with -ffp-contract=off, as the library is.
#include <cstdint>

#include "clm_geometry.hpp"

namespace {
template <class T>
int run(int dim, int kind, const double* Mcol, double cutoff, int lcell, int64_t* nc, double* cs, double* cbmin,
        double* cbmax, double* mal, double* rot, double* rinv) {
  T M[3][3] = {};
  for (int i = 0; i < dim; i++)
    for (int j = 0; j < dim; j++) {
      T v = (T)Mcol[j * dim + i];  // column-major, as clm_set_box takes it
      if (kind == clm::ORTHO && i != j) v = 0;
      M[i][j] = v;
    }
  clm::Geometry<T> g;
  const int st = clm::make_geometry<T>(g, dim, kind, M, (T)cutoff, lcell, nullptr);
  if (st) return st;
  for (int i = 0; i < dim; i++) {
    nc[i] = g.nc[i];
    cs[i] = (double)g.cs[i];
    cbmin[i] = (double)g.cbmin[i];
    cbmax[i] = (double)g.cbmax[i];
    for (int j = 0; j < dim; j++) {
      mal[j * dim + i] = (double)g.Mal[i][j];
      rot[j * dim + i] = (double)g.R[i][j];
      rinv[j * dim + i] = (double)g.Rinv[i][j];
    }
  }
  return 0;
}
}  // namespace

extern "C" int geom_probe(int f64, int dim, int kind, const double* Mcol, double cutoff, int lcell, int64_t* nc,
                          double* cs, double* cbmin, double* cbmax, double* mal, double* rot, double* rinv) {
  return f64 ? run<double>(dim, kind, Mcol, cutoff, lcell, nc, cs, cbmin, cbmax, mal, rot, rinv)
             : run<float>(dim, kind, Mcol, cutoff, lcell, nc, cs, cbmin, cbmax, mal, rot, rinv);
}
