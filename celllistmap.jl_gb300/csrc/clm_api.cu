// C ABI of libcelllist_cuda.so (declared in include/celllistmap_gb300.h).
//
// The handle plays the role of the reference's ParticleSystem private data
// (src/API/ParticleSystem.jl:142-174, src/internals/ParticleSystem.jl:129-224):
// it owns the positions, the Box and the cell lists, rebuilds the lists lazily
// when positions, box or cutoff changed (the `updated` flag of
// ParticleSystemPositions, src/API/ParticleSystemPositions.jl:14-22), and runs
// one built-in operator per clm_run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "celllistmap_gb300.h"
#include "clm_internal.hpp"

using namespace clm;

namespace {

inline int fail(Handle* h, int code, const char* msg) {
  if (h) h->last_error = msg;
  return code;
}

__global__ void k_nl_export(const int* __restrict__ ni, const int* __restrict__ nj, int64_t n, int base,
                            int64_t* __restrict__ oi, int64_t* __restrict__ oj) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  oi[t] = (int64_t)ni[t] + base;
  oj[t] = (int64_t)nj[t] + base;
}

template <class T> void set_geom_matrix(const Handle& h, T M[3][3]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) M[i][j] = 0;
  for (int i = 0; i < h.dim; i++)
    for (int j = 0; j < h.dim; j++) {
      T v = (T)h.M[j * h.dim + i];
      if (h.kind == CLM_ORTHO && i != j) v = 0;
      M[i][j] = v;
    }
}

template <class T> Geometry<T>& geom(Handle& h);
template <> Geometry<double>& geom<double>(Handle& h) { return h.gd; }
template <> Geometry<float>& geom<float>(Handle& h) { return h.gf; }

template <class T> int compute_periodic_geometry(Handle& h) {
  T M[3][3];
  set_geom_matrix<T>(h, M);
  Geometry<T> g;
  int st = make_geometry<T>(g, h.dim, h.kind, M, (T)h.cutoff, h.lcell, nullptr);
  if (st == 2) return fail(&h, ERR_CELL_TOO_SMALL, "Unit cell matrix does not satisfy required conditions "
                                                   "(distance between cell planes must exceed twice the cutoff).");
  if (st) return fail(&h, st, "invalid box");
  geom<T>(h) = g;
  return OK;
}

template <class T> bool same_geometry(const Geometry<T>& a, const Geometry<T>& b) {
  if (a.dim != b.dim || a.kind != b.kind || a.lcell != b.lcell) return false;
  for (int i = 0; i < 3; i++) {
    if (a.nc[i] != b.nc[i] || a.cs[i] != b.cs[i] || a.cbmin[i] != b.cbmin[i] || a.cbmax[i] != b.cbmax[i]) return false;
  }
  return a.cutoff == b.cutoff;
}

template <class T> int build_all(Handle& h, bool sync) {
  if (!h.box_set) return fail(&h, ERR_STATE, "clm_set_box must be called before building");
  for (int attempt = 0; attempt < 3; attempt++) {
    if (attempt > 0) CLM_CUDA_TRY(h, cudaMemsetAsync(h.err.p, 0, 64, h.stream));  // drop the overflow flag
    cudaEventRecord(h.ev[0], h.stream);
    bool rebuild_all = false;
    if (h.kind == CLM_NONPERIODIC) {
      bool any_dirty = false;
      for (int s = 0; s < h.nsets; s++) any_dirty = any_dirty || h.sets[s].dirty || !h.sets[s].built;
      if (any_dirty) {
        T lo[3], hi[3], M[3][3], origin[3] = {0, 0, 0};
        int st = set_limits<T>(h, lo, hi);
        if (st) return st;
        for (int d = 0; d < h.dim; d++)
          if (std::isnan((double)lo[d]) || std::isnan((double)hi[d]))
            return fail(&h, ERR_NAN, "Invalid coordinates found (NaN) in the particle positions.");
        nonperiodic_cell<T>(h.dim, lo, hi, (T)h.cutoff, M, origin);
        Geometry<T> g;
        st = make_geometry<T>(g, h.dim, CLM_NONPERIODIC, M, (T)h.cutoff, h.lcell, origin);
        if (st == 2) return fail(&h, ERR_CELL_TOO_SMALL, "Unit cell matrix does not satisfy required conditions.");
        if (st) return fail(&h, st, "invalid non-periodic box");
        if (!same_geometry(g, geom<T>(h))) rebuild_all = true;
        geom<T>(h) = g;
      }
    }
    for (int s = 0; s < h.nsets; s++) {
      SetData& S = h.sets[s];
      if (S.dirty || !S.built || rebuild_all) {
        int st = build_set<T>(h, s, geom<T>(h));
        if (st) return st;
      }
    }
    cudaEventRecord(h.ev[1], h.stream);
    if (!sync) {
      h.build_timing_pending = true;
      return OK;
    }
    int st = enqueue_build_totals(h);
    if (st) return st;
    CLM_CUDA_TRY(h, cudaStreamSynchronize(h.stream));
    cudaEventElapsedTime(&h.build_ms, h.ev[0], h.ev[1]);
    h.build_timing_pending = false;
    bool overflow = false;
    st = check_build_totals(h, &overflow);
    if (st) return st;
    if (!overflow) return OK;
  }
  return fail(&h, ERR_INTERNAL,
              "cell-list build did not converge on a copy capacity (particles and their periodic images may exceed "
              "2^31 - 1)");
}

int build_dispatch(Handle& h, bool sync = true) {
  return h.dtype == CLM_F64 ? build_all<double>(h, sync) : build_all<float>(h, sync);
}

// A build enqueued by clm_run is checked (copy totals, NaN and overflow bits of the error word) together
// with the map's results.  When that run returned early (an invalid argument), the set is still pending
// and its error bits unread: the next call rebuilds it instead of trusting it.
void drop_unchecked_builds(Handle& h) {
  for (int s = 0; s < h.nsets; s++) {
    if (h.sets[s].pending) {
      h.sets[s].pending = false;
      h.sets[s].dirty = true;
    }
  }
}

}  // namespace

struct clm_handle_s : public Handle {};

extern "C" {

const char* clm_version(void) { return "celllistmap-gb300 0.1.0 (sm_103a)"; }

int32_t clm_create(int32_t dtype, int32_t dim, int32_t nsets, clm_handle* out) {
  if (!out) return ERR_ARG;
  *out = nullptr;
  if ((dtype != CLM_F32 && dtype != CLM_F64) || (dim != 2 && dim != 3) || (nsets != 1 && nsets != 2)) return ERR_ARG;
  clm_handle h = new (std::nothrow) clm_handle_s();
  if (!h) return ERR_NOMEM;
  h->dtype = dtype;
  h->dim = dim;
  h->nsets = nsets;
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return ERR_CUDA;
  }
  h->own_stream = true;
  if (cudaMallocHost((void**)&h->pinned, 256) != cudaSuccess ||
      cudaMallocHost((void**)&h->pres, clm::kResultBytes) != cudaSuccess || !h->err.reserve(64)) {
    if (h->pinned) cudaFreeHost(h->pinned);
    if (h->pres) cudaFreeHost(h->pres);
    cudaStreamDestroy(h->stream);
    delete h;
    return ERR_CUDA;
  }
  cudaMemset(h->err.p, 0, 64);
  for (auto& e : h->ev) cudaEventCreate(&e);
  *out = h;
  return OK;
}

int32_t clm_destroy(clm_handle h) {
  if (!h) return ERR_ARG;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->pinned) cudaFreeHost(h->pinned);
  if (h->pres) cudaFreeHost(h->pres);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return OK;
}

int32_t clm_set_stream(clm_handle h, void* stream) {
  if (!h) return ERR_ARG;
  cudaStreamSynchronize(h->stream);
  if (stream == nullptr) {
    if (!h->own_stream) {
      if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) return ERR_CUDA;
      h->own_stream = true;
    }
    return OK;
  }
  if (h->own_stream) cudaStreamDestroy(h->stream);
  h->stream = (cudaStream_t)stream;
  h->own_stream = false;
  return OK;
}

int32_t clm_set_box(clm_handle h, const double* M, int32_t kind, double cutoff, int32_t lcell) {
  if (!h) return ERR_ARG;
  if (h->batch.on) return fail(h, ERR_STATE, "a batch handle takes clm_batched_set_systems / clm_batched_run");
  if (lcell < 1) return fail(h, ERR_LCELL, "lcell must be greater or equal to 1");
  if (!(cutoff > 0) || !std::isfinite(cutoff)) return fail(h, ERR_ARG, "cutoff must be a positive finite number");
  if (kind != CLM_ORTHO && kind != CLM_TRICLINIC && kind != CLM_NONPERIODIC) return fail(h, ERR_ARG, "unknown cell kind");
  if (h->box_set && h->kind == CLM_NONPERIODIC && kind != CLM_NONPERIODIC)
    return fail(h, ERR_NONPERIODIC_CELL, "Manual updating of the unit cell of non-periodic systems is not allowed.");
  if (kind != CLM_NONPERIODIC) {
    if (!M) return fail(h, ERR_ARG, "unit cell matrix required");
    for (int k = 0; k < h->dim * h->dim; k++)
      if (!std::isfinite(M[k])) return fail(h, ERR_ARG, "unit cell must be finite");
  }
  int old_kind = h->kind, old_lcell = h->lcell;
  double old_cut = h->cutoff;
  double oldM[9];
  std::memcpy(oldM, h->M, sizeof(oldM));
  h->kind = kind;
  h->lcell = lcell;
  h->cutoff = cutoff;
  std::memset(h->M, 0, sizeof(h->M));
  if (M) std::memcpy(h->M, M, sizeof(double) * h->dim * h->dim);
  if (kind != CLM_NONPERIODIC) {
    int st = (h->dtype == CLM_F64) ? compute_periodic_geometry<double>(*h) : compute_periodic_geometry<float>(*h);
    if (st) {
      h->kind = old_kind;
      h->lcell = old_lcell;
      h->cutoff = old_cut;
      std::memcpy(h->M, oldM, sizeof(oldM));
      return st;
    }
  }
  h->box_set = true;
  for (int s = 0; s < h->nsets; s++) h->sets[s].dirty = true;
  h->nl_valid = false;
  return OK;
}

int32_t clm_set_positions(clm_handle h, int32_t set, const void* xyz, int64_t n, int32_t is_device) {
  if (!h) return ERR_ARG;
  if (set < 0 || set >= h->nsets) return fail(h, ERR_ARG, "set index out of range");
  if (n < 0 || n >= ((int64_t)1 << 27)) return fail(h, ERR_ARG, "number of particles must be in [0, 2^27)");
  if (n > 0 && !xyz) return fail(h, ERR_ARG, "null positions");
  SetData& S = h->sets[set];
  const size_t es = (h->dtype == CLM_F64) ? 8 : 4;
  const size_t bytes = es * (size_t)h->dim * (size_t)n;
  if (!S.x.reserve(bytes + 16)) return fail(h, ERR_NOMEM, "device allocation failed (positions)");
  if (n > 0) {
    if (is_device) {
      CLM_CUDA_TRY(*h, cudaMemcpyAsync(S.x.p, xyz, bytes, cudaMemcpyDeviceToDevice, h->stream));
    } else {
      CLM_CUDA_TRY(*h, cudaMemcpyAsync(S.x.p, xyz, bytes, cudaMemcpyHostToDevice, h->stream));
      cudaPointerAttributes attr;
      if (cudaPointerGetAttributes(&attr, xyz) == cudaSuccess && attr.type == cudaMemoryTypeHost) {
        // pinned source: finish reading it before returning (host pointers are not retained)
        CLM_CUDA_TRY(*h, cudaStreamSynchronize(h->stream));
      }
      cudaGetLastError();
    }
  }
  S.n = n;
  S.dirty = true;
  h->nl_valid = false;
  return OK;
}

int32_t clm_set_precision(clm_handle h, int32_t precision) {
  if (!h) return ERR_ARG;
  if (precision != CLM_PREC_EXACT && precision != CLM_PREC_SPLIT) return fail(h, ERR_ARG, "unknown precision form");
  h->precision = precision;
  return OK;
}

int32_t clm_build(clm_handle h) {
  if (!h) return ERR_ARG;
  if (h->batch.on) return fail(h, ERR_STATE, "a batch handle takes clm_batched_set_systems / clm_batched_run");
  drop_unchecked_builds(*h);
  cudaMemsetAsync(h->err.p, 0, 64, h->stream);
  return build_dispatch(*h);
}

int32_t clm_run(clm_handle h, int32_t op_id, const clm_op_params* params, clm_outputs* out) {
  if (!h || !out) return ERR_ARG;
  if (h->batch.on) return fail(h, ERR_STATE, "a batch handle takes clm_batched_set_systems / clm_batched_run");
  if (!h->box_set) return fail(h, ERR_STATE, "clm_set_box must be called before clm_run");
  drop_unchecked_builds(*h);
  for (int attempt = 0; attempt < 3; attempt++) {
    bool need = false;
    for (int s = 0; s < h->nsets; s++) need = need || h->sets[s].dirty || !h->sets[s].built;
    cudaMemsetAsync(h->err.p, 0, 64, h->stream);
    if (need) {
      // enqueued without waiting for the device; its totals are checked with the map's results
      int st = build_dispatch(*h, false);
      if (st) return st;
    }
    h->nl_valid = false;
    int st = (h->dtype == CLM_F64) ? run_pairs<double>(*h, h->gd, op_id, params, out)
                                   : run_pairs<float>(*h, h->gf, op_id, params, out);
    if (st != RERUN_BUILD) return st;
  }
  return fail(h, ERR_INTERNAL, "cell-list build did not converge on a copy capacity");
}

int32_t clm_nl_count(clm_handle h, int64_t* n) {
  if (!h || !n) return ERR_ARG;
  if (!h->nl_valid) return fail(h, ERR_STATE, "no neighbour list: run CLM_OP_NL first");
  *n = h->nl_n;
  return OK;
}

int32_t clm_nl_fetch(clm_handle h, int64_t* i, int64_t* j, void* d, int64_t cap, int32_t index_base,
                     int32_t out_on_device) {
  if (!h) return ERR_ARG;
  if (!h->nl_valid) return fail(h, ERR_STATE, "no neighbour list: run CLM_OP_NL first");
  if (cap < h->nl_n) return fail(h, ERR_CAPACITY, "output capacity smaller than the number of pairs");
  const int64_t n = h->nl_n;
  if (n == 0) return OK;
  const size_t es = (h->dtype == CLM_F64) ? 8 : 4;
  if (out_on_device) {
    k_nl_export<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(h->nl_i.as<int>(), h->nl_j.as<int>(), n, index_base,
                                                                      i, j);
    CLM_CUDA_TRY(*h, cudaGetLastError());
    if (d) CLM_CUDA_TRY(*h, cudaMemcpyAsync(d, h->nl_d.p, es * n, cudaMemcpyDeviceToDevice, h->stream));
    CLM_CUDA_TRY(*h, cudaStreamSynchronize(h->stream));
    return OK;
  }
  std::vector<int> ti((size_t)n), tj((size_t)n);
  CLM_CUDA_TRY(*h, cudaMemcpyAsync(ti.data(), h->nl_i.p, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
  CLM_CUDA_TRY(*h, cudaMemcpyAsync(tj.data(), h->nl_j.p, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
  if (d) CLM_CUDA_TRY(*h, cudaMemcpyAsync(d, h->nl_d.p, es * n, cudaMemcpyDeviceToHost, h->stream));
  CLM_CUDA_TRY(*h, cudaStreamSynchronize(h->stream));
  for (int64_t k = 0; k < n; k++) {
    if (i) i[k] = (int64_t)ti[(size_t)k] + index_base;
    if (j) j[k] = (int64_t)tj[(size_t)k] + index_base;
  }
  return OK;
}

int32_t clm_get_box(clm_handle h, int64_t* nc, double* cell_size, double* cbmin, double* cbmax, double* aligned,
                    double* rotation, double* inv_rotation, double* cutoff) {
  if (!h) return ERR_ARG;
  if (h->batch.on) return fail(h, ERR_STATE, "a batch handle takes clm_batched_set_systems / clm_batched_run");
  if (!h->box_set) return fail(h, ERR_STATE, "box not set");
  if (h->kind == CLM_NONPERIODIC) {
    bool built = true;
    for (int s = 0; s < h->nsets; s++) built = built && h->sets[s].built && !h->sets[s].dirty;
    if (!built) {
      int st = build_dispatch(*h);
      if (st) return st;
    }
  }
  auto emit = [&](auto& g) {
    const int n = h->dim;
    for (int a = 0; a < n; a++) {
      if (nc) nc[a] = g.nc[a];
      if (cell_size) cell_size[a] = (double)g.cs[a];
      if (cbmin) cbmin[a] = (double)g.cbmin[a];
      if (cbmax) cbmax[a] = (double)g.cbmax[a];
      for (int b = 0; b < n; b++) {
        if (aligned) aligned[b * n + a] = (double)g.Mal[a][b];
        if (rotation) rotation[b * n + a] = (double)g.R[a][b];
        if (inv_rotation) inv_rotation[b * n + a] = (double)g.Rinv[a][b];
      }
    }
    if (cutoff) *cutoff = (double)g.cutoff;
  };
  if (h->dtype == CLM_F64) emit(h->gd);
  else emit(h->gf);
  return OK;
}

int32_t clm_get_celllist_info(clm_handle h, int32_t set, int64_t* n_real, int64_t* n_particles,
                              int64_t* n_cells_with_particles, int64_t* n_cells_with_real) {
  if (!h || set < 0 || set >= h->nsets) return ERR_ARG;
  if (h->batch.on) return fail(h, ERR_STATE, "a batch handle takes clm_batched_set_systems / clm_batched_run");
  SetData& S = h->sets[set];
  if (!S.built || S.dirty) {
    int st = clm_build(h);
    if (st) return st;
  }
  if (n_real) *n_real = S.n;
  if (n_particles) *n_particles = S.n_copies;
  if (n_cells_with_real) *n_cells_with_real = S.n_real_cells;
  if (n_cells_with_particles) {
    std::vector<int> cs((size_t)S.ncells + 1);
    CLM_CUDA_TRY(*h, cudaMemcpyAsync(cs.data(), S.cell_start.p, sizeof(int) * cs.size(), cudaMemcpyDeviceToHost, h->stream));
    CLM_CUDA_TRY(*h, cudaStreamSynchronize(h->stream));
    int64_t c = 0;
    for (int64_t k = 0; k < S.ncells; k++) c += (cs[(size_t)k + 1] > cs[(size_t)k]);
    *n_cells_with_particles = c;
  }
  return OK;
}

int32_t clm_fetch_celllist(clm_handle h, int32_t set, int64_t cap, int64_t* cell, int64_t* index, int8_t* real,
                           void* coords, int32_t index_base) {
  if (!h || set < 0 || set >= h->nsets) return ERR_ARG;
  if (h->batch.on) return fail(h, ERR_STATE, "a batch handle takes clm_batched_set_systems / clm_batched_run");
  SetData& S = h->sets[set];
  if (!S.built || S.dirty) {
    int st = clm_build(h);
    if (st) return st;
  }
  const int64_t n = S.n_copies;
  if (cap < n) return fail(h, ERR_CAPACITY, "capacity smaller than the number of copies");
  if (n == 0) return OK;
  const size_t es = (h->dtype == CLM_F64) ? 8 : 4;
  std::vector<int> cs((size_t)S.ncells + 1), code((size_t)n);
  std::vector<char> xs(es * n), ys(es * n), zs(es * n);
  CLM_CUDA_TRY(*h, cudaMemcpyAsync(cs.data(), S.cell_start.p, sizeof(int) * cs.size(), cudaMemcpyDeviceToHost, h->stream));
  CLM_CUDA_TRY(*h, cudaMemcpyAsync(code.data(), S.code.p, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
  CLM_CUDA_TRY(*h, cudaMemcpyAsync(xs.data(), S.px.p, es * n, cudaMemcpyDeviceToHost, h->stream));
  CLM_CUDA_TRY(*h, cudaMemcpyAsync(ys.data(), S.py.p, es * n, cudaMemcpyDeviceToHost, h->stream));
  if (h->dim == 3) CLM_CUDA_TRY(*h, cudaMemcpyAsync(zs.data(), S.pz.p, es * n, cudaMemcpyDeviceToHost, h->stream));
  CLM_CUDA_TRY(*h, cudaStreamSynchronize(h->stream));
  for (int64_t c = 0; c < S.ncells; c++)
    for (int64_t t = cs[(size_t)c]; t < cs[(size_t)c + 1]; t++) {
      if (cell) cell[t] = c;
      int v = code[(size_t)t];
      if (index) index[t] = (int64_t)(v >= 0 ? v : -v - 1) + index_base;
      if (real) real[t] = v >= 0 ? 1 : 0;
      if (coords) {
        char* dst = (char*)coords + es * (size_t)(t * h->dim);
        std::memcpy(dst, xs.data() + es * t, es);
        std::memcpy(dst + es, ys.data() + es * t, es);
        if (h->dim == 3) std::memcpy(dst + 2 * es, zs.data() + es * t, es);
      }
    }
  return OK;
}

int32_t clm_last_timings(clm_handle h, float* build_ms, float* map_ms) {
  if (!h) return ERR_ARG;
  if (build_ms) *build_ms = h->build_ms;
  if (map_ms) *map_ms = h->map_ms;
  return OK;
}

int32_t clm_stats(clm_handle h, int64_t* kernel_launches) {
  if (!h || !kernel_launches) return ERR_ARG;
  *kernel_launches = h->launches;
  return OK;
}

int32_t clm_last_error(clm_handle h, char* buf, size_t n) {
  if (!h || !buf || n == 0) return ERR_ARG;
  std::strncpy(buf, h->last_error.c_str(), n - 1);
  buf[n - 1] = 0;
  return OK;
}

}  // extern "C"
