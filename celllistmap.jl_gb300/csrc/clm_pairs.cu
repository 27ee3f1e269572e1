// Cell-pair map on the GPU, host side: operator staging, launches, reductions and results.
//
// Replaces _pairwise! and its inner loops:
//   self  src/internals/self.jl:106-184      cross src/internals/cross.jl:81-129
//   vicinal cells with projection culling    src/internals/vicinal_cells.jl:4-75,
//                                            src/internals/auxiliary_functions.jl:66-111
//   non-periodic inner loops                 src/internals/NonPeriodicCells.jl:281-352
// and the per-batch output copies + reduce_output! with on-chip reductions.
//
// Work decomposition: one warp per cell (or part of a cell) that contains real
// particles (the reference's batches of `cell_indices_real`).  The warp's lanes hold the
// particles of that cell (split into 1, 2 or 4 lane groups for small cells so
// that each group takes every G-th neighbour); the particles of each cell of
// the stencil are staged 32 at a time in shared memory and broadcast.
//
// Pair rules are the reference's: orthorhombic self = same cell (later slot,
// at least one real) + forward half stencil (at least one real); triclinic self
// = full stencil, real i, index(i) < index(j); cross = full stencil, real i in
// the same cell, (real i or real j) in vicinal orthorhombic cells; non-periodic
// = forward stencil, no realness rules.  Vicinal cells apply the projection
// filter |(x_j - c_i).u| <= margin and |proj_j - proj_i| <= cutoff with the
// reference's arithmetic.
//
// Exact form (CLM_PREC_EXACT): FP32 distances from cell-relative offsets
// discard pairs that are certainly outside the cutoff (a band of 2^-13 relative
// covers the FP32 error); every remaining candidate is re-tested with the
// reference's arithmetic in the input dtype, so the pair set and d are bit-exact.
// Split form (CLM_PREC_SPLIT): pairs certainly inside are accepted from the
// FP32 test and evaluated in FP32; only the band is re-tested in the input
// dtype.  Energies are summed per lane in the pair-value precision over one
// particle chunk, then in FP64; forces are summed with atomics (16-byte FP32
// records, or FP64 components) and converted to the output dtype afterwards.
//
// Cells holding many particles are split into parts (interleaved chunks of 32
// particles) so that every resident warp has work; batches of independent
// systems share one launch, each cell reading its system's geometry.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "clm_internal.hpp"
#include "clm_pairs_args.hpp"
#include "celllistmap_gb300.h"

namespace clm {

using namespace pk;

namespace {

template <class T> __global__ void k_to_f32(const T* __restrict__ in, int64_t n, float* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

// Fixed-order reductions of the per-block partials (deterministic results).
__global__ void k_reduce_scalar(const double* __restrict__ pe, const unsigned long long* __restrict__ pc, int nb,
                                double* __restrict__ out_e, unsigned long long* __restrict__ out_c) {
  __shared__ double se[256];
  __shared__ unsigned long long sc[256];
  double e = 0;
  unsigned long long c = 0;
  for (int b = threadIdx.x; b < nb; b += 256) {
    e += pe[b];
    c += pc[b];
  }
  se[threadIdx.x] = e;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      se[threadIdx.x] += se[threadIdx.x + s];
      sc[threadIdx.x] += sc[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *out_e = se[0];
    *out_c = sc[0];
  }
}

template <class T>
__global__ void k_reduce_min(const T* __restrict__ pd, const int* __restrict__ pij, int nb, T* out_d, int* out_ij) {
  if (threadIdx.x != 0) return;
  T bd = INFINITY;
  int bi = 0x7fffffff, bj = 0x7fffffff;
  for (int b = 0; b < nb; b++) {
    T d = pd[b];
    int i = pij[2 * b], j = pij[2 * b + 1];
    if (d < bd || (d == bd && (i < bi || (i == bi && j < bj)))) {
      bd = d;
      bi = i;
      bj = j;
    }
  }
  *out_d = bd;
  out_ij[0] = bi;
  out_ij[1] = bj;
}

__global__ void k_reduce_vec(const double* __restrict__ pv, int nb, int k, double* __restrict__ out) {
  const int c = threadIdx.x;
  if (c >= k) return;
  double s = 0;
  for (int b = 0; b < nb; b++) s += pv[(int64_t)b * k + c];
  out[c] = s;
}

__global__ void k_reduce_hist(const unsigned long long* __restrict__ pc, const double* __restrict__ ps, int nb,
                              int nbins, unsigned long long* oc, double* os) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  unsigned long long c = 0;
  double s = 0;
  for (int k = 0; k < nb; k++) {
    c += pc[(int64_t)k * nbins + b];
    s += ps[(int64_t)k * nbins + b];
  }
  oc[b] = c;
  os[b] = s;
}

// forces: sums (rotated frame; 16-byte FP32 records or FP64 components) -> output dtype in the original
// frame
template <class T, int N, class FA>
__global__ void k_forces_out(const FA* __restrict__ facc, int64_t n, DevGeom<T> g, int rotate, T* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // FP32 sums are rotated in FP32 (the FP64 pipe is slow on this part); FP64 sums in FP64
  using R = typename std::conditional<std::is_same<FA, float4>::value, float, double>::type;
  R f[N];
  if constexpr (std::is_same<FA, float4>::value) {
    const float4 v = facc[i];
    f[0] = v.x;
    f[1] = v.y;
    if (N == 3) f[N - 1] = v.z;
  } else {
#pragma unroll
    for (int d = 0; d < N; d++) f[d] = facc[i * N + d];
  }
  if (rotate) {
    R r[N];
#pragma unroll
    for (int a = 0; a < N; a++) {
      R s = 0;
#pragma unroll
      for (int k = 0; k < N; k++) s += (R)g.Rinv[a][k] * f[k];
      r[a] = s;
    }
#pragma unroll
    for (int d = 0; d < N; d++) f[d] = r[d];
  }
#pragma unroll
  for (int d = 0; d < N; d++) out[i * N + d] = (T)f[d];
}


}  // namespace

// Estimated number of pairs assuming uniform density (src/internals/neighborlist.jl:43-58)
static double estimated_pairs(const Handle& h, double vol) {
  const double pi = 3.14159265358979323846;
  double sph = (h.dim == 2 ? pi : 4.0 * pi / 3.0) * std::pow(h.cutoff, h.dim);
  double nx = (double)h.sets[0].n;
  if (h.nsets == 1) return std::max(0.0, nx * (nx - 1) / 2 * sph / vol);
  return std::max(0.0, nx * (double)h.sets[1].n * sph / vol);
}

// Parts per cell: cells holding many particles (large cutoff at high density) are split into parts
// that take interleaved particle chunks, so that there are enough work items for every resident warp.
// Each part keeps at least two chunks of 32 particles.
template <class T> int cell_split_for(const Handle& h, const Geometry<T>& g, int opk) {
  (void)opk;
  const double nx = (double)h.sets[0].n;
  double real_cells = 1.0;
  for (int i = 0; i < g.dim; i++) {
    const double inner = (g.kind == NONPERIODIC) ? (double)g.nc[i] : (double)(g.nc[i] - 2 * g.lcell - 1);
    real_cells *= std::max(1.0, inner);
  }
  const double per_cell = nx / real_cells;
  const double warps = 152.0 * 24.0 * 2.0;  // two items per resident warp slot (24 warps per SM)
  int s = (int)std::ceil(warps / real_cells);
  s = std::min(s, (int)(per_cell / 64.0));
  s = std::max(1, std::min(s, 64));
  while (s > 1 && (double)g.ncells() * s >= 2147483647.0) s--;
  return s;
}

template <class T> int run_pairs(Handle& h, const Geometry<T>& g, int op, const void* vparams, void* vout) {
  const clm_op_params* P = static_cast<const clm_op_params*>(vparams);
  clm_outputs* O = static_cast<clm_outputs*>(vout);
  const int opk = opkind_of(op);
  if (opk < 0) {
    h.last_error = "unknown operator id";
    return ERR_ARG;
  }
  const int N = g.dim;
  SetData& X = h.sets[0];
  SetData& Y = (h.nsets == 2) ? h.sets[1] : h.sets[0];
  PairArgs<T> A;
  std::memset(&A, 0, sizeof(A));
  fill_devgeom(g, h.precision, A.g);
  A.X = view_of<T>(X);
  A.Y = view_of<T>(Y);
  A.real_list = X.real_list.as<int>();
  A.n_real_dev = X.real_scan.as<int>() + X.ncells;
  A.self = (h.nsets == 1);
  A.split = (h.precision == 1) && sizeof(T) == 8;  // Float32 inputs: the split form is the exact form
  if (op == 11 && A.split && P && P->bins && P->nbins >= 1 && P->nbins <= 256) {
    // histogram edges finer than the split form's FP32 distance error: run the exact form, so that the
    // bins stay those of the reference
    std::vector<double> edges((size_t)P->nbins + 1);
    if (P->params_on_device)
      CLM_CUDA_TRY(h, cudaMemcpy(edges.data(), P->bins, sizeof(double) * edges.size(), cudaMemcpyDeviceToHost));
    else
      std::copy(P->bins, P->bins + edges.size(), edges.begin());
    if (!split_bins_exact(g, edges.data(), (int)edges.size())) A.split = false;
  }
  A.op = op;
  A.err = h.err.as<int>();
  A.cell_split = cell_split_for(h, g, opk);
  const LaunchSel sel{N, opk, A.self != 0, A.split != 0, false};
  const double c_default = (double)g.cutoff;
  {
    double pp[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; k++) pp[k] = P ? P->p[k] : 0.0;
    if ((op == 6 || op == 7) && pp[0] == 0.0) pp[0] = c_default;
    set_params(A, pp);
  }
  // operator tables staged on the device
  size_t need = 0;
  auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const int64_t nx = X.n, ny = (h.nsets == 2) ? Y.n : 0;
  const bool types = P && (op == 8 || op == 9 || op == 13) && P->ntypes > 0;
  const bool hist = (op == 11);
  const bool weights = (op == 14);
  if (opk == OPK_ADJ) {
    if (h.nsets != 1) {
      h.last_error = "the LJ adjoint is defined for a single set of particles";
      return ERR_ARG;
    }
    if (P && P->ntypes > 2) {
      h.last_error = "the LJ adjoint supports at most 2 particle types";
      return ERR_ARG;
    }
    if (!O->adjoint) {
      h.last_error = "the LJ adjoint needs clm_outputs.adjoint (9 + 2 x type classes doubles)";
      return ERR_ARG;
    }
  }
  if (types) {
    if (!P->types_x || !P->eps_table || !P->sig_table || (h.nsets == 2 && !P->types_y)) {
      h.last_error = "LJ with types needs types_x (types_y), eps_table and sig_table";
      return ERR_ARG;
    }
    need += align(sizeof(int) * nx) + align(sizeof(int) * ny) + 2 * align(sizeof(double) * P->ntypes * P->ntypes) +
            2 * align(sizeof(float) * P->ntypes * P->ntypes);
  }
  if (weights) {
    if (!P || !P->weights_x || (h.nsets == 2 && !P->weights_y)) {
      h.last_error = "WEIGHTED_INV_D needs weights_x (and weights_y for two sets)";
      return ERR_ARG;
    }
    need += align(sizeof(double) * nx) + align(sizeof(double) * ny) + align(sizeof(float) * nx) +
            align(sizeof(float) * ny);
  }
  if (hist) {
    if (!P || P->nbins < 1 || P->nbins > 256 || !P->bins || !P->vel_x || (h.nsets == 2 && !P->vel_y)) {
      h.last_error = "RHIST needs 1..256 bins, bin edges and velocities";
      return ERR_ARG;
    }
    need += align(sizeof(T) * (P->nbins + 1)) + align(sizeof(T) * nx * N) + align(sizeof(T) * ny * N);
    need += align(sizeof(float) * nx * N) + align(sizeof(float) * ny * N);  // FP32 copies (split form)
  }
  if (need && !h.opbuf.reserve(need)) return ERR_NOMEM;
  char* ob = h.opbuf.as<char>();
  size_t at = 0;
  const cudaMemcpyKind k_in = (P && P->params_on_device) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (types) {
    A.ntypes = P->ntypes;
    int* tx = (int*)(ob + at);
    at += align(sizeof(int) * nx);
    int* ty = (int*)(ob + at);
    at += align(sizeof(int) * ny);
    double* et = (double*)(ob + at);
    at += align(sizeof(double) * P->ntypes * P->ntypes);
    double* stb = (double*)(ob + at);
    at += align(sizeof(double) * P->ntypes * P->ntypes);
    CLM_CUDA_TRY(h, cudaMemcpyAsync(tx, P->types_x, sizeof(int) * nx, k_in, h.stream));
    if (ny) CLM_CUDA_TRY(h, cudaMemcpyAsync(ty, P->types_y, sizeof(int) * ny, k_in, h.stream));
    CLM_CUDA_TRY(h, cudaMemcpyAsync(et, P->eps_table, sizeof(double) * P->ntypes * P->ntypes, k_in, h.stream));
    CLM_CUDA_TRY(h, cudaMemcpyAsync(stb, P->sig_table, sizeof(double) * P->ntypes * P->ntypes, k_in, h.stream));
    const int64_t nt2 = (int64_t)P->ntypes * P->ntypes;
    float* etf = (float*)(ob + at);
    at += align(sizeof(float) * nt2);
    float* stf = (float*)(ob + at);
    at += align(sizeof(float) * nt2);
    k_to_f32<double><<<(unsigned)((nt2 + 255) / 256), 256, 0, h.stream>>>(et, nt2, etf);
    k_to_f32<double><<<(unsigned)((nt2 + 255) / 256), 256, 0, h.stream>>>(stb, nt2, stf);
    CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches += 2;
    A.tx = tx;
    A.ty = ty;
    A.eps_t = et;
    A.sig_t = stb;
    A.eps_tf = etf;
    A.sig_tf = stf;
  }
  if (weights) {
    double* wx = (double*)(ob + at);
    at += align(sizeof(double) * nx);
    double* wy = (double*)(ob + at);
    at += align(sizeof(double) * ny);
    float* wxf = (float*)(ob + at);
    at += align(sizeof(float) * nx);
    float* wyf = (float*)(ob + at);
    at += align(sizeof(float) * ny);
    if (nx) CLM_CUDA_TRY(h, cudaMemcpyAsync(wx, P->weights_x, sizeof(double) * nx, k_in, h.stream));
    if (ny) CLM_CUDA_TRY(h, cudaMemcpyAsync(wy, P->weights_y, sizeof(double) * ny, k_in, h.stream));
    if (nx) k_to_f32<double><<<(unsigned)((nx + 255) / 256), 256, 0, h.stream>>>(wx, nx, wxf);
    if (ny) k_to_f32<double><<<(unsigned)((ny + 255) / 256), 256, 0, h.stream>>>(wy, ny, wyf);
    CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches += (nx > 0) + (ny > 0);
    A.wx = wx;
    A.wy = wy;
    A.wxf = wxf;
    A.wyf = wyf;
  }
  if (hist) {
    A.nbins = P->nbins;
    T* bins = (T*)(ob + at);
    at += align(sizeof(T) * (P->nbins + 1));
    T* vx = (T*)(ob + at);
    at += align(sizeof(T) * nx * N);
    T* vy = (T*)(ob + at);
    at += align(sizeof(T) * ny * N);
    // bin edges are given in double; compare in the handle dtype as the reference does
    std::vector<T> b((size_t)P->nbins + 1);
    if (P->params_on_device) {
      std::vector<double> bd((size_t)P->nbins + 1);
      CLM_CUDA_TRY(h, cudaMemcpy(bd.data(), P->bins, sizeof(double) * bd.size(), cudaMemcpyDeviceToHost));
      for (size_t k = 0; k < b.size(); k++) b[k] = (T)bd[k];
    } else {
      for (size_t k = 0; k < b.size(); k++) b[k] = (T)P->bins[k];
    }
    CLM_CUDA_TRY(h, cudaMemcpyAsync(bins, b.data(), sizeof(T) * b.size(), cudaMemcpyHostToDevice, h.stream));
    CLM_CUDA_TRY(h, cudaMemcpyAsync(vx, P->vel_x, sizeof(T) * nx * N, k_in, h.stream));
    if (ny) CLM_CUDA_TRY(h, cudaMemcpyAsync(vy, P->vel_y, sizeof(T) * ny * N, k_in, h.stream));
    A.bins = bins;
    A.vx = vx;
    A.vy = vy;
    if (std::is_same<T, float>::value) {
      A.vxf = reinterpret_cast<const float*>(vx);
      A.vyf = reinterpret_cast<const float*>(vy);
    } else if (A.split) {
      float* fx = (float*)(ob + at);
      at += align(sizeof(float) * nx * N);
      float* fy = (float*)(ob + at);
      at += align(sizeof(float) * ny * N);
      if (nx) k_to_f32<T><<<(unsigned)((nx * N + 255) / 256), 256, 0, h.stream>>>(vx, nx * N, fx);
      if (ny) k_to_f32<T><<<(unsigned)((ny * N + 255) / 256), 256, 0, h.stream>>>(vy, ny * N, fy);
      CLM_CUDA_TRY(h, cudaGetLastError());
      h.launches += (nx > 0) + (ny > 0);
      A.vxf = fx;
      A.vyf = fy;
    }
    CLM_CUDA_TRY(h, cudaStreamSynchronize(h.stream));  // the host vector b goes out of scope
  }
  // grid: static round-robin of real cells over warps (deterministic)
  // the number of real cells is only known on the device: size for all cells (one resident wave at most)
  const int grid_want =
      (int)std::max<int64_t>(1, std::min<int64_t>((X.ncells * A.cell_split + kWarps - 1) / kWarps, 1 << 16));
  int grid = grid_want;
  // partials
  const size_t part_bytes = align(sizeof(double) * grid_want) + align(sizeof(unsigned long long) * grid_want) +
                            align(sizeof(T) * grid_want) + align(sizeof(int) * 2 * grid_want) +
                            (hist ? align(sizeof(unsigned long long) * grid_want * A.nbins) +
                                        align(sizeof(double) * grid_want * A.nbins) : 0) +
                            align(sizeof(double) * kAdjVals * grid_want) + 4 * align(sizeof(double) * 512);
  if (!h.partial.reserve(part_bytes)) return ERR_NOMEM;
  char* pb = h.partial.as<char>();
  at = 0;
  A.part_e = (double*)(pb + at);
  at += align(sizeof(double) * grid_want);
  A.part_c = (unsigned long long*)(pb + at);
  at += align(sizeof(unsigned long long) * grid_want);
  A.part_min_d2 = (T*)(pb + at);
  at += align(sizeof(T) * grid_want);
  A.part_min_ij = (int*)(pb + at);
  at += align(sizeof(int) * 2 * grid_want);
  if (hist) {
    A.part_hc = (unsigned long long*)(pb + at);
    at += align(sizeof(unsigned long long) * grid_want * A.nbins);
    A.part_hs = (double*)(pb + at);
    at += align(sizeof(double) * grid_want * A.nbins);
  }
  A.part_v = (double*)(pb + at);
  at += align(sizeof(double) * kAdjVals * grid_want);
  char* res = pb + at;  // final results
  double* r_e = (double*)res;
  unsigned long long* r_c = (unsigned long long*)(res + 8);
  T* r_md = (T*)(res + 16);
  int* r_mij = (int*)(res + 24);
  unsigned long long* r_hc = (unsigned long long*)(res + 256);
  double* r_hs = (double*)(res + 256 + 8 * 256);
  // outputs
  const bool forces = (opk == OPK_FORCES || opk == OPK_ADJ);
  double* r_v = (double*)(res + 256 + 16 * 256);  // adjoint sums (kAdjVals)
  // forces are summed with atomics (FP32 pair values: 16-byte records; FP64: dim doubles per particle) in
  // the rotated frame and converted to the output after the map
  const bool f4 = !(std::is_same<T, double>::value && !A.split);
  T* dst_x = nullptr;
  T* dst_y = nullptr;
  const size_t acc_bytes = align((f4 ? sizeof(float4) : sizeof(double) * N) * (nx + ny));
  if (forces) {
    if (!h.outbuf.reserve(acc_bytes + sizeof(T) * (nx + ny) * N + 256)) return ERR_NOMEM;
    A.fx = h.outbuf.as<double>();
    A.fy = A.fx + nx * N;
    A.f4x = h.outbuf.as<float4>();
    A.f4y = A.f4x + nx;
    if (!O->out_on_device) {
      // staged after the accumulators when the caller gave host pointers
      dst_x = (T*)(h.outbuf.as<char>() + acc_bytes);
      dst_y = dst_x + nx * N;
    } else {
      dst_x = (T*)O->forces_x;
      dst_y = (T*)O->forces_y;
    }
    CLM_CUDA_TRY(h, cudaMemsetAsync(h.outbuf.p, 0, acc_bytes, h.stream));
  }
  if (opk == OPK_NL) {
    double vol = std::fabs((double)g.det_in);
    int64_t est = (int64_t)(estimated_pairs(h, vol) * 1.15) + 4096;
    if (h.nl_cap < est) h.nl_cap = est;
    if (!h.counters.reserve(64)) return ERR_NOMEM;
    A.nl_count = h.counters.as<unsigned long long>();
  }
  for (int attempt = 0; attempt < 2; attempt++) {
    if (opk == OPK_NL) {
      if (!h.nl_i.reserve(sizeof(int) * h.nl_cap) || !h.nl_j.reserve(sizeof(int) * h.nl_cap) ||
          !h.nl_d.reserve(sizeof(T) * h.nl_cap))
        return ERR_NOMEM;
      A.nl_i = h.nl_i.as<int>();
      A.nl_j = h.nl_j.as<int>();
      A.nl_d = h.nl_d.as<T>();
      A.nl_cap = h.nl_cap;
      CLM_CUDA_TRY(h, cudaMemsetAsync(A.nl_count, 0, sizeof(unsigned long long), h.stream));
    }
    cudaEventRecord(h.ev[2], h.stream);  // brackets the pair kernel alone
    grid = grid_want;
    cudaError_t e = launch_pairs(sel, grid, h.stream, A);
    cudaEventRecord(h.ev[3], h.stream);
    if (e != cudaSuccess) {
      h.last_error = std::string("pair kernel launch failed: ") + cudaGetErrorString(e);
      return ERR_CUDA;
    }
    h.launches++;
    if (opk != OPK_NL) break;
    unsigned long long n_pairs = 0;
    CLM_CUDA_TRY(h, cudaMemcpyAsync(&n_pairs, A.nl_count, sizeof(n_pairs), cudaMemcpyDeviceToHost, h.stream));
    CLM_CUDA_TRY(h, cudaStreamSynchronize(h.stream));
    h.nl_n = (int64_t)n_pairs;
    if ((int64_t)n_pairs <= h.nl_cap) break;
    h.nl_cap = (int64_t)n_pairs + n_pairs / 16 + 1024;  // retry once with the exact size
  }
  if (opk == OPK_ADJ) {
    k_reduce_vec<<<1, 32, 0, h.stream>>>(A.part_v, grid, kAdjVals, r_v);
  } else if (opk == OPK_SCALAR || opk == OPK_FORCES) {
    k_reduce_scalar<<<1, 256, 0, h.stream>>>(A.part_e, A.part_c, grid, r_e, r_c);
  } else if (opk == OPK_MIN) {
    k_reduce_min<T><<<1, 32, 0, h.stream>>>(A.part_min_d2, A.part_min_ij, grid, r_md, r_mij);
  } else if (opk == OPK_HIST) {
    k_reduce_hist<<<(A.nbins + 63) / 64, 64, 0, h.stream>>>(A.part_hc, A.part_hs, grid, A.nbins, r_hc, r_hs);
  }
  CLM_CUDA_TRY(h, cudaGetLastError());
  if (opk != OPK_NL) h.launches++;
  if (forces) {
    const int rot = (g.kind == TRICLINIC) ? 1 : 0;
    DevGeom<T>& dg = A.g;
    h.launches += (nx && dst_x) + (ny && dst_y);
    auto out = [&](int64_t cnt, int64_t first, T* dst) {
      const unsigned blocks = (unsigned)((cnt + 255) / 256);
      if (f4) {
        if (N == 3) k_forces_out<T, 3, float4><<<blocks, 256, 0, h.stream>>>(A.f4x + first, cnt, dg, rot, dst);
        else k_forces_out<T, 2, float4><<<blocks, 256, 0, h.stream>>>(A.f4x + first, cnt, dg, rot, dst);
      } else {
        if (N == 3) k_forces_out<T, 3, double><<<blocks, 256, 0, h.stream>>>(A.fx + first * N, cnt, dg, rot, dst);
        else k_forces_out<T, 2, double><<<blocks, 256, 0, h.stream>>>(A.fx + first * N, cnt, dg, rot, dst);
      }
    };
    if (nx && dst_x) out(nx, 0, dst_x);
    if (ny && dst_y) out(ny, nx, dst_y);
    CLM_CUDA_TRY(h, cudaGetLastError());
    if (!O->out_on_device) {
      if (O->forces_x && nx)
        CLM_CUDA_TRY(h, cudaMemcpyAsync(O->forces_x, dst_x, sizeof(T) * nx * N, cudaMemcpyDeviceToHost, h.stream));
      if (O->forces_y && ny)
        CLM_CUDA_TRY(h, cudaMemcpyAsync(O->forces_y, dst_y, sizeof(T) * ny * N, cudaMemcpyDeviceToHost, h.stream));
    }
  }
  // scalar results (and the totals of a build enqueued without synchronization), into pinned memory: only
  // the part this operator wrote
  const char* hostres = reinterpret_cast<const char*>(h.pres);
  const size_t res_bytes = (opk == OPK_HIST || opk == OPK_ADJ) ? kResultBytes : 32;
  CLM_CUDA_TRY(h, cudaMemcpyAsync(h.pres, res, res_bytes, cudaMemcpyDeviceToHost, h.stream));
  {
    int st = enqueue_build_totals(h);
    if (st) return st;
  }
  CLM_CUDA_TRY(h, cudaStreamSynchronize(h.stream));
  cudaEventElapsedTime(&h.map_ms, h.ev[2], h.ev[3]);
  if (h.build_timing_pending) {
    cudaEventElapsedTime(&h.build_ms, h.ev[0], h.ev[1]);
    h.build_timing_pending = false;
  }
  {
    bool overflow = false;
    int st = check_build_totals(h, &overflow);
    if (st) return st;
    if (overflow) return RERUN_BUILD;
  }
  if (h.pinned[40] & DERR_CELL_RANGE) {
    h.last_error = "pair map consistency check failed (stencil cell outside the grid)";
    return ERR_INTERNAL;
  }
  if (h.pinned[40] & DERR_STAGE) {
    h.last_error = "pair map: a staging wait for bulk copies timed out";
    return ERR_INTERNAL;
  }
  std::memcpy(&O->scalar, hostres, 8);
  unsigned long long cnt;
  std::memcpy(&cnt, hostres + 8, 8);
  O->count = (int64_t)cnt;
  if (opk == OPK_NL) {
    O->count = h.nl_n;
    h.nl_valid = true;
  }
  if (op == 2) O->scalar = (double)cnt;
  if (opk == OPK_MIN) {
    T md;
    int mij[2];
    std::memcpy(&md, hostres + 16, sizeof(T));
    std::memcpy(mij, hostres + 24, 8);
    if (std::isinf((double)md)) {
      O->min_d = INFINITY;
      O->min_i = -1;
      O->min_j = -1;
    } else {
      O->min_d = (double)std::sqrt(md);
      O->min_i = mij[0] + O->index_base;
      O->min_j = mij[1] + O->index_base;
    }
  }
  if (opk == OPK_ADJ) {
    double v[kAdjVals];
    std::memcpy(v, hostres + 256 + 16 * 256, sizeof(v));
    O->scalar = v[0];
    // virial of the rotated frame -> original frame: W = Rinv W' Rinv^T
    double Wp[3][3] = {{v[1], v[4], v[5]}, {v[4], v[2], v[6]}, {v[5], v[6], v[3]}};
    double W[3][3];
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) {
        double acc = 0;
        for (int c = 0; c < 3; c++)
          for (int d = 0; d < 3; d++) {
            double ra = (a < N && c < N) ? (double)g.Rinv[a][c] : (a == c ? 1.0 : 0.0);
            double rb = (b < N && d < N) ? (double)g.Rinv[b][d] : (b == d ? 1.0 : 0.0);
            acc += ra * Wp[c][d] * rb;
          }
        W[a][b] = acc;
      }
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) O->adjoint[a * 3 + b] = W[a][b];
    const int ncls = (P && P->ntypes > 0) ? P->ntypes * (P->ntypes + 1) / 2 : 1;
    for (int k = 0; k < ncls; k++) {
      O->adjoint[9 + k] = v[7 + k];
      O->adjoint[9 + ncls + k] = v[10 + k];
    }
  }
  if (opk == OPK_HIST) {
    if (O->out_on_device) {
      CLM_CUDA_TRY(h, cudaMemcpyAsync(O->hist_count, r_hc, 8 * A.nbins, cudaMemcpyDeviceToDevice, h.stream));
      CLM_CUDA_TRY(h, cudaMemcpyAsync(O->hist_sum, r_hs, 8 * A.nbins, cudaMemcpyDeviceToDevice, h.stream));
    } else {
      if (O->hist_count) std::memcpy(O->hist_count, hostres + 256, 8 * A.nbins);
      if (O->hist_sum) std::memcpy(O->hist_sum, hostres + 256 + 8 * 256, 8 * A.nbins);
    }
  }
  return OK;
}


// Scalar reductions (COUNT, SUM_D2, SUM_D, SUM_INV_D, SOFT_ENERGY, LJ_ENERGY without type tables) and
// MINDIST on an already built handle, with the per-block partials and the final result placed in
// caller-provided device scratch instead of handle buffers.  Allocates nothing; used by clm_run_noalloc.
template <class T>
int run_pairs_scalar_scratch(Handle& h, const Geometry<T>& g, int op, const void* vparams, void* vout, void* scratch,
                             size_t scratch_bytes) {
  const clm_op_params* P = static_cast<const clm_op_params*>(vparams);
  clm_outputs* O = static_cast<clm_outputs*>(vout);
  const int opk = opkind_of(op);
  if (opk != OPK_SCALAR && opk != OPK_MIN) {
    h.last_error = "the allocation-free entry point supports COUNT, SUM_D2, SUM_D, SUM_INV_D, SOFT_ENERGY, "
                   "LJ_ENERGY and MINDIST";
    return ERR_ARG;
  }
  if (P && P->ntypes > 0) {
    h.last_error = "the allocation-free entry point does not take per-type tables";
    return ERR_ARG;
  }
  const int N = g.dim;
  SetData& X = h.sets[0];
  SetData& Y = (h.nsets == 2) ? h.sets[1] : h.sets[0];
  PairArgs<T> A;
  std::memset(&A, 0, sizeof(A));
  fill_devgeom(g, h.precision, A.g);
  A.X = view_of<T>(X);
  A.Y = view_of<T>(Y);
  A.real_list = X.real_list.as<int>();
  A.n_real_dev = X.real_scan.as<int>() + X.ncells;
  A.self = (h.nsets == 1);
  A.split = (h.precision == 1) && sizeof(T) == 8;  // Float32 inputs: the split form is the exact form
  A.op = op;
  A.err = h.err.as<int>();
  A.cell_split = 1;
  const LaunchSel sel{N, opk, A.self != 0, A.split != 0, false};
  {
    double pp[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; k++) pp[k] = P ? P->p[k] : 0.0;
    if (op == 6 && pp[0] == 0.0) pp[0] = (double)g.cutoff;
    set_params(A, pp);
  }
  // scratch layout: [results, 256 B][partial energy][partial count][partial min d2][partial min ij]
  const size_t cap_blocks = noalloc_block_slots(scratch_bytes, sizeof(T));
  const int needed = pairs_scalar_blocks_needed(h, op);
  if (needed < 0 || (size_t)needed > cap_blocks) {
    h.last_error = "the pair map needs more per-block partial slots than the allocation-free scratch holds";
    return ERR_CAPACITY;
  }
  int grid = needed;
  char* base = static_cast<char*>(scratch);
  const size_t nb = cap_blocks;
  A.part_e = (double*)(base + 256);
  A.part_c = (unsigned long long*)(base + 256 + sizeof(double) * nb);
  A.part_min_d2 = (T*)(base + 256 + (sizeof(double) + sizeof(unsigned long long)) * nb);
  A.part_min_ij = (int*)(base + 256 + (sizeof(double) + sizeof(unsigned long long) + sizeof(T)) * nb);
  double* r_e = (double*)base;
  unsigned long long* r_c = (unsigned long long*)(base + 8);
  T* r_md = (T*)(base + 16);
  int* r_mij = (int*)(base + 24);
  cudaError_t e = launch_pairs(sel, grid, h.stream, A);
  if (e != cudaSuccess) {
    h.last_error = std::string("pair kernel launch failed: ") + cudaGetErrorString(e);
    return ERR_CUDA;
  }
  h.launches++;
  if (opk == OPK_SCALAR) k_reduce_scalar<<<1, 256, 0, h.stream>>>(A.part_e, A.part_c, grid, r_e, r_c);
  else k_reduce_min<T><<<1, 32, 0, h.stream>>>(A.part_min_d2, A.part_min_ij, grid, r_md, r_mij);
  CLM_CUDA_TRY(h, cudaGetLastError());
  h.launches++;
  // results through the handle's pinned staging area (allocated when the handle was created)
  CLM_CUDA_TRY(h, cudaMemcpyAsync(h.pinned + 8, base, 32, cudaMemcpyDeviceToHost, h.stream));
  CLM_CUDA_TRY(h, cudaMemcpyAsync(h.pinned + 4, h.err.p, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
  CLM_CUDA_TRY(h, cudaStreamSynchronize(h.stream));
  if (h.pinned[4] & DERR_CELL_RANGE) {
    h.last_error = "pair map consistency check failed (stencil cell outside the grid)";
    return ERR_INTERNAL;
  }
  if (h.pinned[4] & DERR_STAGE) {
    h.last_error = "pair map: a staging wait for bulk copies timed out";
    return ERR_INTERNAL;
  }
  const char* hr = reinterpret_cast<const char*>(h.pinned + 8);
  unsigned long long cnt;
  std::memcpy(&O->scalar, hr, 8);
  std::memcpy(&cnt, hr + 8, 8);
  O->count = (int64_t)cnt;
  if (op == 2) O->scalar = (double)cnt;
  if (opk == OPK_MIN) {
    T md;
    int mij[2];
    std::memcpy(&md, hr + 16, sizeof(T));
    std::memcpy(mij, hr + 24, 8);
    if (std::isinf((double)md)) {
      O->min_d = INFINITY;
      O->min_i = -1;
      O->min_j = -1;
    } else {
      O->min_d = (double)std::sqrt(md);
      O->min_i = mij[0] + O->index_base;
      O->min_j = mij[1] + O->index_base;
    }
  }
  return OK;
}

// Number of per-block partial slots the scalar map needs on this device (one resident wave).
int pairs_scalar_blocks_needed(Handle& h, int op) {
  const int opk = opkind_of(op);
  if (opk != OPK_SCALAR && opk != OPK_MIN) return -1;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const LaunchSel sel{h.dim, opk, h.nsets == 1, h.precision == 1 && h.dtype == 1, false};
  const int per_sm = (h.dtype == 1) ? pairs_blocks_per_sm(sel, (const PairArgs<double>*)nullptr)
                                    : pairs_blocks_per_sm(sel, (const PairArgs<float>*)nullptr);
  if (per_sm <= 0 || sms <= 0) return -1;
  const int64_t want = std::max<int64_t>(1, (h.sets[0].ncells + kWarps - 1) / kWarps);
  return (int)std::min<int64_t>(want, (int64_t)per_sm * sms);
}

template int run_pairs_scalar_scratch<float>(Handle&, const Geometry<float>&, int, const void*, void*, void*, size_t);
template int run_pairs_scalar_scratch<double>(Handle&, const Geometry<double>&, int, const void*, void*, void*, size_t);

template int run_pairs<float>(Handle&, const Geometry<float>&, int, const void*, void*);
template int run_pairs<double>(Handle&, const Geometry<double>&, int, const void*, void*);

}  // namespace clm
