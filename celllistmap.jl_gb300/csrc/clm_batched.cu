// Batches of independent periodic systems: one cell list over a global cell index, one launch per
// kernel for all systems, per-system results, and the step replayed as a CUDA graph.
//
// The reference runs one ParticleSystem per system (src/API/ParticleSystem.jl:142-202,
// src/API/pairwise.jl:48-63); a batch is the loop over systems in one call.  Every system keeps the
// reference's own Box (src/internals/Box.jl:191-270), images and pair rules, so a system's pairs
// and sums are those of a separate ParticleSystem with the same inputs.
//
// Layout on the device:
//   set 0 of the handle     concatenated positions (n_total x dim) and the global cell list
//   gtab[nsys]              DevGeom of each system (cells, images, cutoff thresholds)
//   psys[n_total]           system of each particle
//   cbase[nsys+1]           first global cell of each system (a failed system has no cells)
//   cell_sys[ncells]        system of each global cell
// The pair kernel writes one partial per work item (cell part); a warp per system then sums the
// partials of its cells in a fixed order, so results do not depend on scheduling.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "celllistmap_gb300.h"
#include "clm_internal.hpp"
#include "clm_pairs_args.hpp"

using namespace clm;
using namespace clm::pk;

struct clm_handle_s : public Handle {};

namespace {

constexpr int kMaxOps = 4;

inline int fail(Handle* h, int code, const char* msg) {
  if (h) h->last_error = msg;
  return code;
}

// Sum of the per-item partials of each system, in item order (deterministic).
__global__ void k_seg_reduce(const double* __restrict__ pe, const unsigned long long* __restrict__ pc, int S,
                             const int* __restrict__ real_scan, const int* __restrict__ cbase, int nsys,
                             double* __restrict__ oe, unsigned long long* __restrict__ oc) {
  const int lane = threadIdx.x & 31;
  const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= nsys) return;
  const int b = real_scan[cbase[s]] * S;
  const int e = real_scan[cbase[s + 1]] * S;
  double acc = 0.0;
  unsigned long long c = 0;
  for (int t = b + lane; t < e; t += 32) {
    acc += pe[t];
    c += pc[t];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_xor_sync(0xffffffffu, acc, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if (lane == 0) {
    oe[s] = acc;
    oc[s] = c;
  }
}

template <class T> Geometry<T>& tmpl_geom(Handle& h);
template <> Geometry<double>& tmpl_geom<double>(Handle& h) { return h.gd; }
template <> Geometry<float>& tmpl_geom<float>(Handle& h) { return h.gf; }

bool batch_op_ok(int op) {
  switch (op) {
    case CLM_OP_NL: case CLM_OP_COUNT: case CLM_OP_SUM_D2: case CLM_OP_SUM_D: case CLM_OP_SUM_INV_D:
    case CLM_OP_SOFT_ENERGY: case CLM_OP_LJ_ENERGY: case CLM_OP_SOFT_FORCES: case CLM_OP_LJ_FORCES:
    case CLM_OP_INV_D_FORCES:
      return true;
  }
  return false;
}

// Per-system geometry tables for the current systems, lcell and precision (host work, then uploads).
template <class T> int batch_tables(Handle& h) {
  BatchState& B = h.batch;
  const int N = h.dim;
  const int64_t nsys = B.nsys;
  std::vector<DevGeom<T>> tab((size_t)nsys);
  B.cbase.assign((size_t)nsys + 1, 0);
  B.status.assign((size_t)nsys, OK);
  B.copies_est = B.pairs_est = B.real_cells = 0;
  const double pi = 3.14159265358979323846;
  const double sph = (N == 2 ? pi : 4.0 * pi / 3.0) * std::pow(B.cutoff, N);
  bool have = false;
  int64_t total = 0;
  for (int64_t s = 0; s < nsys; s++) {
    T M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    const double* c = B.cells.data() + (size_t)s * N * N;
    for (int i = 0; i < N; i++)
      for (int j = 0; j < N; j++) M[i][j] = (B.kind == CLM_ORTHO && i != j) ? T(0) : (T)c[j * N + i];
    Geometry<T> g;
    int st = make_geometry<T>(g, N, B.kind, M, (T)B.cutoff, B.lcell, nullptr);
    std::memset(&tab[(size_t)s], 0, sizeof(DevGeom<T>));
    if (st != 0) {
      B.status[(size_t)s] = (st == 2) ? ERR_CELL_TOO_SMALL : ERR_ARG;
      B.cbase[(size_t)s + 1] = (int)total;
      continue;
    }
    fill_devgeom(g, h.precision, tab[(size_t)s]);
    total += g.ncells();
    if (total >= ((int64_t)1 << 30)) return fail(&h, ERR_ARG, "too many cells in the batch (reduce lcell)");
    B.cbase[(size_t)s + 1] = (int)total;
    const double ns = (double)(B.offsets[(size_t)s + 1] - B.offsets[(size_t)s]);
    double vbox = 1.0, real = 1.0;
    for (int i = 0; i < N; i++) {
      vbox *= (double)g.cbmax[i] - (double)g.cbmin[i];
      real *= std::max(1.0, (double)(g.nc[i] - 2 * g.lcell - 1));
    }
    const double vcell = std::fabs((double)g.det_in);
    B.copies_est += (vcell > 0) ? ns * vbox / vcell : 27.0 * ns;
    B.pairs_est += (vcell > 0) ? ns * (ns - 1) / 2 * sph / vcell : 0.0;
    B.real_cells += real;
    if (!have) {
      tmpl_geom<T>(h) = g;
      have = true;
    }
  }
  if (!have) {
    // no valid system: a template geometry so that the build runs on an empty grid
    T M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int i = 0; i < N; i++) M[i][i] = (T)(4.0 * B.cutoff);
    Geometry<T> g;
    if (make_geometry<T>(g, N, B.kind == CLM_TRICLINIC ? CLM_TRICLINIC : CLM_ORTHO, M, (T)B.cutoff, B.lcell, nullptr))
      return fail(&h, ERR_INTERNAL, "template geometry");
    tmpl_geom<T>(h) = g;
  }
  B.ncells = total;
  const int64_t n = B.offsets[(size_t)nsys];
  std::vector<int> psys((size_t)std::max<int64_t>(n, 1));
  for (int64_t s = 0; s < nsys; s++)
    for (int64_t i = B.offsets[(size_t)s]; i < B.offsets[(size_t)s + 1]; i++) psys[(size_t)i] = (int)s;
  std::vector<int> csys((size_t)std::max<int64_t>(total, 1));
  for (int64_t s = 0; s < nsys; s++)
    for (int c = B.cbase[(size_t)s]; c < B.cbase[(size_t)s + 1]; c++) csys[(size_t)c] = (int)s;
  if (!B.gtab.reserve(sizeof(DevGeom<T>) * (size_t)std::max<int64_t>(nsys, 1)) ||
      !B.psys.reserve(sizeof(int) * psys.size()) || !B.cbase_d.reserve(sizeof(int) * B.cbase.size()) ||
      !B.cell_sys.reserve(sizeof(int) * csys.size()) || !B.sys_err.reserve(sizeof(int) * (size_t)(nsys + 1)))
    return fail(&h, ERR_NOMEM, "device allocation failed (batch tables)");
  CLM_CUDA_TRY(h, cudaStreamSynchronize(h.stream));
  if (nsys) CLM_CUDA_TRY(h, cudaMemcpy(B.gtab.p, tab.data(), sizeof(DevGeom<T>) * tab.size(), cudaMemcpyHostToDevice));
  CLM_CUDA_TRY(h, cudaMemcpy(B.psys.p, psys.data(), sizeof(int) * psys.size(), cudaMemcpyHostToDevice));
  CLM_CUDA_TRY(h, cudaMemcpy(B.cbase_d.p, B.cbase.data(), sizeof(int) * B.cbase.size(), cudaMemcpyHostToDevice));
  CLM_CUDA_TRY(h, cudaMemcpy(B.cell_sys.p, csys.data(), sizeof(int) * csys.size(), cudaMemcpyHostToDevice));
  CLM_CUDA_TRY(h, cudaMemset(B.sys_err.p, 0, sizeof(int) * (size_t)(nsys + 1)));
  const size_t hres = (size_t)kMaxOps * nsys * 16 + 64 + sizeof(int) * (size_t)(nsys + 1);
  if (hres > B.hres_bytes) {
    if (B.hres) cudaFreeHost(B.hres);
    B.hres = nullptr;
    B.hres_bytes = 0;
    if (cudaMallocHost((void**)&B.hres, hres) != cudaSuccess) return fail(&h, ERR_NOMEM, "pinned allocation failed");
    B.hres_bytes = hres;
    alloc_count()++;
    alloc_bytes() += (long long)hres;
  }
  B.tables_ready = true;
  B.tables_dtype = h.dtype;
  h.sets[0].dirty = true;
  return OK;
}

void drop_graph(BatchState& B) {
  if (B.gexec) cudaGraphExecDestroy(B.gexec);
  B.gexec = nullptr;
  B.graph_ops.clear();
  B.graph_params.clear();
  B.graph_n = -1;
}

// Offsets inside the pinned result block.
inline double* hres_sum(BatchState& B, int slot) { return (double*)(B.hres + (size_t)slot * B.nsys * 16); }
inline unsigned long long* hres_cnt(BatchState& B, int slot) {
  return (unsigned long long*)(B.hres + (size_t)slot * B.nsys * 16 + (size_t)B.nsys * 8);
}
inline unsigned long long* hres_nl(BatchState& B) { return (unsigned long long*)(B.hres + (size_t)kMaxOps * B.nsys * 16); }
inline int* hres_err(BatchState& B) { return (int*)(B.hres + (size_t)kMaxOps * B.nsys * 16 + 64); }

// Batch forces: sums (rotated frame of each particle's system) -> output dtype in the original frames.
template <class T, int N, class FA>
__global__ void k_forces_out_b(const FA* __restrict__ facc, int64_t n, const DevGeom<T>* __restrict__ gtab,
                               const int* __restrict__ psys, T* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
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
  const DevGeom<T>& g = gtab[psys[i]];
  if (g.kind == TRICLINIC) {
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

// One operator of the step, enqueued without synchronization.
template <class T> int enqueue_op(Handle& h, int slot, int op, const clm_op_params* P) {
  BatchState& B = h.batch;
  const Geometry<T>& g = tmpl_geom<T>(h);
  const int N = h.dim;
  const int opk = opkind_of(op);
  SetData& X = h.sets[0];
  const int64_t n = X.n;
  const int64_t nsys = B.nsys;
  PairArgs<T> A;
  std::memset(&A, 0, sizeof(A));
  fill_devgeom(g, h.precision, A.g);
  A.X = view_of<T>(X);
  A.Y = A.X;
  A.real_list = X.real_list.as<int>();
  A.n_real_dev = X.real_scan.as<int>() + X.ncells;
  A.self = 1;
  A.split = (h.precision == CLM_PREC_SPLIT) && sizeof(T) == 8;  // Float32: the split form is the exact form
  A.op = op;
  A.err = h.err.as<int>();
  A.cell_split = B.cell_split;
  A.gtab = B.gtab.as<DevGeom<T>>();
  A.cell_sys = B.cell_sys.as<int>();
  A.cbase = B.cbase_d.as<int>();
  {
    double pp[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; k++) pp[k] = P ? P->p[k] : 0.0;
    if ((op == CLM_OP_SOFT_ENERGY || op == CLM_OP_SOFT_FORCES) && pp[0] == 0.0) pp[0] = B.cutoff;
    set_params(A, pp);
  }
  // partials: one per work item (cells with real particles x parts; sized for all cells)
  const int64_t items = std::max<int64_t>(1, B.ncells) * B.cell_split;
  const size_t al = 256;
  auto align = [&](size_t v) { return (v + al - 1) / al * al; };
  if (!B.part.reserve(align(sizeof(double) * items) + align(sizeof(unsigned long long) * items)))
    return fail(&h, ERR_NOMEM, "device allocation failed (partials)");
  A.part_e = B.part.as<double>();
  A.part_c = (unsigned long long*)(B.part.as<char>() + align(sizeof(double) * items));
  if (!B.sys_out.reserve((size_t)kMaxOps * std::max<int64_t>(nsys, 1) * 16 + 64))
    return fail(&h, ERR_NOMEM, "device allocation failed (results)");
  double* o_e = (double*)(B.sys_out.as<char>() + (size_t)slot * nsys * 16);
  unsigned long long* o_c = (unsigned long long*)(B.sys_out.as<char>() + (size_t)slot * nsys * 16 + (size_t)nsys * 8);
  const bool forces = (opk == OPK_FORCES);
  // force sums (rotated frames): 16-byte FP32 records, or dim doubles per particle for FP64 pair values;
  // the systems that failed the cell check keep zero sums
  const bool f4 = !(std::is_same<T, double>::value && !A.split);
  const size_t acc_bytes = align((f4 ? sizeof(float4) : sizeof(double) * N) * (size_t)std::max<int64_t>(n, 1));
  if (forces) {
    if (!h.outbuf.reserve(acc_bytes) || !B.forces.reserve(sizeof(T) * n * N + 256))
      return fail(&h, ERR_NOMEM, "device allocation failed (forces)");
    A.fx = h.outbuf.as<double>();
    A.f4x = h.outbuf.as<float4>();
    CLM_CUDA_TRY(h, cudaMemsetAsync(h.outbuf.p, 0, acc_bytes, h.stream));
  }
  if (opk == OPK_NL) {
    const int64_t est = (int64_t)(B.pairs_est * 1.15) + 4096;
    if (h.nl_cap < est) h.nl_cap = est;
    if (!h.counters.reserve(64) || !h.nl_i.reserve(sizeof(int) * h.nl_cap) || !h.nl_j.reserve(sizeof(int) * h.nl_cap) ||
        !h.nl_d.reserve(sizeof(T) * h.nl_cap))
      return fail(&h, ERR_NOMEM, "device allocation failed (neighbour list)");
    A.nl_count = h.counters.as<unsigned long long>();
    A.nl_i = h.nl_i.as<int>();
    A.nl_j = h.nl_j.as<int>();
    A.nl_d = h.nl_d.as<T>();
    A.nl_cap = h.nl_cap;
    CLM_CUDA_TRY(h, cudaMemsetAsync(A.nl_count, 0, sizeof(unsigned long long), h.stream));
  }
  // one resident wave (divided by the tuned factor)
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const LaunchSel sel{N, opk, true, A.split != 0, true};
  int grid = std::max(1, sms) * 64;
  {
    // resident blocks per SM of this instantiation: probe through the plain scalar kernel of the same
    // shape, then apply the divisor
    int per_sm = pairs_blocks_per_sm(LaunchSel{N, OPK_SCALAR, true, A.split != 0, false}, (const PairArgs<T>*)nullptr);
    if (per_sm <= 0) per_sm = 1;
    grid = std::max(1, per_sm * std::max(1, sms) / std::max(1, B.grid_div));
  }
  if (!h.capturing) cudaEventRecord(h.ev[2], h.stream);
  cudaError_t e = launch_pairs(sel, grid, h.stream, A);
  if (!h.capturing) cudaEventRecord(h.ev[3], h.stream);
  if (e != cudaSuccess) {
    h.last_error = std::string("pair kernel launch failed: ") + cudaGetErrorString(e);
    return ERR_CUDA;
  }
  h.launches++;
  if (forces && n > 0) {
    const unsigned blocks = (unsigned)((n + 255) / 256);
    const DevGeom<T>* gt = B.gtab.as<DevGeom<T>>();
    const int* ps = B.psys.as<int>();
    if (f4) {
      if (N == 3) k_forces_out_b<T, 3, float4><<<blocks, 256, 0, h.stream>>>(A.f4x, n, gt, ps, B.forces.as<T>());
      else k_forces_out_b<T, 2, float4><<<blocks, 256, 0, h.stream>>>(A.f4x, n, gt, ps, B.forces.as<T>());
    } else {
      if (N == 3) k_forces_out_b<T, 3, double><<<blocks, 256, 0, h.stream>>>(A.fx, n, gt, ps, B.forces.as<T>());
      else k_forces_out_b<T, 2, double><<<blocks, 256, 0, h.stream>>>(A.fx, n, gt, ps, B.forces.as<T>());
    }
    CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches++;
  }
  if (opk == OPK_SCALAR || opk == OPK_FORCES || opk == OPK_NL) {
    if (nsys > 0) {
      k_seg_reduce<<<(unsigned)((nsys + 3) / 4), 128, 0, h.stream>>>(A.part_e, A.part_c, B.cell_split,
                                                                   X.real_scan.as<int>(), B.cbase_d.as<int>(),
                                                                   (int)nsys, o_e, o_c);
      CLM_CUDA_TRY(h, cudaGetLastError());
      h.launches++;
    }
  }
  if (nsys > 0)
    CLM_CUDA_TRY(h, cudaMemcpyAsync(B.hres + (size_t)slot * nsys * 16, o_e, (size_t)nsys * 16, cudaMemcpyDeviceToHost,
                                    h.stream));
  if (opk == OPK_NL)
    CLM_CUDA_TRY(h, cudaMemcpyAsync(hres_nl(B), A.nl_count, 8, cudaMemcpyDeviceToHost, h.stream));
  return OK;
}

// Build + operators, enqueued without synchronization (also the body of the recorded graph).
template <class T> int enqueue_step(Handle& h, int nops, const int* ops, const clm_op_params* P) {
  BatchState& B = h.batch;
  CLM_CUDA_TRY(h, cudaMemsetAsync(h.err.p, 0, 64, h.stream));
  int st = build_set<T>(h, 0, tmpl_geom<T>(h));
  if (st) return st;
  for (int k = 0; k < nops; k++) {
    st = enqueue_op<T>(h, k, ops[k], P ? &P[k] : nullptr);
    if (st) return st;
  }
  if (B.nsys > 0)
    CLM_CUDA_TRY(h, cudaMemcpyAsync(hres_err(B), B.sys_err.p, sizeof(int) * (size_t)B.nsys, cudaMemcpyDeviceToHost,
                                    h.stream));
  return enqueue_build_totals(h);
}

// After the step's stream work is complete: overflow checks, statuses and results.
template <class T> int finish_step(Handle& h, int nops, const int* ops, clm_batch_outputs* outs, bool* again) {
  BatchState& B = h.batch;
  *again = false;
  bool overflow = false;
  h.pinned[40] &= ~DERR_NAN;  // NaN coordinates are reported per system in a batch
  int st = check_build_totals(h, &overflow);
  if (st) return st;
  if (overflow) {
    *again = true;
    return OK;
  }
  if (h.pinned[40] & DERR_CELL_RANGE) return fail(&h, ERR_INTERNAL, "batch consistency check failed");
  if (h.pinned[40] & DERR_STAGE) return fail(&h, ERR_INTERNAL, "pair map: a staging wait for bulk copies timed out");
  int nl_slot = -1;
  for (int k = 0; k < nops; k++)
    if (ops[k] == CLM_OP_NL) nl_slot = k;
  if (nl_slot >= 0) {
    const unsigned long long npairs = *hres_nl(B);
    if ((int64_t)npairs > h.nl_cap) {
      h.nl_cap = (int64_t)npairs + (int64_t)(npairs / 16) + 1024;
      *again = true;
      return OK;
    }
    h.nl_n = (int64_t)npairs;
    h.nl_valid = true;
  }
  const int* serr = hres_err(B);
  for (int64_t s = 0; s < B.nsys; s++) {
    if (B.status[(size_t)s] == ERR_NAN) B.status[(size_t)s] = OK;
    if (B.status[(size_t)s] == OK && (serr[s] & DERR_NAN)) B.status[(size_t)s] = ERR_NAN;
  }
  const int N = h.dim;
  const int64_t n = h.sets[0].n;
  for (int k = 0; k < nops; k++) {
    clm_batch_outputs& O = outs[k];
    const double* se = hres_sum(B, k);
    const unsigned long long* sc = hres_cnt(B, k);
    std::vector<double> sv((size_t)B.nsys);
    std::vector<int64_t> cv((size_t)B.nsys);
    for (int64_t s = 0; s < B.nsys; s++) {
      const bool oks = B.status[(size_t)s] == OK;
      cv[(size_t)s] = oks ? (int64_t)sc[s] : 0;
      sv[(size_t)s] = !oks ? NAN : (ops[k] == CLM_OP_COUNT ? (double)sc[s] : se[s]);
    }
    const cudaMemcpyKind kind = O.out_on_device ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
    if (O.scalar && B.nsys) CLM_CUDA_TRY(h, cudaMemcpy(O.scalar, sv.data(), 8 * (size_t)B.nsys, kind));
    if (O.count && B.nsys) CLM_CUDA_TRY(h, cudaMemcpy(O.count, cv.data(), 8 * (size_t)B.nsys, kind));
    if (opkind_of(ops[k]) == OPK_FORCES && O.forces && n > 0) {
      CLM_CUDA_TRY(h, cudaMemcpyAsync(O.forces, B.forces.p, sizeof(T) * n * N,
                                      O.out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h.stream));
      CLM_CUDA_TRY(h, cudaStreamSynchronize(h.stream));
    }
  }
  return OK;
}

template <class T> int batch_run(Handle& h, int nops, const int* ops, const clm_op_params* P, clm_batch_outputs* outs) {
  BatchState& B = h.batch;
  if (!B.on) return fail(&h, ERR_STATE, "not a batch handle");
  if (B.nsys <= 0 && B.offsets.empty()) return fail(&h, ERR_STATE, "clm_batched_set_systems must be called first");
  if (nops < 1 || nops > kMaxOps || !ops || !outs) return fail(&h, ERR_ARG, "1 to 4 operators per step");
  int n_nl = 0;
  for (int k = 0; k < nops; k++) {
    if (!batch_op_ok(ops[k])) return fail(&h, ERR_ARG, "operator not available for batches");
    if (P && P[k].ntypes > 0) return fail(&h, ERR_ARG, "batches take no per-type tables");
    n_nl += (ops[k] == CLM_OP_NL);
  }
  if (n_nl > 1) return fail(&h, ERR_ARG, "at most one neighbour-list operator per step");
  if (h.sets[0].n != B.offsets[(size_t)B.nsys])
    return fail(&h, ERR_DIM, "the positions do not match the systems' offsets");
  if (!B.tables_ready || B.tables_dtype != h.dtype) {
    drop_graph(B);
    int st = batch_tables<T>(h);
    if (st) return st;
  }
  h.nl_valid = false;
  const int64_t l0 = h.launches;
  // key of a recorded step: operators, parameters, sizes
  std::vector<double> key;
  key.push_back((double)h.precision);  // a recording is only valid for the precision form it ran with
  for (int k = 0; k < nops; k++)
    for (int q = 0; q < 4; q++) key.push_back(P ? P[k].p[q] : 0.0);
  const bool same_ops = B.gexec && B.graph_ops == std::vector<int>(ops, ops + nops) && B.graph_params == key &&
                        B.graph_n == h.sets[0].n;
  if (B.use_graph && same_ops) {
    h.sets[0].pending = true;
    cudaEventRecord(h.ev[0], h.stream);
    CLM_CUDA_TRY(h, cudaGraphLaunch(B.gexec, h.stream));
    cudaEventRecord(h.ev[1], h.stream);
    CLM_CUDA_TRY(h, cudaStreamSynchronize(h.stream));
    cudaEventElapsedTime(&B.step_ms, h.ev[0], h.ev[1]);
    bool again = false;
    int st = finish_step<T>(h, nops, ops, outs, &again);
    if (st) return st;
    if (!again) {
      B.step_launches = B.graph_launches;
      return OK;
    }
    drop_graph(B);  // capacities changed: run directly, then record again
  }
  bool again = true;
  for (int attempt = 0; attempt < 3 && again; attempt++) {
    const int64_t la = h.launches;
    cudaEventRecord(h.ev[0], h.stream);
    int st = enqueue_step<T>(h, nops, ops, P);
    if (st) return st;
    cudaEventRecord(h.ev[1], h.stream);
    CLM_CUDA_TRY(h, cudaStreamSynchronize(h.stream));
    cudaEventElapsedTime(&B.step_ms, h.ev[0], h.ev[1]);
    cudaEventElapsedTime(&h.map_ms, h.ev[2], h.ev[3]);
    st = finish_step<T>(h, nops, ops, outs, &again);
    if (st) return st;
    B.step_launches = h.launches - la;
  }
  if (again) return fail(&h, ERR_INTERNAL, "batch step did not converge on its capacities");
  if (B.use_graph) {
    // record the step as it just ran (same sizes, so nothing is allocated while recording)
    drop_graph(B);
    cudaGraph_t graph = nullptr;
    const int64_t la = h.launches;
    CLM_CUDA_TRY(h, cudaStreamBeginCapture(h.stream, cudaStreamCaptureModeRelaxed));
    h.capturing = true;
    int st = enqueue_step<T>(h, nops, ops, P);
    h.capturing = false;
    cudaError_t ce = cudaStreamEndCapture(h.stream, &graph);
    if (st) {
      if (graph) cudaGraphDestroy(graph);
      return st;
    }
    if (ce != cudaSuccess) return fail(&h, ERR_CUDA, "stream capture of the batch step failed");
    ce = cudaGraphInstantiate(&B.gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      B.gexec = nullptr;
      return fail(&h, ERR_CUDA, "graph instantiation failed");
    }
    B.graph_launches = h.launches - la;
    h.launches = la;  // recorded, not launched
    B.graph_ops.assign(ops, ops + nops);
    B.graph_params = key;
    B.graph_n = h.sets[0].n;
    h.sets[0].pending = false;
  }
  (void)l0;
  return OK;
}

}  // namespace

extern "C" {

int32_t clm_lj_adjoint(clm_handle h, const clm_op_params* params, clm_outputs* out) {
  return clm_run(h, CLM_OP_LJ_ADJOINT, params, out);
}

int32_t clm_batched_create(int32_t dtype, int32_t dim, clm_handle* out) {
  int32_t st = clm_create(dtype, dim, 1, out);
  if (st) return st;
  (*out)->batch.on = true;
  return OK;
}

int32_t clm_batched_set_systems(clm_handle h, int64_t nsys, const int64_t* offsets, const double* cells,
                                int32_t cell_kind, double cutoff, int32_t lcell) {
  if (!h) return ERR_ARG;
  if (!h->batch.on) return fail(h, ERR_STATE, "not a batch handle (clm_batched_create)");
  if (nsys < 0 || nsys >= ((int64_t)1 << 24)) return fail(h, ERR_ARG, "number of systems out of range");
  if (nsys > 0 && (!offsets || !cells)) return fail(h, ERR_ARG, "offsets and cells are required");
  if (lcell < 1) return fail(h, ERR_LCELL, "lcell must be greater or equal to 1");
  if (!(cutoff > 0) || !std::isfinite(cutoff)) return fail(h, ERR_ARG, "cutoff must be a positive finite number");
  if (cell_kind != CLM_ORTHO && cell_kind != CLM_TRICLINIC)
    return fail(h, ERR_ARG, "batches take orthorhombic or triclinic periodic cells");
  const int N = h->dim;
  BatchState& B = h->batch;
  std::vector<int64_t> off((size_t)nsys + 1, 0);
  if (nsys > 0) {
    if (offsets[0] != 0) return fail(h, ERR_ARG, "offsets[0] must be 0");
    for (int64_t s = 0; s <= nsys; s++) {
      off[(size_t)s] = offsets[s];
      if (s > 0 && offsets[s] < offsets[s - 1]) return fail(h, ERR_ARG, "offsets must be non-decreasing");
    }
    if (off[(size_t)nsys] >= ((int64_t)1 << 27)) return fail(h, ERR_ARG, "at most 2^27 - 1 particles in a batch");
  }
  const int per = (cell_kind == CLM_ORTHO) ? N : N * N;
  std::vector<double> cm((size_t)nsys * N * N, 0.0);
  for (int64_t s = 0; s < nsys; s++) {
    for (int k = 0; k < per; k++)
      if (!std::isfinite(cells[s * per + k])) return fail(h, ERR_ARG, "unit cells must be finite");
    double* d = cm.data() + (size_t)s * N * N;
    if (cell_kind == CLM_ORTHO) {
      for (int i = 0; i < N; i++) d[i * N + i] = cells[s * per + i];
    } else {
      for (int k = 0; k < N * N; k++) d[k] = cells[s * per + k];
    }
  }
  drop_graph(B);
  B.nsys = nsys;
  B.kind = cell_kind;
  B.lcell = lcell;
  B.cutoff = cutoff;
  B.offsets.swap(off);
  B.cells.swap(cm);
  B.tables_ready = false;
  B.status.assign((size_t)nsys, OK);
  h->kind = cell_kind;
  h->lcell = lcell;
  h->cutoff = cutoff;
  h->box_set = true;
  h->sets[0].dirty = true;
  h->nl_valid = false;
  return OK;
}

int32_t clm_batched_run(clm_handle h, int32_t nops, const int32_t* ops, const clm_op_params* params,
                        clm_batch_outputs* outs) {
  if (!h) return ERR_ARG;
  std::vector<int> o(ops ? ops : nullptr, ops ? ops + std::max(0, nops) : nullptr);
  return h->dtype == CLM_F64 ? batch_run<double>(*h, nops, o.data(), params, outs)
                             : batch_run<float>(*h, nops, o.data(), params, outs);
}

int32_t clm_batched_status(clm_handle h, int32_t* status, int64_t nsys) {
  if (!h || !status) return ERR_ARG;
  if (!h->batch.on) return fail(h, ERR_STATE, "not a batch handle");
  if (nsys < h->batch.nsys) return fail(h, ERR_CAPACITY, "status array smaller than the number of systems");
  for (int64_t s = 0; s < h->batch.nsys; s++)
    status[s] = (s < (int64_t)h->batch.status.size()) ? h->batch.status[(size_t)s] : OK;
  return OK;
}

int32_t clm_batched_set_graph(clm_handle h, int32_t enable) {
  if (!h) return ERR_ARG;
  if (!h->batch.on) return fail(h, ERR_STATE, "not a batch handle");
  h->batch.use_graph = enable != 0;
  if (!enable) drop_graph(h->batch);
  return OK;
}

int32_t clm_batched_set_config(clm_handle h, int32_t lcell, int32_t cell_split, int32_t grid_div) {
  if (!h) return ERR_ARG;
  BatchState& B = h->batch;
  if (!B.on) return fail(h, ERR_STATE, "not a batch handle");
  if (cell_split > 64 || grid_div > 64) return fail(h, ERR_ARG, "cell_split and grid_div are at most 64");
  if (lcell > 0 && lcell != B.lcell) {
    B.lcell = lcell;
    h->lcell = lcell;
    B.tables_ready = false;
  }
  if (cell_split > 0) B.cell_split = cell_split;
  if (grid_div > 0) B.grid_div = grid_div;
  drop_graph(B);
  h->sets[0].dirty = true;
  return OK;
}

int32_t clm_batched_autotune(clm_handle h, int32_t nops, const int32_t* ops, const clm_op_params* params,
                             int32_t reps, int32_t* config, float* best_ms) {
  if (!h) return ERR_ARG;
  BatchState& B = h->batch;
  if (!B.on) return fail(h, ERR_STATE, "not a batch handle");
  if (reps < 1) reps = 3;
  const bool graph = B.use_graph;
  B.use_graph = false;
  std::vector<clm_batch_outputs> outs((size_t)std::max(1, nops));
  for (auto& o : outs) std::memset(&o, 0, sizeof(o));
  float best = INFINITY;
  int bl = B.lcell, bs = B.cell_split, bg = B.grid_div;
  for (int lc = 1; lc <= 3; lc++)
    for (int sp = 1; sp <= 2; sp++)
      for (int gd = 1; gd <= 2; gd++) {
        int st = clm_batched_set_config(h, lc, sp, gd);
        if (st) return st;
        st = clm_batched_run(h, nops, ops, params, outs.data());  // sizes the buffers
        if (st) {
          B.use_graph = graph;
          return st;
        }
        std::vector<float> t;
        for (int r = 0; r < reps; r++) {
          h->sets[0].dirty = true;
          st = clm_batched_run(h, nops, ops, params, outs.data());
          if (st) {
            B.use_graph = graph;
            return st;
          }
          t.push_back(B.step_ms);
        }
        std::sort(t.begin(), t.end());
        const float med = t[t.size() / 2];
        if (med < best) {
          best = med;
          bl = lc;
          bs = sp;
          bg = gd;
        }
      }
  int st = clm_batched_set_config(h, bl, bs, bg);
  B.use_graph = graph;
  if (st) return st;
  if (config) {
    config[0] = bl;
    config[1] = bs;
    config[2] = bg;
  }
  if (best_ms) *best_ms = best;
  return OK;
}

int32_t clm_device_allocations(int64_t* count, int64_t* bytes) {
  if (count) *count = (int64_t)alloc_count().load();
  if (bytes) *bytes = (int64_t)alloc_bytes().load();
  return OK;
}

int32_t clm_batched_last_step(clm_handle h, float* step_ms, int64_t* launches) {
  if (!h) return ERR_ARG;
  if (step_ms) *step_ms = h->batch.step_ms;
  if (launches) *launches = h->batch.step_launches;
  return OK;
}

}  // extern "C"
