// Cell-pair map kernel (self and cross pairs, operator epilogues), included by the translation units
// that instantiate it.
//
// Replaces _pairwise! and its inner loops:
//   self  src/internals/self.jl:106-184      cross src/internals/cross.jl:81-129
//   vicinal cells with projection culling    src/internals/vicinal_cells.jl:4-75,
//                                            src/internals/auxiliary_functions.jl:66-111
//   non-periodic inner loops                 src/internals/NonPeriodicCells.jl:281-352
// and the per-batch output copies + reduce_output! with on-chip reductions.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "clm_pairs_args.hpp"

namespace clm {
namespace pk {

template <class T> __device__ __forceinline__ T pos_of(const SetView<T>& S, int d, int t) {
  return d == 0 ? S.px[t] : (d == 1 ? S.py[t] : S.pz[t]);
}

// Reciprocal and reciprocal square root for pair VALUES (energies, forces), which are checked against
// tolerances, never used for pair membership or neighbour-list distances.
//  FP32: hardware approximations (rcp.approx / rsqrt.approx, a couple of ulp).
//  FP64: the hardware FP64 estimate y refined by the second-order terms of a series in its residual e,
//        which cubes the relative error (from the estimate's ~2^-22 to far below FP64 rounding):
//        1/x = y / (1 - e) = y (1 + e + e^2 + ...) with e = 1 - x y;
//        1/sqrt(x) = y (1 - e)^(-1/2) = y (1 + e/2 + 3e^2/8 + ...) with e = 1 - x y^2.
//        Three and five FP64 instructions, where two Newton-Raphson steps take four and eight: GB300's FP64
//        pipe takes 16 cycles per warp instruction and bounds the FP64 pair kernels.
__device__ __forceinline__ float vrcp(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float vrsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double vrcp(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x, y, 1.0);
  e = fma(e, e, e);  // e + e^2
  return fma(y, e, y);
}
__device__ __forceinline__ double vrsqrt(double x) {
  double y;
  asm("rsqrt.approx.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y * y, 1.0);
  const double p = fma(0.375, e, 0.5);  // 1/2 + 3e/8
  return fma(y * e, p, y);
}

// 1/sqrt(x) for the FP64 radial-histogram term: the hardware estimate refined by one Newton-Raphson step,
// which squares its relative error (about 2^-23) to within ~1e-14 of 1/sqrt(x), far inside the 1e-10 to
// which the per-bin sums are compared; each FP64 instruction saved frees the FP64 pipe that bounds the exact
// histogram.
__device__ __forceinline__ double vrsqrt_1nr(double x) {
  double y;
  asm("rsqrt.approx.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y * y, 1.0);
  return fma(0.5 * y, e, y);
}

// a <= b and a < b for non-negative values (squared distances, the cutoff, +inf), decided on the bit
// patterns, which are ordered like the values for non-negative IEEE numbers: for FP64 an integer compare,
// which leaves the FP64 pipe (one warp instruction per 16 cycles on GB300) to arithmetic.
template <class T> __device__ __forceinline__ bool nonneg_le(T a, T b) {
  if constexpr (std::is_same<T, double>::value) return __double_as_longlong(a) <= __double_as_longlong(b);
  else return a <= b;
}
template <class T> __device__ __forceinline__ bool nonneg_lt(T a, T b) {
  if constexpr (std::is_same<T, double>::value) return __double_as_longlong(a) < __double_as_longlong(b);
  else return a < b;
}

// Operator parameter k and the LJ type tables in the precision of the pair value (no conversions per pair).
template <class V, class T> __device__ __forceinline__ V par(const PairArgs<T>& A, int k) {
  if constexpr (std::is_same<V, float>::value) return A.pf[k];
  else return (V)A.p[k];
}
template <class V, class T> __device__ __forceinline__ V eps_tab(const PairArgs<T>& A, int k) {
  if constexpr (std::is_same<V, float>::value) return A.eps_tf[k];
  else return (V)A.eps_t[k];
}
template <class V, class T> __device__ __forceinline__ V sig_tab(const PairArgs<T>& A, int k) {
  if constexpr (std::is_same<V, float>::value) return A.sig_tf[k];
  else return (V)A.sig_t[k];
}
// Per-particle weight of particle k of set x (or y when ys).
template <class V, class T> __device__ __forceinline__ V weight(const PairArgs<T>& A, bool ys, int k) {
  if constexpr (std::is_same<V, float>::value) return (ys ? A.wyf : A.wxf)[k];
  else return (V)(ys ? A.wy : A.wx)[k];
}

// Per-pair energy u and g = (du/dr)/r (force contribution df = g*(x_i - x_j)).
template <class V, class T>
__device__ __forceinline__ void pair_value(const PairArgs<T>& A, int op, V d2, int i, int j, V& u, V& g) {
  switch (op) {
    case 2:  // COUNT
      u = V(1);
      g = V(0);
      break;
    case 3:  // SUM_D2
      u = d2;
      g = V(0);
      break;
    case 4:  // SUM_D
      u = d2 * vrsqrt(d2);
      g = V(0);
      break;
    case 5:  // SUM_INV_D
      u = vrsqrt(d2);
      g = V(0);
      break;
    case 6:
    case 7: {  // SOFT (c - d)^2
      V ri = vrsqrt(d2);
      V d = d2 * ri;
      V c = par<V>(A, 0);
      u = (c - d) * (c - d);
      g = V(-2) * (c - d) * ri;
      break;
    }
    case 8:
    case 9:
    case 13: {  // LJ eps*(c12 (s/d)^12 - c6 (s/d)^6)
      V eps = par<V>(A, 0), sig = par<V>(A, 1);
      if (A.ntypes > 0) {
        int ti = A.tx[i];
        int tj = A.self ? A.tx[j] : A.ty[j];
        eps = eps_tab<V>(A, ti * A.ntypes + tj);
        sig = sig_tab<V>(A, ti * A.ntypes + tj);
      }
      V c12 = par<V>(A, 2), c6 = par<V>(A, 3);
      V r2i = vrcp(d2);
      V sr2 = (sig * sig) * r2i;
      V sr6 = sr2 * sr2 * sr2;
      V sr12 = sr6 * sr6;
      u = eps * (c12 * sr12 - c6 * sr6);
      g = eps * (V(-12) * c12 * sr12 + V(6) * c6 * sr6) * r2i;
      break;
    }
    case 14: {  // weighted 1/d: u = -c w_i w_j / d, g = (c w_i w_j / d^2) / d
      const V cw = par<V>(A, 0) * weight<V>(A, false, i) * weight<V>(A, A.self == 0, j);
      const V ri = vrsqrt(d2);
      u = -(cw * ri);
      g = cw * (ri * ri * ri);
      break;
    }
    case 12: {  // 1/d with gradient accumulation
      V ri = vrsqrt(d2);
      u = ri;
      g = ri * ri * ri;
      break;
    }
    default:
      u = V(0);
      g = V(0);
  }
}

// Sum of `v` over the lanes of a match group (`peers`: the lanes sharing this lane's key), returned in
// the group's lowest lane.  Pairwise tree: at each step every lane at an even position of its group adds
// the value of the next remaining peer, and the lanes at odd positions drop out, so a group of g lanes
// needs ceil(log2 g) steps and the whole warp at most 5, however many groups there are.  All lanes of
// the warp call it.
template <class V> __device__ __forceinline__ V group_sum(unsigned peers, V v, int lane) {
  unsigned pos = __popc(peers & ((1u << lane) - 1u));  // position of this lane in its group
  unsigned rest = peers & ~((2u << lane) - 1u);         // peers above this lane (lane 31: none)
  if (lane == 31) rest = 0u;
  while (__any_sync(0xffffffffu, rest != 0u)) {
    const int nxt = __ffs(rest);                          // 1 + lane of the next remaining peer, 0 if none
    const V t = __shfl_sync(0xffffffffu, v, nxt > 0 ? nxt - 1 : lane);
    if (nxt > 0) v += t;
    const unsigned gone = __ballot_sync(0xffffffffu, (pos & 1u) != 0u);  // consumed by their left neighbour
    rest &= ~gone;
    pos >>= 1;
  }
  return v;
}

// Asynchronous global -> shared copies (cp.async, sm_80+): 16 bytes, cached in L1.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Bulk asynchronous copies (cp.async.bulk, the TMA unit's untiled form) from this GPU's global memory into
// shared memory, completing on an mbarrier that counts the bytes (expect_tx / complete_tx).  Addresses are
// 16-byte aligned and sizes multiples of 16 bytes (the candidate records are 16-byte float4).
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// makes mbarrier initialisations visible to the asynchronous proxy
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
// orders this thread's earlier shared-memory accesses before later asynchronous-proxy writes
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the phase of the given parity to complete, giving up after about a second (2^31 cycles).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > (1ll << 31)) return false;
  }
  return true;
}

// Geometry of the cell being processed: the launch's own (one system) or that of the cell's system
// (batches); `cb` returns the first global cell of that system.
template <bool B, class T>
__device__ __forceinline__ const DevGeom<T>& geo_of(const PairArgs<T>& A, int li, int& cb) {
  if constexpr (B) {
    const int s = A.cell_sys[li];
    cb = A.cbase[s];
    return A.gtab[s];
  } else {
    cb = 0;
    return A.g;
  }
}

// Adds a force term to the sums of particle `idx` (set y when `ys`): one 16-byte vector atomic for FP32
// pair values, one FP64 atomic per component otherwise.
template <class T, int N, class FA>
__device__ __forceinline__ void force_add(const PairArgs<T>& A, bool ys, int idx, const FA* v) {
  if constexpr (std::is_same<FA, float>::value) {
    atomicAdd((ys ? A.f4y : A.f4x) + idx, make_float4(v[0], v[1], (N == 3) ? v[2] : 0.f, 0.f));
  } else {
    double* f = (ys ? A.fy : A.fx) + (int64_t)idx * N;
#pragma unroll
    for (int d = 0; d < N; d++) atomicAdd(f + d, (double)v[d]);
  }
}

// Pair map kernel.  CROSS: x-y pairs; otherwise self pairs.  Every pair is visited once, from the side
// the reference visits it (forward half stencil, or the full stencil with index_i < index_j for
// triclinic cells); forces add -df to the particle's sums and +df to the partner's.
//
// Each warp takes one cell (or one part of a crowded cell); the cells of its stencil are concatenated
// into one candidate stream, staged in windows of 128 candidates into shared memory by bulk copies: each
// lane holds one stencil cell and copies that cell's part of the window (its records are contiguous in
// the cell list) with one cp.async.bulk, completing on the warp's mbarrier; the next window is copied
// while the current one is tested.  Triclinic self pairs visit each pair of cells once (the forward half
// stencil, and the backward cells without real particles: sym_stencil_offset), as orthorhombic self pairs
// do.  Phase A: every lane tests its particle against 32 staged candidates per round with an FP32
// distance (FMA) and records the candidates inside cutoff^2 (1 + 2^-13) in a bit mask.  Phase B: the set
// bits of all lanes are compacted into a queue that all lanes work through: the reference's pair rules,
// the re-test in the input dtype where needed, and the operator epilogue.  The projection filter of the reference is
// evaluated only for pairs with d2 > cutoff^2 (1 - 2^-13): any pair further inside passes it (the
// projection of the separation on a unit vector cannot exceed the separation, and the margin covers the
// half cell), so skipping it elsewhere leaves the pair set unchanged.
// Resident blocks per SM (6 for Float32, 3 for Float64: at most 85 / 170 registers per thread; the
// kernels use 64-80 / 113-152) were picked by timing 4..8 and 3..4 on GB300; fewer registers spill in the
// pair epilogues.  The split-form histogram of Float64 handles runs 5 blocks (at most 102 registers, small
// spills): timed at 3..6 blocks on the two-set workload, 5 gave 1.37x (3D) and 1.2x (2D) over 3; the exact
// histogram keeps 3 (its FP64 pipe is the bound at any of these).
// OPC: the operator id when fixed at compile time (the LJ force loop), 0 = read from the arguments.
template <class T, int N, int OPK, bool SPLIT, bool CROSS, bool BATCH, int OPC = 0>
__global__ void __launch_bounds__(kThreads, (sizeof(T) == 4) ? 6 : ((OPK == OPK_HIST && SPLIT) ? 5 : 3))
    k_pairs(const PairArgs<T> A) {
  using V = T;
  using FA = typename std::conditional<std::is_same<T, double>::value && !SPLIT, double, float>::type;
  constexpr bool IS_F = (OPK == OPK_FORCES) || (OPK == OPK_ADJ);
  constexpr bool FP64 = std::is_same<T, double>::value;
  constexpr bool ABS_PF = !FP64 && !SPLIT;  // FP32 exact form: the prefilter uses the coordinates themselves
  constexpr int JC = 128;                   // staging window: 32 candidates per lane group (G <= 4)
  const DevGeom<T>& g = A.g;
  const int op = OPC ? OPC : A.op;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const unsigned FULL = 0xffffffffu;

  __shared__ int s_st_start[kWarps][32];
  __shared__ int s_st_pref[kWarps][33];
  __shared__ int s_st_meta[kWarps][32];
  // staged candidates, two windows (the next one is copied while the current one is tested)
  __shared__ __align__(16) float4 s_pf[2][kWarps][JC];  // prefilter coordinates; .w carries the particle code
  __shared__ int s_meta[2][kWarps][ABS_PF ? 1 : JC];    // stencil offset and flags of the candidate's cell
  __shared__ int s_tj[2][kWarps][ABS_PF ? 1 : JC];       // position of the candidate in the cell list
  __shared__ __align__(8) unsigned long long s_mbar[kWarps][2];  // completion of the bulk copies of a window
  __shared__ unsigned short s_q[kWarps][1024];  // compacted candidates: (particle slot << 8) | staged index
  // particles of the current chunk of the cell: prefilter coordinates with the particle code in .w, and
  // (Float64 handles) the coordinates in the handle dtype for the exact re-test
  __shared__ __align__(16) float4 s_i4[kWarps][32];
  __shared__ T s_ix[kWarps][3][ABS_PF ? 1 : 32];
  __shared__ FA s_if[kWarps][3][IS_F ? 32 : 1];  // force sums of those particles
  // radial histogram (dynamic shared memory, layout in hist_smem): block bins in FP64, bin edges, and
  // per-warp bins that the warp updates without atomics
  extern __shared__ __align__(16) unsigned char s_dyn[];
  const HistSmem hl = hist_smem((OPK == OPK_HIST) ? A.nbins : 0, (int)sizeof(T), (int)sizeof(FA));
  double* s_hs = reinterpret_cast<double*>(s_dyn + hl.hs);
  unsigned long long* s_hc = reinterpret_cast<unsigned long long*>(s_dyn + hl.hc);
  T* s_bins = reinterpret_cast<T*>(s_dyn + hl.bins);
  float* s_binf = reinterpret_cast<float*>(s_dyn + hl.binf);
  FA* s_ws = reinterpret_cast<FA*>(s_dyn + hl.ws) + warp * A.nbins;
  unsigned* s_wc = reinterpret_cast<unsigned*>(s_dyn + hl.wc) + warp * A.nbins;
  __shared__ double s_red[kWarps];
  __shared__ unsigned long long s_redc[kWarps];

  constexpr int F_SAME = 1 << 24;
  const bool tri = (g.kind == TRICLINIC);
  const bool nonper = (g.kind == NONPERIODIC);
  const bool sym = tri && !CROSS;  // triclinic self pairs: each pair of cells once (sym_stencil_offset)
  const int l = g.lcell;
  const int w = 2 * l + 1;
  const int wN = (N == 3) ? w * w * w : w * w;
  const int nf = (wN - 1) / 2;
  // entry 0 is the cell itself; then all neighbours (cross pairs), the forward and the backward half
  // (triclinic self pairs) or the forward half
  const int nent = CROSS ? wN : (sym ? 2 * nf + 1 : nf + 1);
  const T band = (T)g.thr_lo;  // d2 above this: projection filter applies
  if (lane == 0) {
    mbar_init(&s_mbar[warp][0], 1);
    mbar_init(&s_mbar[warp][1], 1);
    fence_mbar_init();
  }
  __syncwarp();
  unsigned ph = 0u;  // bit b: parity of the next phase of s_mbar[warp][b] to complete
  bool bad = false;  // a staging wait gave up (error reported): this warp stops

  if constexpr (OPK == OPK_HIST) {
    for (int b = threadIdx.x; b < A.nbins; b += kThreads) {
      s_hc[b] = 0ull;
      s_hs[b] = 0.0;
    }
    for (int b = lane; b < A.nbins; b += 32) {
      s_ws[b] = FA(0);
      s_wc[b] = 0u;
    }
    for (int b = threadIdx.x; b <= A.nbins; b += kThreads) {
      s_bins[b] = A.bins[b];
      s_binf[b] = (float)A.bins[b];
    }
    __syncthreads();
  }

  double e_tot = 0.0;  // per-lane energy (FP64); FP32 partial sums are folded in per particle chunk
  FA e_part = 0;
  FA adj[kAdjVals - 1];  // adjoint accumulators: virial (6), dU/deps (3), dU/dsigma (3)
#pragma unroll
  for (int k = 0; k < kAdjVals - 1; k++) adj[k] = FA(0);
  unsigned long long c_acc = 0;
  T best_d2 = INFINITY;
  int best_i = 0x7fffffff, best_j = 0x7fffffff;

  const int gw = blockIdx.x * kWarps + warp;
  const int nw = gridDim.x * kWarps;
  const int n_real = *A.n_real_dev;
  const int S = A.cell_split;  // the host keeps cells x parts below 2^31
  const int n_items = n_real * S;
  for (int r = gw; r < n_items && !bad; r += nw) {
    const int rcell = r / S;
    const int part = r - rcell * S;
    const int li = A.real_list[rcell];
    int cb = 0;  // first global cell of the system (batches)
    const DevGeom<T>& gc = geo_of<BATCH>(A, li, cb);
    int ci[3];
    cart_of(li - cb, gc.nc, N, ci);
    T ctr_i[3] = {0, 0, 0};
    cell_center<T, N>(gc, ci, ctr_i);
    const int si = A.X.cell_start[li];
    const int ni = A.X.cell_start[li + 1] - si;
    const int G = (ni <= 8) ? 4 : ((ni <= 16) ? 2 : 1);
    const int LP = 32 / G;
    const int grp = lane % G;  // the G lanes of one particle are adjacent: the hit queue is ordered by particle
    const int il = lane / G;

    for (int ib = part * LP; ib < ni && !bad; ib += LP * S) {
      const int ii = ib + il;
      const bool vi = ii < ni;
      const int ti = si + (vi ? ii : 0);
      T xi[3] = {0, 0, 0};
      float pi[3] = {0.f, 0.f, 0.f};
      int code_i = 0;
      if (vi) {
#pragma unroll
        for (int d = 0; d < N; d++) xi[d] = pos_of(A.X, d, ti);
        code_i = A.X.code[ti];
        if (ABS_PF) {
#pragma unroll
          for (int d = 0; d < N; d++) pi[d] = (float)xi[d];
        } else {
          float4 oi = A.X.off[ti];
          pi[0] = oi.x;
          pi[1] = oi.y;
          pi[2] = oi.z;
        }
      }
      const bool real_i = code_i >= 0;
      const int idx_i = real_i ? code_i : -code_i - 1;
      const bool act_i = (tri && CROSS) ? (vi && real_i) : vi;
      if (grp == 0) {
        s_i4[warp][il] = make_float4(pi[0], pi[1], pi[2], __int_as_float(code_i));
#pragma unroll
        for (int d = 0; d < 3; d++) {
          if constexpr (!ABS_PF) s_ix[warp][d][il] = xi[d];
          if constexpr (IS_F) s_if[warp][d][il] = FA(0);
        }
      }
      __syncwarp();

      for (int k0 = 0; k0 < nent && !bad; k0 += 32) {
        // ---- stencil table for entries k0 .. k0+31: lane k holds entry k0 + k (first copy, copies, offset)
        int e_start = 0, e_cnt = 0, e_pref = 0;
        {
          const int kk = k0 + lane;
          int meta = 0;
          if (kk < nent) {
            int o[3] = {0, 0, 0};
            bool back = false;
            if (kk > 0) {
              if (CROSS) {
                if (l == 1) stencil_offset<1>(false, l, N, kk - 1, o);
                else stencil_offset(false, l, N, kk - 1, o);
              } else {
                if (l == 1) sym_stencil_offset<1>(l, N, nf, kk - 1, o, &back);
                else sym_stencil_offset(l, N, nf, kk - 1, o, &back);
              }
            }
            int cj[3] = {1, 1, 1};
            bool inr = true;
#pragma unroll
            for (int d = 0; d < N; d++) {
              cj[d] = ci[d] + o[d];
              inr = inr && cj[d] >= 1 && cj[d] <= gc.nc[d];
            }
            if (!inr) {
              atomicOr(A.err, DERR_CELL_RANGE);
            } else {
              int lj = cj[0] - 1 + cb;
              if (N == 3) lj += gc.nc[0] * ((cj[1] - 1) + gc.nc[1] * (cj[2] - 1));
              else lj += gc.nc[0] * (cj[1] - 1);
              // a backward cell holding real particles is an item of its own, which visits this pair of cells
              if (!back || !A.Y.cell_real[lj]) {
                e_start = A.Y.cell_start[lj];
                e_cnt = A.Y.cell_start[lj + 1] - e_start;
              }
              meta = (o[0] + 128) | ((o[1] + 128) << 8) | ((o[2] + 128) << 16);
              if (kk == 0) meta |= F_SAME;
            }
          }
          int incl = e_cnt;
#pragma unroll
          for (int o2 = 1; o2 < 32; o2 <<= 1) {
            int y = __shfl_up_sync(FULL, incl, o2);
            if (lane >= o2) incl += y;
          }
          e_pref = incl - e_cnt;
          s_st_pref[warp][lane + 1] = incl;
          if (lane == 0) s_st_pref[warp][0] = 0;
          s_st_start[warp][lane] = e_start;
          s_st_meta[warp][lane] = meta;
        }
        __syncwarp();
        const int total = s_st_pref[warp][32];
        const int same_end = (k0 == 0) ? s_st_pref[warp][1] : 0;  // stream positions of the cell itself

        const int JR = 32 * G;  // candidates per round: each lane tests exactly 32
        // ---- stage window wi (stream positions wi*JC .. +JC-1) into buffer wi & 1: each lane copies the part
        // of its stencil cell inside the window with one bulk copy (16-byte records: coordinates or cell
        // offsets, the particle code in .w); lane 0 registers the window's bytes on the buffer's mbarrier
        const float4* rec = ABS_PF ? A.Y.xq : A.Y.off;
        auto issue = [&](int wi) {
          const int w0 = wi * JC, bsel = wi & 1;
          const int wc = min(JC, total - w0);
          fence_proxy_async_smem();  // earlier reads and writes of this buffer come before the copy's writes
          if (lane == 0) mbar_arrive_expect_tx(&s_mbar[warp][bsel], (unsigned)wc * 16u);
          __syncwarp();
          const int lo = max(e_pref, w0), hi = min(e_pref + e_cnt, w0 + wc);
          if (lo < hi)
            bulk_g2s(&s_pf[bsel][warp][lo - w0], rec + e_start + (lo - e_pref), (unsigned)(hi - lo) * 16u,
                     &s_mbar[warp][bsel]);
        };
        const int nwin = (total + JC - 1) / JC;
        if (nwin > 0) issue(0);
        for (int wi = 0; wi < nwin; wi++) {
          const int bsel = wi & 1, w0 = wi * JC, wc = min(JC, total - w0);
          if (wi + 1 < nwin) issue(wi + 1);  // the next window's copies overlap this window's tests
          {
            const bool ok = __all_sync(FULL, mbar_wait_bounded(&s_mbar[warp][bsel], (ph >> bsel) & 1u));
            ph ^= 1u << bsel;
            if (!ok) {
              // report, let the copies of the other buffer land (bounded), and stop this warp
              if (lane == 0) atomicOr(A.err, DERR_STAGE);
              if (wi + 1 < nwin) mbar_wait_bounded(&s_mbar[warp][bsel ^ 1], (ph >> (bsel ^ 1)) & 1u);
              bad = true;
              break;
            }
          }
          if constexpr (!ABS_PF) {
            // shift the offsets by the cell displacement so that x_i - x_j ~ off_i - pf, and record each
            // candidate's cell (stencil offset, same-cell flag) and position in the cell list
            for (int q = lane; q < wc; q += 32) {
              const int e = w0 + q;
              int lo = 0;  // last stencil entry whose prefix is <= e (that entry is not empty)
#pragma unroll
              for (int st = 16; st > 0; st >>= 1)
                if (s_st_pref[warp][lo + st] <= e) lo += st;
              const int meta = s_st_meta[warp][lo];
              float4 v = s_pf[bsel][warp][q];
              v.x += gc.csf[0] * (float)((meta & 255) - 128);
              v.y += gc.csf[1] * (float)(((meta >> 8) & 255) - 128);
              v.z += gc.csf[2] * (float)(((meta >> 16) & 255) - 128);
              s_pf[bsel][warp][q] = v;
              s_meta[bsel][warp][q] = meta;
              s_tj[bsel][warp][q] = s_st_start[warp][lo] + (e - s_st_pref[warp][lo]);
            }
            __syncwarp();
          }
          for (int rb = 0; rb < wc; rb += JR) {
            const int cntr = min(JR, wc - rb);
            // ---- phase A: 32 FP32 distance tests per lane into a bit mask.  A test passes when the sign bit
            // of d2 - thr is set and that of the AND of the two particle codes is clear (a pair of two images is
            // never the reference's pair); the sign bits are shifted into the mask, candidate b landing on bit
            // b.  thr carries a 2^-13 relative margin, far above the FP32 rounding of dx^2 - thr + dy^2 + dz^2,
            // so the strict comparison keeps every pair the exact test can accept.
            unsigned mask = 0u;
            {
              const float thr = g.thr_hi;
              // the lane's 32 candidates are rb + grp, rb + grp + G, ...: G fixed at compile time per
              // variant, so that every record is read at a constant offset
              auto test32 = [&](auto g_const) {
                constexpr int GG = decltype(g_const)::value;
                const float4* pp = &s_pf[bsel][warp][rb + grp];
#pragma unroll
                for (int b = 31; b >= 0; b--) {
                  const float4 p = pp[b * GG];
                  const float dx = pi[0] - p.x, dy = pi[1] - p.y, dz = (N == 3) ? pi[2] - p.z : 0.f;
                  const float e = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, -thr)));  // d2 - thr
                  const int v = __float_as_int(e) & ~(code_i & __float_as_int(p.w));  // .w: particle code
                  mask = __funnelshift_l((unsigned)v, mask, 1);  // (mask << 1) | sign bit of v
                }
              };
              if (G == 2) test32(std::integral_constant<int, 2>());
              else if (G == 1) test32(std::integral_constant<int, 1>());
              else test32(std::integral_constant<int, 4>());
            }
            {
              // bit b is stream position base + b G.  Dropped: positions past the window's end (stale
              // records), and in the cell itself the pairs the reference does not visit from this copy: the
              // earlier slots for self pairs (each pair of the cell once), every slot for an image copy in
              // cross pairs of orthorhombic cells (the particle copy must be real there).  What remains of
              // the pair rules is in phase B (triclinic self pairs of a real copy and an image).
              const int base = w0 + rb + grp;
              const int nb = (cntr - grp + G - 1) / G;
              if (!act_i || nb <= 0) mask = 0u;
              else if (nb < 32) mask &= (1u << nb) - 1u;
              int lim = -1;  // last dropped position of the cell itself
              if (!CROSS) lim = min(ii, same_end - 1);
              else if (!tri && !nonper && code_i < 0) lim = same_end - 1;
              if (lim >= base) {
                const int nr = (lim - base) / G + 1;
                mask &= (nr >= 32) ? 0u : ~((1u << nr) - 1u);
              }
            }
            // ---- phase B: compact the candidates of all lanes into a queue and process them with every lane
            // busy; each lane takes a contiguous run of the queue (runs are grouped by particle, so force
            // sums stay in registers and are flushed to shared memory only when the particle changes)
            int H;
            {
              const int nh = __popc(mask);
              int incl = nh;
#pragma unroll
              for (int o2 = 1; o2 < 32; o2 <<= 1) {
                int y = __shfl_up_sync(FULL, incl, o2);
                if (lane >= o2) incl += y;
              }
              H = __shfl_sync(FULL, incl, 31);
              int pos = incl - nh;
              unsigned m = mask;
              while (m) {
                const int b = __ffs(m) - 1;
                m &= m - 1u;
                s_q[warp][pos++] = (unsigned short)((il << 8) | (rb + b * G + grp));
              }
            }
            __syncwarp();
            const int per = (H + 31) >> 5;
            const int qbeg = lane * per;
            // Where the FP32 value decides the pairs well inside the cutoff (Float32 inputs, the split form),
            // the first sweep of the queue only marks the others (a band of 2^-13 around the cutoff, for the
            // exact re-test and the projection filter), and a second sweep over the same runs, made only when
            // a lane marked one, evaluates them: the main loop carries no exact path.
            constexpr bool DEFER = !FP64 || SPLIT;
            bool marked = false;
            auto sweep = [&](auto rare_c) {
            constexpr bool RARE = decltype(rare_c)::value;
            int cur = -1;  // the particle slot of this lane's run (its data below, its force sums in acc)
            float4 xi4 = make_float4(0.f, 0.f, 0.f, 0.f);
            FA acc[3] = {0, 0, 0};
            for (int t = 0; t < per; t++) {
              const int q = qbeg + t;
              const bool has = q < H;
              bool live = has;  // the entry is evaluated in this sweep
              int j = 0, ie = (cur < 0) ? 0 : cur;
              if (has) {
                const int ent = s_q[warp][q];
                ie = (ent >> 8) & 31;
                j = ent & 255;
                if constexpr (RARE) live = (ent & 0x8000) != 0;
              }
              // `cur` follows every queue entry (hit or not), so the lanes holding a particle are exactly the
              // lanes whose runs cover its entries: adjacent, and only the last one moves past it inside its
              // run; no other lane updates that particle's sums during the loop
              if (has && ie != cur) {
                if constexpr (IS_F) {
                  if (cur >= 0) {
#pragma unroll
                    for (int d = 0; d < N; d++) s_if[warp][d][cur] += acc[d];
                  }
#pragma unroll
                  for (int d = 0; d < N; d++) acc[d] = FA(0);
                }
                cur = ie;
                xi4 = s_i4[warp][ie];
              }
              const float pi[3] = {xi4.x, xi4.y, xi4.z};
              T xi[3] = {0, 0, 0};
              if constexpr (ABS_PF) {
                xi[0] = xi4.x;
                xi[1] = xi4.y;
                xi[2] = xi4.z;
              }
              auto load_xi = [&]() {
                if constexpr (!ABS_PF) {
#pragma unroll
                  for (int d = 0; d < 3; d++) xi[d] = s_ix[warp][d][ie];
                }
              };
              const int code_i = __float_as_int(xi4.w);
              const bool real_i = code_i >= 0;
              const int idx_i = real_i ? code_i : ~code_i;
              bool hit = false, sure = false;
              int idx_j = 0;
              int oi = 0, oj = 0;  // the pair as the reference orients it (i, j)
              float d2f = 0.f;
              float dvf[3] = {0.f, 0.f, 0.f};
              T d2 = 0;
              T xj[3] = {0, 0, 0};
              T dxs[3] = {0, 0, 0};  // x_i - x_j of the exact re-test, reused by the force epilogues
              int tjj = 0;  // the candidate's position in the cell list (coordinates read only when needed)
              auto load_xj = [&]() {
                if constexpr (!ABS_PF) {
#pragma unroll
                  for (int d = 0; d < N; d++) xj[d] = pos_of(A.Y, d, tjj);
                }
              };
              if (live) {
                const float4 p = s_pf[bsel][warp][j];
                const int code_j = __float_as_int(p.w);
                idx_j = code_j >= 0 ? code_j : ~code_j;
                // the rest of the pair rules: in triclinic self pairs of a real copy and an image, the copy of
                // the lower index is the reference's i and must be real
                bool cand = true;
                if (sym && (code_i ^ code_j) < 0) cand = sym_mixed_keeps(code_i, code_j);
                const bool sw = sym && idx_j < idx_i;
                oi = sw ? idx_j : idx_i;
                oj = sw ? idx_i : idx_j;
                if (cand) {
                  dvf[0] = pi[0] - p.x;
                  dvf[1] = pi[1] - p.y;
                  dvf[2] = (N == 3) ? pi[2] - p.z : 0.f;
                  d2f = fmaf(dvf[2], dvf[2], fmaf(dvf[1], dvf[1], dvf[0] * dvf[0]));
                  if (ABS_PF) {
                    xj[0] = (T)p.x;
                    xj[1] = (T)p.y;
                    if (N == 3) xj[N - 1] = (T)p.z;
                  }
                  if (DEFER && !RARE) {
                    // FP32 input or split form: well inside the cutoff the FP32 value decides; the others are
                    // marked for the second sweep
                    if (d2f <= g.thr_lo) {
                      hit = true;
                      sure = true;
                    } else {
                      s_q[warp][q] = (unsigned short)(s_q[warp][q] | 0x8000u);
                      marked = true;
                    }
                  }
                  if constexpr (!DEFER || RARE) {
                    load_xi();
                    int meta = 0;
                    if constexpr (!ABS_PF) {
                      meta = s_meta[bsel][warp][j];
                      tjj = s_tj[bsel][warp][j];
                    }
                    load_xj();
#pragma unroll
                    for (int d = 0; d < N; d++) dxs[d] = xsub(xi[d], xj[d]);
                    d2 = xmul(dxs[0], dxs[0]);
#pragma unroll
                    for (int d = 1; d < N; d++) d2 = xadd(d2, xmul(dxs[d], dxs[d]));
                    hit = nonneg_le(d2, g.cutoff_sqr);
                    const int epos = w0 + j;  // position in the stream
                    if (hit && nonneg_lt(band, d2) && epos >= same_end) {
                      // the reference's projection filter, seen from the cell of the reference's i
                      if constexpr (ABS_PF) {
                        int lo = 0;
#pragma unroll
                        for (int st = 16; st > 0; st >>= 1)
                          if (s_st_pref[warp][lo + st] <= epos) lo += st;
                        meta = s_st_meta[warp][lo];
                      }
                      int cj[3] = {ci[0] + (meta & 255) - 128, ci[1] + ((meta >> 8) & 255) - 128,
                                   ci[2] + ((meta >> 16) & 255) - 128};
                      T ctr_j[3];
                      cell_center<T, N>(gc, cj, ctr_j);
                      hit = sw ? projection_pass<T, N>(gc, ctr_j, ctr_i, xj, xi)
                               : projection_pass<T, N>(gc, ctr_i, ctr_j, xi, xj);
                    }
                  }
                }
              }
              // ---------------- operator epilogues
              if constexpr (OPK == OPK_NL) {
                if constexpr (BATCH) c_acc += hit ? 1ull : 0ull;  // pairs per system
                unsigned bal = __ballot_sync(FULL, hit);
                if (bal) {
                  unsigned long long base = 0;
                  int leader = __ffs(bal) - 1;
                  if (lane == leader) base = atomicAdd(A.nl_count, (unsigned long long)__popc(bal));
                  base = __shfl_sync(FULL, base, leader);
                  if (hit) {
                    T dval;
                    if (sure && ABS_PF) {
                      T dx = xsub(xi[0], xj[0]);
                      T e2 = xmul(dx, dx);
#pragma unroll
                      for (int d = 1; d < N; d++) {
                        T dd = xsub(xi[d], xj[d]);
                        e2 = xadd(e2, xmul(dd, dd));
                      }
                      dval = xsqrt(e2);
                    } else {
                      dval = sure ? (T)sqrtf(d2f) : xsqrt(d2);
                    }
                    unsigned long long pos = base + __popc(bal & ((1u << lane) - 1u));
                    if ((long long)pos < A.nl_cap) {
                      A.nl_i[pos] = oi;
                      A.nl_j[pos] = oj;
                      A.nl_d[pos] = dval;
                    }
                  }
                }
              } else if constexpr (OPK == OPK_SCALAR) {
                if (hit) {
                  if (op == 2) {
                    c_acc++;
                  } else if (sure) {
                    float uu, gg;
                    pair_value<float, T>(A, op, d2f, oi, oj, uu, gg);
                    e_part += (FA)uu;
                  } else {
                    V uu, gg;
                    pair_value<V, T>(A, op, (V)d2, oi, oj, uu, gg);
                    e_part += (FA)uu;
                  }
                }
              } else if constexpr (IS_F) {
                if (hit) {
                  FA uu, gg;
                  FA df[3] = {0, 0, 0};
                  FA dv[3] = {0, 0, 0};
                  if (sure) {
                    float uf, gf;
                    pair_value<float, T>(A, op, d2f, oi, oj, uf, gf);
                    uu = (FA)uf;
                    gg = (FA)gf;
#pragma unroll
                    for (int d = 0; d < N; d++) dv[d] = (FA)dvf[d];
                  } else {
                    V uv, gv;
                    pair_value<V, T>(A, op, (V)d2, oi, oj, uv, gv);
                    uu = (FA)uv;
                    gg = (FA)gv;
#pragma unroll
                    for (int d = 0; d < N; d++) dv[d] = (FA)dxs[d];
                  }
#pragma unroll
                  for (int d = 0; d < N; d++) df[d] = gg * dv[d];
                  if constexpr (OPK == OPK_ADJ) {
                    {
                      // virial W += g dx dx^T (g = u'(r)/r), and the parameter derivatives of the LJ term
                      adj[0] += gg * dv[0] * dv[0];
                      adj[1] += gg * dv[1] * dv[1];
                      adj[2] += gg * dv[2] * dv[2];
                      adj[3] += gg * dv[0] * dv[1];
                      adj[4] += gg * dv[0] * dv[2];
                      adj[5] += gg * dv[1] * dv[2];
                      FA eps = par<FA>(A, 0), sig = par<FA>(A, 1);
                      int cls = 0;
                      if (A.ntypes > 0) {
                        const int ti = A.tx[oi], tj = A.tx[oj];
                        eps = eps_tab<FA>(A, ti * A.ntypes + tj);
                        sig = sig_tab<FA>(A, ti * A.ntypes + tj);
                        cls = ti + tj;  // 2 types: AA = 0, AB = 1, BB = 2
                      }
                      const FA c12 = par<FA>(A, 2), c6 = par<FA>(A, 3);
                      const FA dd2 = sure ? (FA)d2f : (FA)d2;
                      const FA sr2 = sig * sig * vrcp(dd2);
                      const FA sr6 = sr2 * sr2 * sr2;
                      const FA sr12 = sr6 * sr6;
                      const FA lj = c12 * sr12 - c6 * sr6;
                      const FA dsg = eps * (FA(12) * c12 * sr12 - FA(6) * c6 * sr6) * vrcp(sig);
#pragma unroll
                      for (int k = 0; k < 3; k++) {
                        adj[6 + k] += (cls == k) ? lj : FA(0);
                        adj[9 + k] += (cls == k) ? dsg : FA(0);
                      }
                    }
                  }
#pragma unroll
                  for (int d = 0; d < N; d++) acc[d] -= df[d];
                  e_part += uu;
                  force_add<T, N, FA>(A, CROSS, idx_j, df);  // the partner's share
                }
              } else if constexpr (OPK == OPK_MIN) {
                if (hit) {
                  T dd2 = sure ? (T)d2f : d2;
                  if (sure && ABS_PF) {
                    T dx = xsub(xi[0], xj[0]);
                    dd2 = xmul(dx, dx);
#pragma unroll
                    for (int d = 1; d < N; d++) {
                      T dd = xsub(xi[d], xj[d]);
                      dd2 = xadd(dd2, xmul(dd, dd));
                    }
                  }
                  if (nonneg_lt(dd2, best_d2) ||
                      (!nonneg_lt(best_d2, dd2) && (oi < best_i || (oi == best_i && oj < best_j)))) {
                    best_d2 = dd2;
                    best_i = oi;
                    best_j = oj;
                  }
                }
              } else if constexpr (OPK == OPK_HIST) {
                int hb = -1;   // bin of this lane's pair (-1: none)
                FA hv = 0;     // its accumulator term
                if (hit) {
                  bool exact_r = !sure;
                  T r = 0;
                  float rfl = 0.f;  // the distance in FP32 for the FP32 pair value (no FP64 conversions)
                  double rinv = 0.0;  // exact form of Float64 handles: 1/r of the accumulator term
                  int b = -1;
                  if constexpr (std::is_same<FA, double>::value) {
                    // exact form (the d2 of the exact re-test): the bin from the FP32 distance, decided again
                    // from the IEEE distance when an edge lies within 2^-12 of it (as in the split form; the
                    // FP32 distance of the exact d2 is within 2^-23 of the IEEE one); the term's 1/r from the
                    // FP64 rsqrt estimate refined by one Newton step (vrsqrt_1nr), without an IEEE sqrt and
                    // divide per pair
                    const float rf = sqrtf((float)d2);
                    const int lo = first_edge_at_or_above(s_binf, A.nbins, rf);
                    b = lo - 1;
                    if (near_edge(s_binf, A.nbins, lo, rf)) b = first_edge_at_or_above(s_bins, A.nbins, xsqrt(d2)) - 1;
                    rinv = vrsqrt_1nr((double)d2);
                    exact_r = false;
                  } else if (sure) {
                    float rf = sqrtf(d2f);
                    const int lo = first_edge_at_or_above(s_binf, A.nbins, rf);
                    b = lo - 1;
                    if (near_edge(s_binf, A.nbins, lo, rf)) exact_r = true;  // an edge within 2^-12: decide exactly
                    rfl = rf;
                    if constexpr (!std::is_same<FA, float>::value) r = (T)rf;
                  }
                  if (exact_r) {
                    T e2 = d2;  // the exact re-test's d2 (not sure), or recomputed near a bin edge
                    if (sure) {
                      load_xi();
                      if constexpr (!ABS_PF) tjj = s_tj[bsel][warp][j];
                      load_xj();
                      T dx = xsub(xi[0], xj[0]);
                      e2 = xmul(dx, dx);
#pragma unroll
                      for (int d = 1; d < N; d++) {
                        T dd = xsub(xi[d], xj[d]);
                        e2 = xadd(e2, xmul(dd, dd));
                      }
                    }
                    r = xsqrt(e2);
                    rfl = (float)r;
                    b = first_edge_at_or_above(s_bins, A.nbins, r) - 1;
                  }
                  if (b >= 0 && b < A.nbins) {
                    FA dv[3] = {0, 0, 0};
                    if (sure) {
#pragma unroll
                      for (int d = 0; d < N; d++) dv[d] = (FA)dvf[d];
                    } else {
#pragma unroll
                      for (int d = 0; d < N; d++) dv[d] = (FA)dxs[d];
                    }
                    if (tri) {
                      FA rv[3];
#pragma unroll
                      for (int a = 0; a < N; a++) {
                        FA s = 0;
#pragma unroll
                        for (int k = 0; k < N; k++) s += (FA)gc.Rinv[a][k] * dv[k];
                        rv[a] = s;
                      }
#pragma unroll
                      for (int a = 0; a < N; a++) dv[a] = rv[a];
                    }
                    FA dot = 0;
                    if constexpr (std::is_same<FA, float>::value) {
                      // FP32 pair values: velocities converted once by the host code
                      const float* vy = CROSS ? A.vyf : A.vxf;
#pragma unroll
                      for (int d = 0; d < N; d++)
                        dot += (A.vxf[(int64_t)idx_i * N + d] - vy[(int64_t)idx_j * N + d]) * dv[d];
                      hv = dot * vrcp(rfl);
                    } else {
                      const T* vy = CROSS ? A.vy : A.vx;
#pragma unroll
                      for (int d = 0; d < N; d++)
                        dot += ((FA)A.vx[(int64_t)idx_i * N + d] - (FA)vy[(int64_t)idx_j * N + d]) * dv[d];
                      hv = dot * (FA)rinv;
                    }
                    hb = b;
                  }
                }
                // lanes holding the same bin are summed by a tree over their group; the group's first lane
                // then updates the warp's own bin (groups have distinct bins: no atomics)
                if (__any_sync(FULL, hb >= 0)) {
                  const unsigned peers = __match_any_sync(FULL, hb);
                  const FA v = group_sum(peers, hv, lane);
                  if (hb >= 0 && lane == __ffs(peers) - 1) {
                    s_ws[hb] += v;
                    s_wc[hb] += (unsigned)__popc(peers);
                  }
                }
              }
            }
            if constexpr (IS_F) {
              // lanes ending on the same particle are adjacent: sum each run of equal `cur` into its first
              // lane, which alone adds it to the particle's sums
              __syncwarp();
#pragma unroll
              for (int off = 1; off < 32; off <<= 1) {
                const int co = __shfl_down_sync(FULL, cur, off);
                FA t[3];
#pragma unroll
                for (int d = 0; d < N; d++) t[d] = __shfl_down_sync(FULL, acc[d], off);
                if (lane + off < 32 && co == cur) {
#pragma unroll
                  for (int d = 0; d < N; d++) acc[d] += t[d];
                }
              }
              const int cprev = __shfl_up_sync(FULL, cur, 1);
              if (cur >= 0 && (lane == 0 || cprev != cur)) {
#pragma unroll
                for (int d = 0; d < N; d++) s_if[warp][d][cur] += acc[d];
              }
            }
            };
            sweep(std::false_type());
            if (DEFER && __any_sync(FULL, marked)) {
              __syncwarp();
              sweep(std::true_type());
            }
            if constexpr (OPK == OPK_HIST) {
              // move the warp's bins (at most 1024 pairs of this round) into the block's FP64 bins
              __syncwarp();
              for (int b = lane; b < A.nbins; b += 32) {
                const unsigned c = s_wc[b];
                if (c) {
                  atomicAdd(&s_hc[b], (unsigned long long)c);
                  atomicAdd(&s_hs[b], (double)s_ws[b]);
                  s_wc[b] = 0u;
                  s_ws[b] = FA(0);
                }
              }
            }
            __syncwarp();
          }
          __syncwarp();
        }
      }
      e_tot += (double)e_part;
      e_part = 0;
      if constexpr (IS_F) {
        __syncwarp();
        FA f[3];
#pragma unroll
        for (int d = 0; d < 3; d++) f[d] = s_if[warp][d][il];
        if (grp == 0 && vi && (f[0] != FA(0) || f[1] != FA(0) || f[2] != FA(0)))
          force_add<T, N, FA>(A, false, idx_i, f);
        __syncwarp();
      }
    }
    if constexpr (BATCH) {
      // per work item partials, reduced per system in a fixed order afterwards
      double e = e_tot;
      unsigned long long c = c_acc;
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) {
        e += __shfl_xor_sync(FULL, e, s);
        c += __shfl_xor_sync(FULL, c, s);
      }
      if (lane == 0) {
        A.part_e[r] = e;
        A.part_c[r] = c;
      }
      e_tot = 0.0;
      c_acc = 0;
    }
  }
  if constexpr (BATCH) return;

  // ---------------- block reductions to per-block partials
  if constexpr (OPK == OPK_SCALAR || OPK == OPK_FORCES) {
    double e = e_tot;
    unsigned long long c = c_acc;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      e += __shfl_xor_sync(FULL, e, s);
      c += __shfl_xor_sync(FULL, c, s);
    }
    if (lane == 0) {
      s_red[warp] = e;
      s_redc[warp] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double es = 0;
      unsigned long long cs = 0;
      for (int k = 0; k < kWarps; k++) {
        es += s_red[k];
        cs += s_redc[k];
      }
      A.part_e[blockIdx.x] = es;
      A.part_c[blockIdx.x] = cs;
    }
  } else if constexpr (OPK == OPK_ADJ) {
    __shared__ double s_adj[kWarps][kAdjVals];
    double v[kAdjVals];
    v[0] = e_tot;
#pragma unroll
    for (int k = 1; k < kAdjVals; k++) v[k] = (double)adj[k - 1];
#pragma unroll
    for (int k = 0; k < kAdjVals; k++) {
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) v[k] += __shfl_xor_sync(FULL, v[k], s);
    }
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < kAdjVals; k++) s_adj[warp][k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < kAdjVals) {
      double acc = 0;
      for (int w = 0; w < kWarps; w++) acc += s_adj[w][threadIdx.x];
      A.part_v[(int64_t)blockIdx.x * kAdjVals + threadIdx.x] = acc;
    }
  } else if constexpr (OPK == OPK_MIN) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      T od = __shfl_xor_sync(FULL, best_d2, s);
      int oi_ = __shfl_xor_sync(FULL, best_i, s);
      int oj_ = __shfl_xor_sync(FULL, best_j, s);
      if (od < best_d2 || (od == best_d2 && (oi_ < best_i || (oi_ == best_i && oj_ < best_j)))) {
        best_d2 = od;
        best_i = oi_;
        best_j = oj_;
      }
    }
    __shared__ T s_md[kWarps];
    __shared__ int s_mi[kWarps], s_mj[kWarps];
    if (lane == 0) {
      s_md[warp] = best_d2;
      s_mi[warp] = best_i;
      s_mj[warp] = best_j;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      T bd = s_md[0];
      int bi = s_mi[0], bj = s_mj[0];
      for (int k = 1; k < kWarps; k++) {
        if (s_md[k] < bd || (s_md[k] == bd && (s_mi[k] < bi || (s_mi[k] == bi && s_mj[k] < bj)))) {
          bd = s_md[k];
          bi = s_mi[k];
          bj = s_mj[k];
        }
      }
      A.part_min_d2[blockIdx.x] = bd;
      A.part_min_ij[2 * blockIdx.x] = bi;
      A.part_min_ij[2 * blockIdx.x + 1] = bj;
    }
  } else if constexpr (OPK == OPK_HIST) {
    __syncthreads();
    for (int b = threadIdx.x; b < A.nbins; b += kThreads) {
      A.part_hc[(int64_t)blockIdx.x * A.nbins + b] = s_hc[b];
      A.part_hs[(int64_t)blockIdx.x * A.nbins + b] = s_hs[b];
    }
  }
}

// One wave of resident blocks (the warps loop over cells): grid = min(cells/warps, SMs x blocks per SM).
template <class K> int resident_grid(K kernel, int want, size_t dyn = 0) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, dyn) != cudaSuccess || per_sm <= 0) {
    cudaGetLastError();
    per_sm = 1;
  }
  return std::max(1, std::min(want, per_sm * sms));
}

template <class T, int N, int OPK, bool SPLIT, bool CROSS, bool BATCH = false, int OPC = 0>
cudaError_t launch_k(int& grid, cudaStream_t st, const PairArgs<T>& A) {
  auto k = k_pairs<T, N, OPK, SPLIT, CROSS, BATCH, OPC>;
  using FA = typename std::conditional<std::is_same<T, double>::value && !SPLIT, double, float>::type;
  size_t dyn = 0;
  if (OPK == OPK_HIST) {
    dyn = hist_smem(A.nbins, (int)sizeof(T), (int)sizeof(FA)).total;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
  }
  grid = resident_grid(k, grid, dyn);
  k<<<grid, kThreads, dyn, st>>>(A);
  return cudaGetLastError();
}

template <class T, int N, bool SPLIT, bool CROSS>
cudaError_t launch_s(int opk, int& grid, cudaStream_t st, const PairArgs<T>& A) {
  switch (opk) {
    case OPK_NL: return launch_k<T, N, OPK_NL, SPLIT, CROSS>(grid, st, A);
    case OPK_SCALAR: return launch_k<T, N, OPK_SCALAR, SPLIT, CROSS>(grid, st, A);
    case OPK_FORCES:
      if (A.op == 9) return launch_k<T, N, OPK_FORCES, SPLIT, CROSS, false, 9>(grid, st, A);  // LJ forces
      return launch_k<T, N, OPK_FORCES, SPLIT, CROSS>(grid, st, A);
    case OPK_MIN: return launch_k<T, N, OPK_MIN, SPLIT, CROSS>(grid, st, A);
    case OPK_HIST: return launch_k<T, N, OPK_HIST, SPLIT, CROSS>(grid, st, A);
    case OPK_ADJ:
      if constexpr (!CROSS) return launch_k<T, N, OPK_ADJ, SPLIT, false, false, 13>(grid, st, A);
      return cudaErrorInvalidValue;
  }
  return cudaErrorInvalidValue;
}

// Plain launches of one dtype: every operator kind, self and cross pairs, exact and split forms.
template <class T>
cudaError_t launch_plain_t(const LaunchSel& s, int& grid, cudaStream_t st, const PairArgs<T>& A) {
  if constexpr (std::is_same<T, float>::value) {
    // Float32 inputs: the split form is the exact form (the input arithmetic is FP32 already)
    if (s.dim == 3) return s.self ? launch_s<T, 3, false, false>(s.opk, grid, st, A) : launch_s<T, 3, false, true>(s.opk, grid, st, A);
    return s.self ? launch_s<T, 2, false, false>(s.opk, grid, st, A) : launch_s<T, 2, false, true>(s.opk, grid, st, A);
  } else {
    if (s.dim == 3) {
      if (s.self) return s.split ? launch_s<T, 3, true, false>(s.opk, grid, st, A) : launch_s<T, 3, false, false>(s.opk, grid, st, A);
      return s.split ? launch_s<T, 3, true, true>(s.opk, grid, st, A) : launch_s<T, 3, false, true>(s.opk, grid, st, A);
    }
    if (s.self) return s.split ? launch_s<T, 2, true, false>(s.opk, grid, st, A) : launch_s<T, 2, false, false>(s.opk, grid, st, A);
    return s.split ? launch_s<T, 2, true, true>(s.opk, grid, st, A) : launch_s<T, 2, false, true>(s.opk, grid, st, A);
  }
}

// Batched launches: self pairs of many systems; neighbour lists, scalar reductions and forces.
template <class T, int N, bool SPLIT>
cudaError_t launch_b(int opk, int& grid, cudaStream_t st, const PairArgs<T>& A) {
  switch (opk) {
    case OPK_NL: return launch_k<T, N, OPK_NL, SPLIT, false, true>(grid, st, A);
    case OPK_SCALAR: return launch_k<T, N, OPK_SCALAR, SPLIT, false, true>(grid, st, A);
    case OPK_FORCES: return launch_k<T, N, OPK_FORCES, SPLIT, false, true>(grid, st, A);
  }
  return cudaErrorInvalidValue;
}

template <class T>
cudaError_t launch_batch_t(const LaunchSel& s, int& grid, cudaStream_t st, const PairArgs<T>& A) {
  if (!s.self) return cudaErrorInvalidValue;
  if constexpr (std::is_same<T, float>::value) {
    return s.dim == 3 ? launch_b<T, 3, false>(s.opk, grid, st, A) : launch_b<T, 2, false>(s.opk, grid, st, A);
  } else {
    if (s.dim == 3) return s.split ? launch_b<T, 3, true>(s.opk, grid, st, A) : launch_b<T, 3, false>(s.opk, grid, st, A);
    return s.split ? launch_b<T, 2, true>(s.opk, grid, st, A) : launch_b<T, 2, false>(s.opk, grid, st, A);
  }
}

template <class K> int occupancy_of(K kernel) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return per_sm;
}

// Occupancy of the scalar and min-distance instantiations (the allocation-free entry point sizes its
// partials with it).  Float32 handles have no split instantiation (their split form is the exact one).
template <class T, int N, int OPK> int occupancy_pick(bool split, bool self) {
  if constexpr (std::is_same<T, float>::value) {
    (void)split;
    return self ? occupancy_of(k_pairs<T, N, OPK, false, false, false>) : occupancy_of(k_pairs<T, N, OPK, false, true, false>);
  } else {
    if (split)
      return self ? occupancy_of(k_pairs<T, N, OPK, true, false, false>) : occupancy_of(k_pairs<T, N, OPK, true, true, false>);
    return self ? occupancy_of(k_pairs<T, N, OPK, false, false, false>) : occupancy_of(k_pairs<T, N, OPK, false, true, false>);
  }
}

template <class T>
int occupancy_t(const LaunchSel& s) {
  if (s.opk == OPK_SCALAR)
    return s.dim == 3 ? occupancy_pick<T, 3, OPK_SCALAR>(s.split, s.self) : occupancy_pick<T, 2, OPK_SCALAR>(s.split, s.self);
  if (s.opk == OPK_MIN)
    return s.dim == 3 ? occupancy_pick<T, 3, OPK_MIN>(s.split, s.self) : occupancy_pick<T, 2, OPK_MIN>(s.split, s.self);
  return 0;
}

}  // namespace pk
}  // namespace clm
