// Argument block of the cell-pair map kernel and the launch interface shared by the host code
// (clm_pairs.cu) and the translation units that instantiate the kernel (clm_pairs_f32.cu,
// clm_pairs_f64.cu, clm_pairs_batch.cu).
#pragma once
#include <cuda_runtime.h>

#include "clm_device.cuh"
#include "clm_geometry.hpp"
#include "clm_internal.hpp"

namespace clm {
namespace pk {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;

template <class T> struct SetView {
  const T* px;
  const T* py;
  const T* pz;
  const float4* off;  // FP32 offsets from the cell origin; .w = particle code
  const float4* xq;   // Float32 handles: coordinates; .w = particle code
  const int* code;
  const int* cell_start;
  const int* cell_real;  // per cell: 1 when it holds a real particle
};

template <class T> struct PairArgs {
  DevGeom<T> g;
  SetView<T> X, Y;
  const int* real_list;
  const int* n_real_dev;  // number of cells with real particles (device)
  int self;
  int split;
  int op;
  int* err;
  // operator parameters
  double p[4];
  float pf[4];  // the same in FP32 (set by set_params)
  int ntypes;
  const int* tx;
  const int* ty;
  const double* eps_t;
  const double* sig_t;
  const float* eps_tf;  // the same tables in FP32 (pair values of the FP32 forms)
  const float* sig_tf;
  const T* vx;
  const T* vy;
  const T* bins;
  int nbins;
  const float* vxf;  // velocities in FP32 (pair values of the FP32 forms)
  const float* vyf;
  const double* wx;   // per-particle weights (WEIGHTED_INV_D) of x and y, and FP32 copies
  const double* wy;
  const float* wxf;
  const float* wyf;
  // outputs
  int* nl_i;
  int* nl_j;
  T* nl_d;
  unsigned long long* nl_count;
  long long nl_cap;
  // force sums in the rotated frame, added with atomics (f[i] -= df, f[j] += df for each visited pair):
  // FP32 pair values into one 16-byte record per particle, FP64 pair values into n * dim doubles
  float4* f4x;
  float4* f4y;      // cross: set y
  double* fx;
  double* fy;       // cross: set y
  double* part_e;   // per-block energy
  unsigned long long* part_c;  // per-block count
  T* part_min_d2;
  int* part_min_ij;
  unsigned long long* part_hc;  // nbins per block
  double* part_hs;              // nbins per block
  double* part_v;               // kAdjVals per block (adjoint)
  // work decomposition and batches of independent systems
  int cell_split;               // parts per cell: part p takes the particle chunks p, p + S, p + 2S, ...
  const DevGeom<T>* gtab;       // batch: geometry of each system
  const int* cell_sys;          // batch: system of each global cell
  const int* cbase;             // batch: first global cell of each system
};

// Operator parameters in both precisions.
template <class T> inline void set_params(PairArgs<T>& A, const double* p) {
  for (int k = 0; k < 4; k++) {
    A.p[k] = p[k];
    A.pf[k] = (float)p[k];
  }
}

enum OpKind { OPK_NL = 0, OPK_SCALAR = 1, OPK_FORCES = 2, OPK_MIN = 3, OPK_HIST = 4, OPK_ADJ = 5 };
constexpr int kAdjVals = 13;  // energy, virial (xx yy zz xy xz yz), dU/deps[3], dU/dsigma[3]

// Dynamic shared memory of the radial-histogram kernel: block bins (FP64 sums, 64-bit counts), the bin
// edges in the handle dtype and in FP32, and per-warp bins (sums in the accumulation type, counts).
struct HistSmem {
  size_t hs, hc, bins, binf, ws, wc, total;
};
__host__ __device__ inline HistSmem hist_smem(int nb, int tsize, int fsize) {
  auto up = [](size_t v) { return (v + 15) / 16 * 16; };
  HistSmem m;
  m.hs = 0;
  m.hc = up(m.hs + 8 * (size_t)nb);
  m.bins = up(m.hc + 8 * (size_t)nb);
  m.binf = up(m.bins + (size_t)tsize * (nb + 1));
  m.ws = up(m.binf + 4 * (size_t)(nb + 1));
  m.wc = up(m.ws + (size_t)fsize * kWarps * nb);
  m.total = up(m.wc + 4 * (size_t)kWarps * nb);
  return m;
}

// Which instantiation of the kernel a launch needs.
struct LaunchSel {
  int dim;     // 2 or 3
  int opk;     // OpKind
  bool self;   // one set (self pairs) or two (cross pairs)
  bool split;  // FP32-split arithmetic
  bool batch;  // many independent systems in one launch (self pairs only)
};

// Launch on `st` with at most `grid` blocks (one resident wave); `grid` returns the blocks used.
cudaError_t launch_pairs_plain(const LaunchSel& s, int& grid, cudaStream_t st, const PairArgs<float>& A);
cudaError_t launch_pairs_plain(const LaunchSel& s, int& grid, cudaStream_t st, const PairArgs<double>& A);
cudaError_t launch_pairs_batch(const LaunchSel& s, int& grid, cudaStream_t st, const PairArgs<float>& A);
cudaError_t launch_pairs_batch(const LaunchSel& s, int& grid, cudaStream_t st, const PairArgs<double>& A);
// Resident blocks per SM of that instantiation (0 if none).
int pairs_blocks_per_sm(const LaunchSel& s, const PairArgs<float>* tag);
int pairs_blocks_per_sm(const LaunchSel& s, const PairArgs<double>* tag);

template <class T> inline SetView<T> view_of(const SetData& S) {
  SetView<T> v;
  v.px = S.px.as<T>();
  v.py = S.py.as<T>();
  v.pz = S.pz.as<T>();
  v.off = S.off.as<float4>();
  v.xq = S.xq.as<float4>();
  v.code = S.code.as<int>();
  v.cell_start = S.cell_start.as<int>();
  v.cell_real = S.cell_flags.as<int>();
  return v;
}

inline int opkind_of(int op) {
  switch (op) {
    case 1: return OPK_NL;
    case 2: case 3: case 4: case 5: case 6: case 8: return OPK_SCALAR;
    case 7: case 9: case 12: case 14: return OPK_FORCES;
    case 13: return OPK_ADJ;
    case 10: return OPK_MIN;
    case 11: return OPK_HIST;
    default: return -1;
  }
}

template <class T> inline cudaError_t launch_pairs(const LaunchSel& s, int& grid, cudaStream_t st, const PairArgs<T>& A) {
  return s.batch ? launch_pairs_batch(s, grid, st, A) : launch_pairs_plain(s, grid, st, A);
}

}  // namespace pk
}  // namespace clm
