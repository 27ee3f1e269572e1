// Host-side state of a library handle (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "clm_device.cuh"
#include "clm_geometry.hpp"

namespace clm {

enum Status {
  RERUN_BUILD = -1,  // internal: the copies overflowed the capacity; rebuild with the exact size and rerun
  OK = 0, ERR_ARG = 1, ERR_CELL_TOO_SMALL = 2, ERR_NAN = 3, ERR_DIM = 4, ERR_CUDA = 5, ERR_CAPACITY = 6,
  ERR_STATE = 7, ERR_TIMEOUT = 8, ERR_NOMEM = 9, ERR_LCELL = 10, ERR_NONPERIODIC_CELL = 11, ERR_INTERNAL = 12
};

// Process-wide count and size of the device (and pinned host) allocations the library made; steady-state
// steps with unchanged sizes make none (reported by clm_device_allocations).
inline std::atomic<long long>& alloc_count() {
  static std::atomic<long long> c{0};
  return c;
}
inline std::atomic<long long>& alloc_bytes() {
  static std::atomic<long long> b{0};
  return b;
}

// Grow-only device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  // Ensures capacity for `nbytes`; returns false on allocation failure.
  bool reserve(size_t nbytes) {
    if (nbytes <= bytes && p) return true;
    size_t want = nbytes + nbytes / 4 + 256;
    void* q = nullptr;
    if (cudaMalloc(&q, want) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    alloc_count()++;
    alloc_bytes() += (long long)want;
    if (p) cudaFree(p);
    p = q;
    bytes = want;
    return true;
  }
  template <class U> U* as() const { return static_cast<U*>(p); }
};

// One particle set and its cell list on the device.
struct SetData {
  int64_t n = 0;
  bool dirty = true;
  bool built = false;
  DevBuf x;                 // positions as given (n x dim, column-major dim x n)
  DevBuf wrapped;           // wrapped (and rotated) positions, n x dim
  DevBuf mask;              // per particle: bit k set if image k lies in the computing box
  DevBuf ncopy, copy_off;   // copies per particle and their exclusive scan
  DevBuf keys[2], vals[2];  // (cell, particle<<5 | image) pairs: particle order, then grouped by cell
  DevBuf cell_count;        // one system: scan words and per-cell {copies, real} counters (zeroed per build)
  size_t cell_count_zero = 0;  // bytes of cell_count left cleared by the last build (0: clear before use)
  DevBuf cell_start, cell_flags;
  DevBuf real_list, real_scan;
  DevBuf px, py, pz;        // copies in cell order (SoA), handle dtype
  DevBuf off;               // FP32 cell-relative offsets (float4, .w = code) for the prefilter
  DevBuf xq;                // Float32 handles: coordinates (float4, .w = code)
  DevBuf code;              // particle index (>= 0 real copy, -(index+1) image)
  DevBuf rs_hist;
  DevBuf minmax;            // non-periodic limits scratch
  int64_t n_copies = 0;      // valid once the build was synchronized (pending == false)
  int64_t n_real_cells = 0;
  int64_t copy_cap = 0;      // capacity for copies learned from previous builds
  int64_t cap_used = 0;      // capacity used by the last build
  bool pending = false;      // the device totals of the last build were not read back yet
  bool counted = false;      // the last build was the counting build (its largest cell is read back)
  bool prefer_radix = false; // a counting build met a cell of more than kRadixAbovePerCell copies
  int tile_mult = 0;         // counting build: staging slots per particle of a tile (0: from the estimate)
  int64_t n_cells_with_particles = 0;
  int64_t ncells = 0;
};

struct ScanTemp {
  DevBuf level[4];
};

// Many independent periodic systems in one handle (one cell list over a global cell index; every
// system keeps its own box, cells and images).  Set 0 of the handle holds the concatenated positions.
struct BatchState {
  bool on = false;
  int64_t nsys = 0;
  int kind = 0;                  // ORTHO or TRICLINIC (all systems)
  int lcell = 1;
  double cutoff = 0;
  std::vector<int64_t> offsets;  // nsys + 1: particles of system s are offsets[s] .. offsets[s+1]-1
  std::vector<double> cells;     // nsys x dim x dim, column-major per system
  std::vector<int> status;       // per system: OK, ERR_CELL_TOO_SMALL, ERR_NAN
  std::vector<int> cbase;        // nsys + 1: first global cell of each system
  int64_t ncells = 0;            // total cells
  double real_cells = 0;         // cells with real particles (geometric estimate)
  double copies_est = 0;         // reals + images (uniform-density estimate)
  double pairs_est = 0;          // pairs within the cutoff (uniform-density estimate)
  bool tables_ready = false;     // device tables match (systems, lcell, precision)
  int tables_dtype = -1;
  DevBuf gtab;                   // DevGeom<T> per system
  DevBuf psys;                   // system of each particle
  DevBuf cbase_d;                // cbase on the device
  DevBuf cell_sys;               // system of each global cell
  DevBuf sys_err;                // per-system device error bits
  DevBuf part;                   // per work item partial sums and counts
  DevBuf sys_out;                // per op: per-system sums and counts
  DevBuf forces;                 // forces in the handle dtype (n x dim)
  int cell_split = 1;            // parts per cell (autotuned)
  int grid_div = 1;              // resident blocks per SM divided by this (autotuned)
  // one step (build + operators) captured as a CUDA graph
  bool use_graph = false;
  cudaGraphExec_t gexec = nullptr;
  std::vector<int> graph_ops;
  std::vector<double> graph_params;
  int64_t graph_n = -1;
  float step_ms = 0;
  int64_t step_launches = 0;
  int64_t graph_launches = 0;     // kernels in the recorded step
  unsigned char* hres = nullptr;  // pinned host results of one step
  size_t hres_bytes = 0;
  int nl_slot = -1;               // which op of the step produced the neighbour list
  ~BatchState() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (hres) cudaFreeHost(hres);
  }
};

struct Handle {
  int dtype = 1, dim = 3, nsets = 1;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool box_set = false;
  int kind = 0, lcell = 1;
  double M[9] = {};
  double cutoff = 0;
  int precision = 0;
  Geometry<double> gd;
  Geometry<float> gf;
  SetData sets[2];
  ScanTemp scan;
  DevBuf err;        // device error word
  DevBuf counters;   // device counters (NL count, etc.)
  DevBuf nl_i, nl_j, nl_d;
  int64_t nl_cap = 0, nl_n = 0;
  bool nl_valid = false;
  DevBuf partial;    // per-block partial reductions
  DevBuf opbuf;      // operator parameter staging (types, tables, velocities, bins)
  DevBuf outbuf;     // device outputs staged before copying to the caller
  int* pinned = nullptr;       // small pinned host staging area (256 bytes)
  unsigned char* pres = nullptr;  // pinned host copy of a map's results (kResultBytes)
  cudaEvent_t ev[4] = {};
  float build_ms = 0, map_ms = 0;
  bool build_timing_pending = false;
  int64_t launches = 0;        // kernels launched by this handle (cumulative)
  std::string last_error;
  BatchState batch;
  bool capturing = false;      // a stream capture is open: no synchronization, no timing events
};

// Results of one map on the device: scalar, count, minimum and its pair (first 256 bytes), histogram counts
// and sums (16 x 256 bytes), adjoint sums.
constexpr size_t kResultBytes = 256 + 16 * 256 + 128;

// Status helpers
#define CLM_CUDA_TRY(h, call)                                                            \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      (h).last_error = std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call; \
      return ERR_CUDA;                                                                   \
    }                                                                                    \
  } while (0)

// Build (clm_build.cu)
int scan_exclusive(Handle& h, const int* in, int* out, int64_t m, int* total, int depth = 0);
template <class T> int build_set(Handle& h, int set, const Geometry<T>& g);
int enqueue_build_totals(Handle& h);
int check_build_totals(Handle& h, bool* overflow);
template <class T> int set_limits(Handle& h, T* lo, T* hi);
template <class T> void fill_devgeom(const Geometry<T>& g, int precision, DevGeom<T>& d);

// Per-block partial slots that a scratch area of `scratch_bytes` holds for the allocation-free scalar map
// (the first 256 bytes hold the final result): an energy, a count, a minimum d2 in the handle dtype (tsize
// bytes) and its pair of indices per block.  A launch of more blocks than this is refused.
inline size_t noalloc_block_slots(size_t scratch_bytes, size_t tsize) {
  const size_t slot = sizeof(double) + sizeof(unsigned long long) + tsize + 2 * sizeof(int);
  return scratch_bytes > 256 ? (scratch_bytes - 256) / slot : 0;
}

// Map (clm_pairs.cu)
struct OpRequest;
template <class T> int run_pairs(Handle& h, const Geometry<T>& g, int op, const void* params, void* outputs);
template <class T>
int run_pairs_scalar_scratch(Handle& h, const Geometry<T>& g, int op, const void* params, void* outputs, void* scratch,
                             size_t scratch_bytes);
int pairs_scalar_blocks_needed(Handle& h, int op);
template <class T> int cell_split_for(const Handle& h, const Geometry<T>& g, int opk);

}  // namespace clm
