// Cell-list construction on the GPU.
//
// Replaces UpdateCellList! (src/internals/CellLists.jl:727-927, serial order
// of add_particles! 940-950 and add_particle_to_celllist! 983-1057) and the
// non-periodic build (src/internals/NonPeriodicCells.jl:93-251).
//
// One system (counting build, four launches after one memset):
//   k_wrap_emit     wrap into the first cell (wrap_to_first, CellOperations.jl:91-94),
//                   rotate, test the 3^N-1 translation images against the computing
//                   box (replicate_particle!, Box.jl:556-566), scan the copies per
//                   particle (decoupled look-back), write one (cell, particle<<5|image)
//                   key/value per copy (particle_cell + real_particle_border_case), and
//                   count the copies of every cell (atomic adds)
//   k_cell_scan     cell starts and the list of cells that contain real particles
//   k_cell_scatter  copies to their cells' slots in arrival order (atomic cursors)
//   k_rank_gather   each copy to its rank by value inside its cell (particle-index
//                   order, the reference's serial order), with its coordinates (SoA),
//                   particle code and 16-byte candidate record
// One system with crowded cells (more than kCountingMaxPerCell copies per cell
// expected): k_wrap_emit without the counters, a stable LSD radix sort of the keys by
// cell, k_gather (cell starts from the sorted keys) and k_compact_1pass.
// Batches (global cell index over all systems): k_wrap_count_b, a scan of the
// copies, k_emit_b, the radix sort, k_gather_b, and the real-cell scan and
// compaction.
//
// Every kernel bounds-checks its indices; inconsistencies set bits of the
// handle's device error word instead of faulting.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "clm_build_steps.cuh"
#include "clm_internal.hpp"

namespace clm {

namespace {

constexpr int kBlock = 256;

// ------------------------------------------------------------------ scan
constexpr int SCAN_IPT = 8;
constexpr int SCAN_TILE = kBlock * SCAN_IPT;

// Single-pass exclusive scan with decoupled look-back: tiles take increasing tickets, publish their
// aggregate, then one warp reads the published words of the 32 preceding tiles at a time (aggregate or
// inclusive prefix) and sums back to the nearest inclusive prefix.  A tile only waits on tiles that took their tickets before it (and
// so are running); every wait is bounded, and a tile that gives up sets DERR_SCAN and carries on.
// status[t]: (state << 32) | value, state 1 = aggregate, 2 = inclusive prefix; zeroed before the launch
// together with the ticket counter.  In-place use (in == out) is safe: a tile reads only its own inputs.
constexpr unsigned long long kScanAgg = 1ull << 32, kScanPrefix = 2ull << 32;
constexpr int kScanSpinLimit = 1 << 20;

// Decoupled look-back of tile `tile` (called by one whole warp of the tile's block): publishes the tile's aggregate,
// sums the published words of earlier tiles back to the nearest inclusive prefix, publishes the tile's own
// inclusive prefix and returns its exclusive prefix (in every lane).
__device__ __forceinline__ int lookback(int tile, int agg, unsigned long long* __restrict__ status,
                                        int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  int excl = 0;
  if (tile == 0) {
    if (lane == 0) atomicExch(&status[0], kScanPrefix | (unsigned)agg);
    return 0;
  }
  if (lane == 0) atomicExch(&status[tile], kScanAgg | (unsigned)agg);
  // look back over windows of 32 earlier tiles (lane k reads tile top - k; below tile 0 reads as a zero
  // prefix) until a window holds an inclusive prefix with every nearer tile published
  int top = tile - 1;
  int spins = 0;
  bool gave_up = false;
  while (true) {
    const int jj = top - lane;
    unsigned long long wd = 2ull << 32;  // a zero inclusive prefix below tile 0
    if (jj >= 0) wd = *(volatile unsigned long long*)&status[jj];
    const unsigned long long state = wd & ~0xffffffffull;
    const unsigned pend = __ballot_sync(0xffffffffu, state == 0ull);
    const unsigned pref = __ballot_sync(0xffffffffu, state == kScanPrefix);
    const int first = pref ? __ffs(pref) - 1 : 31;  // nearest prefix, or the whole window
    const unsigned need = (first == 31) ? 0xffffffffu : ((2u << first) - 1u);
    if (pend & need) {
      if (++spins > kScanSpinLimit) {
        gave_up = true;
        break;
      }
      __nanosleep(32);
      continue;
    }
    int val = (lane <= first) ? (int)(unsigned)(wd & 0xffffffffull) : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
    excl += val;
    if (pref & need) break;
    top -= 32;
  }
  if (lane == 0) {
    if (gave_up) atomicOr(err, DERR_SCAN);
    atomicExch(&status[tile], kScanPrefix | (unsigned)(excl + agg));
  }
  return excl;
}

// Exclusive scan of the block's NT x IPT values v (thread-major), in place; returns the block aggregate to
// every thread and leaves in `thread_off` the exclusive prefix of this thread's first value.  wsum holds
// NT / 32 + 1 ints (NT <= 1024).
template <int IPT, int NT = kBlock>
__device__ __forceinline__ int block_scan(int (&v)[IPT], int& thread_off, int* wsum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int s = 0;
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    const int t = v[k];
    v[k] = s;
    s += t;
  }
  int incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  int agg = 0;
  if (warp == 0) {
    int w = (lane < NT / 32) ? wsum[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < NT / 32) wsum[lane] = wi - w;
    const int a = __shfl_sync(0xffffffffu, wi, NT / 32 - 1);
    if (lane == 0) wsum[NT / 32] = a;
  }
  __syncthreads();
  agg = wsum[NT / 32];
  thread_off = (incl - s) + wsum[warp];
  return agg;
}

__global__ void __launch_bounds__(kBlock) k_scan_1pass(const int* in, int* out, int64_t m, int* __restrict__ total,
                                                       unsigned long long* __restrict__ status,
                                                       unsigned* __restrict__ ticket, int64_t ntiles,
                                                       int* __restrict__ err) {
  __shared__ int wsum[kBlock / 32 + 1];
  __shared__ int s_tile, s_excl;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(ticket, 1u);
  __syncthreads();
  const int tile = s_tile;
  const int64_t base = (int64_t)tile * SCAN_TILE + (int64_t)threadIdx.x * SCAN_IPT;
  int v[SCAN_IPT];
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    int64_t idx = base + k;
    v[k] = (idx < m) ? in[idx] : 0;
  }
  int off = 0;
  const int agg = block_scan<SCAN_IPT>(v, off, wsum);
  if (threadIdx.x < 32) {
    const int excl = lookback(tile, agg, status, err);
    if (threadIdx.x == 0) {
      s_excl = excl;
      if (total && tile == ntiles - 1) *total = excl + agg;
    }
  }
  __syncthreads();
  off += s_excl;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    int64_t idx = base + k;
    if (idx < m) out[idx] = v[k] + off;
  }
}

__global__ void __launch_bounds__(kBlock) k_scan_tiles(const int* __restrict__ in, int* __restrict__ out, int64_t m,
                                                       int* __restrict__ tile_sums) {
  __shared__ int wsum[kBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_IPT;
  int v[SCAN_IPT];
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    int64_t idx = base + k;
    int t = (idx < m) ? in[idx] : 0;
    v[k] = s;
    s += t;
  }
  int incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = (lane < kBlock / 32) ? wsum[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < kBlock / 32) wsum[lane] = wi - w;
  }
  __syncthreads();
  const int off = (incl - s) + wsum[warp];
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    int64_t idx = base + k;
    if (idx < m) out[idx] = v[k] + off;
  }
  if (threadIdx.x == kBlock - 1) tile_sums[blockIdx.x] = off + s;
}

// ------------------------------------------------------------------ radix sort (8-bit digits)
constexpr int RS_IPT = 8;
constexpr int RS_TILE = kBlock * RS_IPT;  // 2048 keys per tile
constexpr int RS_WARPS = kBlock / 32;

// B-bit digits (8..10): the host picks the fewest passes that cover the cell index and the smallest
// digit that does it.
template <int B>
__global__ void __launch_bounds__(kBlock) k_rs_hist(const uint32_t* __restrict__ keys, const int* __restrict__ n_dev,
                                                    int cap, int shift, int* __restrict__ hist, int ntiles) {
  constexpr int D = 1 << B;
  __shared__ int h[D];
  const int n = min(*n_dev, cap);
  for (int d = threadIdx.x; d < D; d += kBlock) h[d] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
#pragma unroll
  for (int k = 0; k < RS_IPT; k++) {
    int64_t idx = base + (int64_t)k * kBlock + threadIdx.x;
    if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & (uint32_t)(D - 1)], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < D; d += kBlock) hist[(int64_t)d * ntiles + blockIdx.x] = h[d];
}

// Stable scatter: items of a tile are ranked in tile order (warp, then item
// slot, then lane) with warp-level match_any, then placed at the scanned
// digit offset of the tile.
template <int B>
__global__ void __launch_bounds__(kBlock) k_rs_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                       uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                       const int* __restrict__ n_dev, int cap, int shift,
                                                       const int* __restrict__ offs, int ntiles) {
  constexpr int D = 1 << B;
  __shared__ int wcnt[RS_WARPS][D + 1];
  const int n = min(*n_dev, cap);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < RS_WARPS * (D + 1); d += kBlock) (&wcnt[0][0])[d] = 0;
  __syncthreads();
  const int64_t wbase = (int64_t)blockIdx.x * RS_TILE + (int64_t)warp * (32 * RS_IPT);
  uint32_t kk[RS_IPT], vv[RS_IPT];
  int rank[RS_IPT], dig[RS_IPT];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < RS_IPT; k++) {
    int64_t idx = wbase + k * 32 + lane;
    bool valid = idx < n;
    kk[k] = valid ? kin[idx] : 0u;
    vv[k] = valid ? vin[idx] : 0u;
    int d = valid ? (int)((kk[k] >> shift) & (uint32_t)(D - 1)) : D;
    dig[k] = d;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    int leader = __ffs(peers) - 1;
    int cur = wcnt[warp][d];
    __syncwarp();
    if (lane == leader) wcnt[warp][d] = cur + __popc(peers);
    __syncwarp();
    rank[k] = cur + __popc(peers & lt);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < D; d += kBlock) {
    int run = offs[(int64_t)d * ntiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) {
      int t = wcnt[w][d];
      wcnt[w][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < RS_IPT; k++) {
    if (dig[k] < D) {
      int pos = wcnt[warp][dig[k]] + rank[k];
      if (pos >= 0 && pos < n) {
        kout[pos] = kk[k];
        vout[pos] = vv[k];
      }
    }
  }
}

// ------------------------------------------------------------------ batches: wrap, images, copy count
// (the per-particle step, wrap_count_at, is in clm_build_steps.cuh)
// Each particle uses its system's geometry; a NaN marks only its system; particles of systems
// that failed the unit-cell check get no copies.
template <class T, int N>
__global__ void __launch_bounds__(kBlock) k_wrap_count_b(const DevGeom<T>* __restrict__ gtab,
                                                         const int* __restrict__ psys, const T* __restrict__ x, int n,
                                                         T* __restrict__ wrapped, uint32_t* __restrict__ mask,
                                                         int* __restrict__ ncopy, int* __restrict__ sys_err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = psys[i];
  const DevGeom<T>& g = gtab[s];
  if (g.ncells == 0) {
#pragma unroll
    for (int k = 0; k < N; k++) wrapped[(int64_t)i * N + k] = T(0);
    mask[i] = 0;
    ncopy[i] = 0;
    return;
  }
  if (!wrap_count_at<T, N>(g, x, i, wrapped, mask, ncopy)) atomicOr(&sys_err[s], DERR_NAN);
}

// ------------------------------------------------------------------ batches: keys of every copy
template <class T, int N>
__global__ void __launch_bounds__(kBlock) k_emit_b(const DevGeom<T>* __restrict__ gtab, const int* __restrict__ psys,
                                                   const int* __restrict__ cbase, const T* __restrict__ wrapped,
                                                   const uint32_t* __restrict__ mask, const int* __restrict__ ncopy,
                                                   const int* __restrict__ copy_off, int n, int cap,
                                                   uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                   int* __restrict__ err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = psys[i];
  emit_at<T, N>(gtab[s], cbase[s], wrapped, mask, ncopy, copy_off, i, cap, keys, vals, err);
}

// ------------------------------------------------------------------ one system: wrap, scan and keys in one pass
// Each tile of WE_TILE particles wraps its particles and tests their images (wrap_count_regs), scans the
// copy counts in particle order, takes the copy offset of its first particle by decoupled look-back, and
// writes the key and value of every copy (the cells of copy_cell, in emit_copies' order): the same copies at
// the same positions as a separate wrap kernel, scan and key kernel would.  The last tile writes the total number of copies.  With
// COUNT, every copy also adds one to its cell's counter and the real copy marks its cell (cell_cf holds
// {copies, holds a real particle} per cell, zeroed before the launch); the adds return nothing, so no thread
// waits on them.  The wrapped positions are stored for the gather; the rest stays in registers.
constexpr int WE_PPT = 1;
// One system: above this many expected copies per cell the build sorts by radix instead of counting; a set
// whose counting build met a cell of more than kRadixAbovePerCell copies (clustered particles, which the
// uniform-density estimate misses) is built by radix from then on: the in-cell ranking costs a cell's size
// per copy, the radix sort does not depend on it.
constexpr double kCountingMaxPerCell = 64.0;
constexpr int kRadixAbovePerCell = 1024;
constexpr int WE_BLOCK = 256;  // threads (particles) per tile of the wrap kernel
constexpr int WE_TILE = WE_BLOCK * WE_PPT;

template <class T, int N>
__global__ void __launch_bounds__(WE_BLOCK) k_wrap_emit(DevGeom<T> g, const T* __restrict__ x, int n,
                                                      T* __restrict__ wrapped, int cap, uint32_t* __restrict__ keys,
                                                      uint32_t* __restrict__ vals, int* __restrict__ total,
                                                      unsigned long long* __restrict__ status,
                                                      unsigned* __restrict__ ticket, int ntiles,
                                                      int* __restrict__ err) {
  static_assert(WE_PPT == 1, "one particle per thread");
  __shared__ int wsum[WE_BLOCK / 32 + 1];
  __shared__ int s_tile, s_excl;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(ticket, 1u);
  __syncthreads();
  const int tile = s_tile;
  const int i = tile * WE_TILE + threadIdx.x;  // this thread's particle
  T p[N];
  uint32_t m = 0u;
  int v[1] = {0};
  if (i < n) {
    if (!wrap_count_regs<T, N>(g, x, i, p, m, v[0])) atomicOr(err, DERR_NAN);
#pragma unroll
    for (int d = 0; d < N; d++) wrapped[(int64_t)i * N + d] = p[d];
  }
  int nc = v[0];
  int off = 0;
  const int agg = block_scan<1, WE_BLOCK>(v, off, wsum);
  if (threadIdx.x < 32) {
    const int excl = lookback(tile, agg, status, err);
    if (threadIdx.x == 0) {
      s_excl = excl;
      if (tile == ntiles - 1) *total = excl + agg;
    }
  }
  __syncthreads();
  const int base = v[0] + off + s_excl;
  if (nc > 0 && (base < 0 || base + nc > cap)) {
    atomicOr(err, DERR_COPY_OVERFLOW);  // the build is repeated with the exact size
    nc = 0;
  }
  // the copies of the particle: the real copy, then the images in increasing image code
  for (int c = 0; c < nc; c++) {
    int k = g.zero_code;
    if (c > 0) {
      k = lowest_bit(m);
      m &= m - 1u;
    }
    keys[base + c] = (uint32_t)copy_cell<T, N>(g, p, k, err);
    vals[base + c] = ((uint32_t)i << 5) | (uint32_t)k;
  }
}

// One system, counting build: the same wrap, image tests and keys, with the copies of each tile of
// WE_BLOCK particles in the tile's own range of `slots` staging slots (the in-cell ranking orders a cell by
// value, so the copies need no position in particle order, and no tile waits on an earlier one).  Each
// tile writes its number of copies; a tile with more copies than slots writes none and flags
// DERR_TILE_OVERFLOW (the build is repeated with more slots).  Every copy adds one to its cell's counter
// (the lanes of a warp whose copies share a cell with one add) and the real copy marks its cell; cell_cf
// holds {copies, holds a real particle} per cell, zeroed before the launch.  Tile 0 clears the word of
// the largest cell that k_cell_scan finds.
template <class T, int N, int SH = kShapeGeneral>
__global__ void __launch_bounds__(WE_BLOCK) k_wrap_stage(DevGeom<T> g, const T* __restrict__ x, int n,
                                                       T* __restrict__ wrapped, int slots, uint32_t* __restrict__ keys,
                                                       uint32_t* __restrict__ vals, int* __restrict__ tile_count,
                                                       int* __restrict__ cell_cf, int* __restrict__ max_cell,
                                                       int* __restrict__ err) {
  static_assert(WE_PPT == 1, "one particle per thread");
  __shared__ int wsum[WE_BLOCK / 32 + 1];
  const int tile = blockIdx.x;
  const int i = tile * WE_TILE + threadIdx.x;  // this thread's particle
  if (tile == 0 && threadIdx.x == 0) *max_cell = 0;
  T p[N];
  uint32_t m = 0u;
  int v[1] = {0};
  if (i < n) {
    if (!wrap_count_regs<T, N, SH>(g, x, i, p, m, v[0])) atomicOr(err, DERR_NAN);
#pragma unroll
    for (int d = 0; d < N; d++) wrapped[(int64_t)i * N + d] = p[d];
  }
  int nc = v[0];
  int off = 0;
  const int agg = block_scan<1, WE_BLOCK>(v, off, wsum);
  if (agg > slots) nc = 0;  // the whole tile (agg is the tile's)
  if (threadIdx.x == 0) {
    tile_count[tile] = (agg > slots) ? 0 : agg;
    if (agg > slots) atomicOr(err, DERR_TILE_OVERFLOW);
  }
  const int64_t base = (int64_t)tile * slots + v[0] + off;
  // the copies of the particle (the real copy, then the images in increasing image code), walked by the
  // lanes of a warp together: in each round the lanes whose copies fall in the same cell add to that cell's
  // counter with one add (match_any groups them)
  const int lane = threadIdx.x & 31;
  const int rounds = __reduce_max_sync(0xffffffffu, nc);
  for (int c = 0; c < rounds; c++) {
    uint32_t key = 0xffffffffu;  // no copy in this round
    if (c < nc) {
      int k = g.zero_code;
      if (c > 0) {
        k = lowest_bit(m);
        m &= m - 1u;
      }
      key = (uint32_t)copy_cell<T, N>(g, p, k, err);
      keys[base + c] = key;
      vals[base + c] = ((uint32_t)i << 5) | (uint32_t)k;
      if (c == 0) cell_cf[2 * key + 1] = 1;  // the cell holds a real particle
    }
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (key != 0xffffffffu && lane == __ffs(peers) - 1) atomicAdd(&cell_cf[2 * key], __popc(peers));
  }
}

// Cell starts and the list of cells with real particles, in one pass over cell_cf: each tile scans its
// cells' copy counts and real flags, takes both prefixes by decoupled look-back (warp 0 the counts, warp 1
// the flags; one ticket orders the tiles of both), and writes cell_start, the real flags the pair kernel
// reads, and the real cells in linear order.  The last tile closes cell_start and writes the number of
// real cells.  Each cell's counters are cleared after reading: they are the scatter's cursors next.
__global__ void __launch_bounds__(kBlock) k_cell_scan(int* __restrict__ cell_cf, int ncells,
                                                      int* __restrict__ cell_start, int* __restrict__ cell_flags,
                                                      int* __restrict__ real_list, int* __restrict__ n_real,
                                                      int* __restrict__ max_cell,
                                                      unsigned long long* __restrict__ status_c,
                                                      unsigned long long* __restrict__ status_f,
                                                      unsigned* __restrict__ ticket, int ntiles,
                                                      int* __restrict__ err) {
  __shared__ int wsum_c[kBlock / 32 + 1], wsum_f[kBlock / 32 + 1];
  __shared__ int s_tile, s_excl_c, s_excl_f;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(ticket, 1u);
  __syncthreads();
  const int tile = s_tile;
  const int c0 = tile * SCAN_TILE + threadIdx.x * SCAN_IPT;
  int vc[SCAN_IPT], vf[SCAN_IPT], f[SCAN_IPT];
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    int2 cf = make_int2(0, 0);
    if (c0 + k < ncells) {
      cf = reinterpret_cast<const int2*>(cell_cf)[c0 + k];
      reinterpret_cast<int2*>(cell_cf)[c0 + k] = make_int2(0, 0);
    }
    vc[k] = cf.x;
    f[k] = cf.y != 0;
    vf[k] = f[k];
  }
  {
    int m = 0;  // the largest cell of this thread's, then of the warp's
#pragma unroll
    for (int k = 0; k < SCAN_IPT; k++) m = max(m, vc[k]);
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(max_cell, m);
  }
  int off_c = 0, off_f = 0;
  const int agg_c = block_scan<SCAN_IPT>(vc, off_c, wsum_c);
  const int agg_f = block_scan<SCAN_IPT>(vf, off_f, wsum_f);
  const int warp = threadIdx.x >> 5;
  if (warp == 0) {
    const int excl = lookback(tile, agg_c, status_c, err);
    if (threadIdx.x == 0) {
      s_excl_c = excl;
      if (tile == ntiles - 1) cell_start[ncells] = excl + agg_c;
    }
  } else if (warp == 1) {
    const int excl = lookback(tile, agg_f, status_f, err);
    if ((threadIdx.x & 31) == 0) {
      s_excl_f = excl;
      if (tile == ntiles - 1) *n_real = excl + agg_f;
    }
  }
  __syncthreads();
  off_c += s_excl_c;
  off_f += s_excl_f;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    const int c = c0 + k;
    if (c < ncells) {
      cell_start[c] = vc[k] + off_c;
      cell_flags[c] = f[k];
      if (f[k]) real_list[vf[k] + off_f] = c;
    }
  }
}

// Every staged copy to its cell's slots in arrival order: block b walks the tile_count[b] copies staged in
// tile b's slots, 256 at a time.  The copies of one warp that share a cell take consecutive slots with one
// atomic on the cell's cursor (cleared by k_cell_scan).  The sorted keys and values come out grouped by cell,
// each cell's values in arrival order; a total beyond `cap` is flagged (the build is repeated larger).
__global__ void __launch_bounds__(kBlock) k_cell_scatter(const uint32_t* __restrict__ keys,
                                                         const uint32_t* __restrict__ vals,
                                                         const int* __restrict__ tile_count, int slots, int cap,
                                                         int ncells, const int* __restrict__ cell_start,
                                                         int* __restrict__ cursor, uint32_t* __restrict__ skeys,
                                                         uint32_t* __restrict__ svals, int* __restrict__ err) {
  const int count = min(tile_count[blockIdx.x], slots);
  const int64_t first_slot = (int64_t)blockIdx.x * slots;
  const int lane = threadIdx.x & 31;
  for (int at = 0; at < count; at += kBlock) {  // the same trip count in every thread
    const int j = at + (int)threadIdx.x;
    uint32_t li = 0xffffffffu;  // no copy
    if (j < count) {
      li = keys[first_slot + j];
      if (li >= (uint32_t)ncells) {
        atomicOr(err, DERR_CELL_RANGE);
        li = 0xffffffffu;
      }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, li);
    const int leader = __ffs(peers) - 1;
    int first = 0;
    if (li != 0xffffffffu && lane == leader) first = atomicAdd(&cursor[2 * li], __popc(peers));
    first = __shfl_sync(0xffffffffu, first, leader);
    if (li == 0xffffffffu) continue;
    const int pos = cell_start[li] + first + __popc(peers & ((1u << lane) - 1u));
    if (pos < 0 || pos >= cell_start[li + 1]) {
      atomicOr(err, DERR_CELL_RANGE);
      continue;
    }
    if (pos >= cap) {
      atomicOr(err, DERR_COPY_OVERFLOW);
      continue;
    }
    skeys[pos] = li;
    svals[pos] = vals[first_slot + j];
  }
}

// The gather after the counting placement: slot q of the placed list holds a copy of cell li in arrival order; the
// copy's final slot is the cell's start plus its rank by value in the cell (rank_in_cell), which puts
// every cell in particle-index order.  The copy's coordinates, code and 16-byte record are written there.
// The scan words and per-cell counters (`zero`, `zwords` 64-bit words), used for the last time by the
// scatter, are cleared for the next build.
template <class T, int N>
__global__ void __launch_bounds__(kBlock) k_rank_gather(DevGeom<T> g, const T* __restrict__ wrapped,
                                                        const uint32_t* __restrict__ skeys,
                                                        const uint32_t* __restrict__ svals,
                                                        const int* __restrict__ cell_start, int ncells, int cap, int n,
                                                        T* __restrict__ px, T* __restrict__ py, T* __restrict__ pz,
                                                        float4* __restrict__ off, float4* __restrict__ xq,
                                                        int* __restrict__ code, int* __restrict__ cell_flags,
                                                        unsigned long long* __restrict__ zero, int64_t zwords,
                                                        int* __restrict__ err) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t w = q; w < zwords; w += (int64_t)gridDim.x * blockDim.x) zero[w] = 0ull;
  const int tot = min(cell_start[ncells], cap);
  if (q >= tot) return;
  const uint32_t li = skeys[q];
  const uint32_t v = svals[q];
  if (li >= (uint32_t)ncells) {
    atomicOr(err, DERR_CELL_RANGE);
    return;
  }
  const int s = cell_start[li];
  const int e = min(cell_start[li + 1], tot);
  const int t = s + rank_in_cell(svals, s, e, v);
  int p = (int)(v >> 5);
  int k = (int)(v & 31u);
  if (t < s || t >= e || p >= n || k >= g.nimg) {
    atomicOr(err, DERR_CELL_RANGE);
    return;
  }
  gather_at<T, N>(g, wrapped, t, p, k, (int)li, px, py, pz, off, xq, code, cell_flags, 0);
}

// Crowded cells (radix path of one system): the cells with real particles, in linear order, in one pass:
// each tile scans its cells' flags, takes its first slot by decoupled look-back, and lists its flagged
// cells; the last tile writes their number.
__global__ void __launch_bounds__(kBlock) k_compact_1pass(const int* __restrict__ flags, int ncells,
                                                          int* __restrict__ list, int* __restrict__ total,
                                                          unsigned long long* __restrict__ status,
                                                          unsigned* __restrict__ ticket, int ntiles,
                                                          int* __restrict__ err) {
  __shared__ int wsum[kBlock / 32 + 1];
  __shared__ int s_tile, s_excl;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(ticket, 1u);
  __syncthreads();
  const int tile = s_tile;
  const int c0 = tile * SCAN_TILE + threadIdx.x * SCAN_IPT;
  int v[SCAN_IPT], f[SCAN_IPT];
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    f[k] = (c0 + k < ncells && flags[c0 + k]) ? 1 : 0;
    v[k] = f[k];
  }
  int off = 0;
  const int agg = block_scan<SCAN_IPT>(v, off, wsum);
  if (threadIdx.x < 32) {
    const int excl = lookback(tile, agg, status, err);
    if (threadIdx.x == 0) {
      s_excl = excl;
      if (tile == ntiles - 1) *total = excl + agg;
    }
  }
  __syncthreads();
  off += s_excl;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++)
    if (f[k]) list[v[k] + off] = c0 + k;
}

// ------------------------------------------------------------------ gather in cell order after the radix sort
// One system: copy t of the sorted keys
template <class T, int N>
__global__ void __launch_bounds__(kBlock) k_gather(DevGeom<T> g, const T* __restrict__ wrapped,
                                                   const uint32_t* __restrict__ skeys,
                                                   const uint32_t* __restrict__ svals, const int* __restrict__ n_dev,
                                                   int cap, int n, T* __restrict__ px, T* __restrict__ py,
                                                   T* __restrict__ pz, float4* __restrict__ off, float4* __restrict__ xq,
                                                   int* __restrict__ code, int* __restrict__ cell_flags,
                                                   int ncells, int* __restrict__ cell_start, int* __restrict__ err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = min(*n_dev, cap);
  if (t > nc) return;
  cell_starts_at(skeys, t, nc, ncells, cell_start);
  if (t == nc) return;
  uint32_t v = svals[t];
  int p = (int)(v >> 5);
  int k = (int)(v & 31u);
  int li = (int)skeys[t];
  if (p >= n || k >= g.nimg || li < 0 || li >= g.ncells) {
    atomicOr(err, DERR_CELL_RANGE);
    p = 0;
    k = g.zero_code;
    li = 0;
  }
  gather_at<T, N>(g, wrapped, t, p, k, li, px, py, pz, off, xq, code, cell_flags, 0);
}

template <class T, int N>
__global__ void __launch_bounds__(kBlock) k_gather_b(const DevGeom<T>* __restrict__ gtab, const int* __restrict__ psys,
                                                     const int* __restrict__ cbase, const T* __restrict__ wrapped,
                                                     const uint32_t* __restrict__ skeys,
                                                     const uint32_t* __restrict__ svals, const int* __restrict__ n_dev,
                                                     int cap, int n, T* __restrict__ px, T* __restrict__ py,
                                                     T* __restrict__ pz, float4* __restrict__ off,
                                                     float4* __restrict__ xq, int* __restrict__ code,
                                                     int* __restrict__ cell_flags, int ncells,
                                                     int* __restrict__ cell_start, int* __restrict__ err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = min(*n_dev, cap);
  if (t > nc) return;
  cell_starts_at(skeys, t, nc, ncells, cell_start);
  if (t == nc) return;
  uint32_t v = svals[t];
  int p = (int)(v >> 5);
  int k = (int)(v & 31u);
  if (p >= n) {
    atomicOr(err, DERR_CELL_RANGE);
    p = 0;
  }
  const int s = psys[p];
  const DevGeom<T>& g = gtab[s];
  int li = (int)skeys[t] - cbase[s];
  if (k >= g.nimg || li < 0 || li >= g.ncells) {
    atomicOr(err, DERR_CELL_RANGE);
    k = g.zero_code;
    li = 0;
  }
  gather_at<T, N>(g, wrapped, t, p, k, li, px, py, pz, off, xq, code, cell_flags, cbase[s]);
}

__global__ void k_compact(const int* __restrict__ flags, const int* __restrict__ scanned, int ncells,
                          int* __restrict__ list) {
  int li = blockIdx.x * blockDim.x + threadIdx.x;
  if (li >= ncells) return;
  if (flags[li]) list[scanned[li]] = li;
}

template <class T, int N>
__global__ void __launch_bounds__(kBlock) k_minmax(const T* __restrict__ x, int n, T* __restrict__ part) {
  __shared__ T smin[N][kBlock], smax[N][kBlock];
  T lo[N], hi[N];
#pragma unroll
  for (int d = 0; d < N; d++) {
    lo[d] = INFINITY;
    hi[d] = -INFINITY;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int d = 0; d < N; d++) {
      T v = x[(int64_t)i * N + d];
      lo[d] = fmin(lo[d], v);
      hi[d] = fmax(hi[d], v);
    }
  }
#pragma unroll
  for (int d = 0; d < N; d++) {
    smin[d][threadIdx.x] = lo[d];
    smax[d][threadIdx.x] = hi[d];
  }
  __syncthreads();
  for (int s = kBlock / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
#pragma unroll
      for (int d = 0; d < N; d++) {
        smin[d][threadIdx.x] = fmin(smin[d][threadIdx.x], smin[d][threadIdx.x + s]);
        smax[d][threadIdx.x] = fmax(smax[d][threadIdx.x], smax[d][threadIdx.x + s]);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int d = 0; d < N; d++) {
      part[(int64_t)blockIdx.x * 2 * N + d] = smin[d][0];
      part[(int64_t)blockIdx.x * 2 * N + N + d] = smax[d][0];
    }
  }
}

inline int grid_for(int64_t n, int block = kBlock) { return (int)std::max<int64_t>(1, (n + block - 1) / block); }

}  // namespace

// ------------------------------------------------------------------ host side
int scan_exclusive(Handle& h, const int* in, int* out, int64_t m, int* total, int depth) {
  if (m <= 0) {
    if (total) CLM_CUDA_TRY(h, cudaMemsetAsync(total, 0, sizeof(int), h.stream));
    return OK;
  }
  if (depth < 0 || depth >= 4) {
    h.last_error = "scan buffer index out of range";
    return ERR_INTERNAL;
  }
  int64_t ntiles = (m + SCAN_TILE - 1) / SCAN_TILE;
  if (ntiles == 1) {
    k_scan_tiles<<<1, kBlock, 0, h.stream>>>(in, out, m, total);
    CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches++;
    return OK;
  }
  // one launch: tile status words and the ticket counter, zeroed first
  DevBuf& sb = h.scan.level[depth];
  if (!sb.reserve((size_t)(ntiles + 2) * sizeof(unsigned long long))) return ERR_NOMEM;
  unsigned long long* status = sb.as<unsigned long long>();
  unsigned* ticket = reinterpret_cast<unsigned*>(status + ntiles);
  CLM_CUDA_TRY(h, cudaMemsetAsync(status, 0, (size_t)(ntiles + 1) * sizeof(unsigned long long), h.stream));
  k_scan_1pass<<<(unsigned)ntiles, kBlock, 0, h.stream>>>(in, out, m, total, status, ticket, ntiles,
                                                         h.err.as<int>());
  CLM_CUDA_TRY(h, cudaGetLastError());
  h.launches++;
  return OK;
}

template <class T> int set_limits(Handle& h, T* lo, T* hi) {
  // limits over x (and y for two sets): src/internals/CellOperations.jl:262-324
  const int N = h.dim;
  bool any = false;
  T glo[3], ghi[3];
  for (int s = 0; s < h.nsets; s++) {
    SetData& S = h.sets[s];
    T slo[3] = {0, 0, 0}, shi[3] = {0, 0, 0};
    if (S.n > 0) {
      int nb = std::min<int64_t>(1024, (S.n + kBlock - 1) / kBlock);
      if (!S.minmax.reserve(sizeof(T) * 2 * N * nb)) return ERR_NOMEM;
      if (N == 3) k_minmax<T, 3><<<nb, kBlock, 0, h.stream>>>(S.x.as<T>(), (int)S.n, S.minmax.as<T>());
      else k_minmax<T, 2><<<nb, kBlock, 0, h.stream>>>(S.x.as<T>(), (int)S.n, S.minmax.as<T>());
      CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches++;
      std::vector<T> part((size_t)(2 * N * nb));
      CLM_CUDA_TRY(h, cudaMemcpyAsync(part.data(), S.minmax.p, part.size() * sizeof(T), cudaMemcpyDeviceToHost, h.stream));
      CLM_CUDA_TRY(h, cudaStreamSynchronize(h.stream));
      for (int d = 0; d < N; d++) {
        slo[d] = part[d];
        shi[d] = part[N + d];
      }
      for (int b = 1; b < nb; b++)
        for (int d = 0; d < N; d++) {
          slo[d] = geo::jmin(slo[d], part[(size_t)b * 2 * N + d]);
          shi[d] = geo::jmax(shi[d], part[(size_t)b * 2 * N + N + d]);
        }
    }
    for (int d = 0; d < N; d++) {
      glo[d] = any ? geo::jmin(glo[d], slo[d]) : slo[d];
      ghi[d] = any ? geo::jmax(ghi[d], shi[d]) : shi[d];
    }
    any = true;
  }
  for (int d = 0; d < N; d++) {
    lo[d] = glo[d];
    hi[d] = ghi[d];
  }
  return OK;
}

// Capacity for the copies (reals + images) of a set: the largest of the previous build's count and the
// uniform-density estimate (computing-box volume / unit-cell volume), with a margin.  The build never
// waits for the device: if the copies exceed the capacity, the key kernel flags it, the result is discarded at
// the next host synchronization and the build is repeated with the exact size.
template <class T> int64_t copy_capacity(const SetData& S, const Geometry<T>& g) {
  const int64_t n = S.n;
  if (g.kind == NONPERIODIC) return n + 64;
  double vbox = 1.0;
  for (int i = 0; i < g.dim; i++) vbox *= (double)g.cbmax[i] - (double)g.cbmin[i];
  const double vcell = std::fabs((double)g.det_in);
  double est = (vcell > 0) ? (double)n * vbox / vcell : 27.0 * (double)n;
  est = std::min(est * 1.15 + 4096.0, 27.0 * (double)n + 64.0);
  return std::max<int64_t>(std::max<int64_t>(S.copy_cap, (int64_t)est), n + 64);
}

// One system: the counting build.  One zeroed region holds the look-back words of the cell scan and the
// per-cell {copies, real} counters; then four launches: wrap + keys staged per tile + cell counts
// (k_wrap_stage), cell starts + real-cell list (k_cell_scan), placement by arrival (k_cell_scatter), and the
// gather at each copy's rank in its cell (k_rank_gather).  The number of copies is the last cell start.
template <class T>
int build_counting(Handle& h, SetData& S, const DevGeom<T>& dg, int N, int64_t n, int64_t ncells, int64_t cap) {
  int* err = h.err.as<int>();
  const int64_t tiles = (n + WE_TILE - 1) / WE_TILE;
  const int64_t ct = (ncells + SCAN_TILE - 1) / SCAN_TILE;
  // staging slots per tile: a few per particle, from the capacity's copies per particle (more after a tile
  // overflowed), a multiple of 32
  if (S.tile_mult <= 0) S.tile_mult = (int)std::min<int64_t>(27, std::max<int64_t>(2, (cap * 5 / 4 + n - 1) / n + 1));
  const int slots = WE_BLOCK * S.tile_mult;
  const int64_t nslots = tiles * slots;
  // 64-bit words: cell-scan count status + ticket, cell-scan flag status, then the per-cell counters (two ints
  // per cell)
  const int64_t w_c = ct + 1, w_f = ct;
  const size_t zero_bytes = sizeof(unsigned long long) * (size_t)(w_c + w_f + ncells + 1);
  const void* zero_at = S.cell_count.p;
  if (!S.cell_count.reserve(zero_bytes) || !S.wrapped.reserve(sizeof(T) * N * n) ||
      !S.ncopy.reserve(sizeof(int) * (tiles + 1)) || !S.keys[0].reserve(sizeof(uint32_t) * nslots) ||
      !S.vals[0].reserve(sizeof(uint32_t) * nslots) || !S.keys[1].reserve(sizeof(uint32_t) * cap) ||
      !S.vals[1].reserve(sizeof(uint32_t) * cap) || !S.px.reserve(sizeof(T) * cap) ||
      !S.py.reserve(sizeof(T) * cap) || !S.pz.reserve(sizeof(T) * cap) ||
      !S.off.reserve(std::is_same<T, float>::value ? 16 : sizeof(float4) * cap) || !S.code.reserve(sizeof(int) * cap) ||
      !S.xq.reserve(std::is_same<T, float>::value ? sizeof(float4) * cap : 16))
    return ERR_NOMEM;
  if (S.cell_count.p != zero_at) S.cell_count_zero = 0;  // a new allocation holds no cleared words
  unsigned long long* z = S.cell_count.as<unsigned long long>();
  unsigned long long* st_c = z;
  unsigned long long* st_f = st_c + w_c;
  int* cell_cf = reinterpret_cast<int*>(st_f + w_f);
  // cleared by the previous build's gather unless the region grew or moved
  if (S.cell_count_zero < zero_bytes) CLM_CUDA_TRY(h, cudaMemsetAsync(z, 0, zero_bytes, h.stream));
  S.cell_count_zero = 0;
  int* tile_count = S.ncopy.as<int>();
  int* max_cell = S.copy_off.as<int>() + n + 1;  // the largest cell
  // Float64 3D cells whose input matrix has exact zeros take a wrap that skips them (wrap_point_shaped)
  bool shaped = false;
  if constexpr (std::is_same<T, double>::value) {
    if (N == 3 && dg.shape == kShapeDiag) {
      k_wrap_stage<T, 3, kShapeDiag><<<(unsigned)tiles, WE_BLOCK, 0, h.stream>>>(
          dg, S.x.as<T>(), (int)n, S.wrapped.as<T>(), slots, S.keys[0].as<uint32_t>(), S.vals[0].as<uint32_t>(),
          tile_count, cell_cf, max_cell, err);
      shaped = true;
    } else if (N == 3 && dg.shape == kShapeUpper) {
      k_wrap_stage<T, 3, kShapeUpper><<<(unsigned)tiles, WE_BLOCK, 0, h.stream>>>(
          dg, S.x.as<T>(), (int)n, S.wrapped.as<T>(), slots, S.keys[0].as<uint32_t>(), S.vals[0].as<uint32_t>(),
          tile_count, cell_cf, max_cell, err);
      shaped = true;
    }
  }
  if (!shaped && N == 3)
    k_wrap_stage<T, 3><<<(unsigned)tiles, WE_BLOCK, 0, h.stream>>>(dg, S.x.as<T>(), (int)n, S.wrapped.as<T>(), slots,
                                                                  S.keys[0].as<uint32_t>(), S.vals[0].as<uint32_t>(),
                                                                  tile_count, cell_cf, max_cell, err);
  else if (!shaped)
    k_wrap_stage<T, 2><<<(unsigned)tiles, WE_BLOCK, 0, h.stream>>>(dg, S.x.as<T>(), (int)n, S.wrapped.as<T>(), slots,
                                                                  S.keys[0].as<uint32_t>(), S.vals[0].as<uint32_t>(),
                                                                  tile_count, cell_cf, max_cell, err);
  CLM_CUDA_TRY(h, cudaGetLastError());
  h.launches++;
  k_cell_scan<<<(unsigned)ct, kBlock, 0, h.stream>>>(cell_cf, (int)ncells, S.cell_start.as<int>(), S.cell_flags.as<int>(),
                                                     S.real_list.as<int>(), S.real_scan.as<int>() + ncells, max_cell,
                                                     st_c, st_f, reinterpret_cast<unsigned*>(st_c + ct), (int)ct, err);
  CLM_CUDA_TRY(h, cudaGetLastError());
  h.launches++;
  k_cell_scatter<<<(unsigned)tiles, kBlock, 0, h.stream>>>(S.keys[0].as<uint32_t>(), S.vals[0].as<uint32_t>(),
                                                           tile_count, slots, (int)cap, (int)ncells,
                                                           S.cell_start.as<int>(), cell_cf, S.keys[1].as<uint32_t>(),
                                                           S.vals[1].as<uint32_t>(), err);
  CLM_CUDA_TRY(h, cudaGetLastError());
  h.launches++;
  const int gc = grid_for(cap);
  const int64_t zwords = (int64_t)(zero_bytes / sizeof(unsigned long long));
  if (N == 3)
    k_rank_gather<T, 3><<<gc, kBlock, 0, h.stream>>>(dg, S.wrapped.as<T>(), S.keys[1].as<uint32_t>(),
                                                     S.vals[1].as<uint32_t>(), S.cell_start.as<int>(), (int)ncells,
                                                     (int)cap, (int)n, S.px.as<T>(), S.py.as<T>(), S.pz.as<T>(),
                                                     S.off.as<float4>(), S.xq.as<float4>(), S.code.as<int>(),
                                                     S.cell_flags.as<int>(), z, zwords, err);
  else
    k_rank_gather<T, 2><<<gc, kBlock, 0, h.stream>>>(dg, S.wrapped.as<T>(), S.keys[1].as<uint32_t>(),
                                                     S.vals[1].as<uint32_t>(), S.cell_start.as<int>(), (int)ncells,
                                                     (int)cap, (int)n, S.px.as<T>(), S.py.as<T>(), S.pz.as<T>(),
                                                     S.off.as<float4>(), S.xq.as<float4>(), S.code.as<int>(),
                                                     S.cell_flags.as<int>(), z, zwords, err);
  CLM_CUDA_TRY(h, cudaGetLastError());
  h.launches++;
  S.cell_count_zero = zero_bytes;
  return OK;
}

template <class T> int build_set(Handle& h, int set, const Geometry<T>& g) {
  SetData& S = h.sets[set];
  const int N = g.dim;
  const int64_t n = S.n;
  const bool batch = h.batch.on;
  const int64_t ncells = batch ? h.batch.ncells : g.ncells();
  if (batch && (!h.batch.tables_ready || set != 0)) {
    h.last_error = "batch tables are not ready";
    return ERR_STATE;
  }
  if (ncells > (int64_t)1 << 30) {
    h.last_error = "too many cells for the cell grid (reduce lcell or enlarge cutoff)";
    return ERR_ARG;
  }
  S.ncells = ncells;
  DevGeom<T> dg;
  fill_devgeom(g, h.precision, dg);
  int* err = h.err.as<int>();
  if (!S.cell_start.reserve(sizeof(int) * (ncells + 1)) || !S.cell_flags.reserve(sizeof(int) * (ncells + 1)) ||
      !S.real_scan.reserve(sizeof(int) * (ncells + 1)) || !S.real_list.reserve(sizeof(int) * (ncells + 1)) ||
      !S.copy_off.reserve(sizeof(int) * (n + 2)))  // copies per particle scan, total, largest cell
    return ERR_NOMEM;
  if (n == 0) CLM_CUDA_TRY(h, cudaMemsetAsync(S.cell_flags.p, 0, sizeof(int) * (ncells + 1), h.stream));
  S.built = true;
  S.dirty = false;
  S.pending = true;
  if (n == 0) {
    CLM_CUDA_TRY(h, cudaMemsetAsync(S.cell_start.p, 0, sizeof(int) * (ncells + 1), h.stream));
    CLM_CUDA_TRY(h, cudaMemsetAsync(S.real_scan.p, 0, sizeof(int) * (ncells + 1), h.stream));
    CLM_CUDA_TRY(h, cudaMemsetAsync(S.copy_off.p, 0, sizeof(int), h.stream));
    S.cap_used = 0;
    S.counted = false;
    return OK;
  }
  int64_t cap = 0;
  if (batch) {
    const double est = std::min(h.batch.copies_est * 1.15 + 4096.0, 27.0 * (double)n + 64.0);
    cap = std::max<int64_t>(std::max<int64_t>(S.copy_cap, (int64_t)est), n + 64);
    CLM_CUDA_TRY(h, cudaMemsetAsync(h.batch.sys_err.p, 0, sizeof(int) * (h.batch.nsys + 1), h.stream));
  } else {
    cap = copy_capacity(S, g);
  }
  if (cap > (int64_t)INT32_MAX - 1) {
    h.last_error = "too many particle copies for one set";
    return ERR_ARG;
  }
  if (n >= ((int64_t)1 << 27)) {
    h.last_error = "at most 2^27 - 1 particles per set";
    return ERR_ARG;
  }
  S.cap_used = cap;
  // One system: the counting build, unless the cells are expected to be crowded (copies per cell from the
  // uniform-density capacity): its in-cell ranking takes a cell's size in steps per copy, where the radix
  // sort's cost does not depend on it.  Either gives the same cell list.
  const bool crowded = !batch && (S.prefer_radix || (double)cap > kCountingMaxPerCell * (double)ncells);
  S.counted = !batch && !crowded;
  if (S.counted) return build_counting<T>(h, S, dg, N, n, ncells, cap);
  // the radix path's gather sets the real flags of the cells it fills
  CLM_CUDA_TRY(h, cudaMemsetAsync(S.cell_flags.p, 0, sizeof(int) * (ncells + 1), h.stream));
  const int ntiles = (int)((cap + RS_TILE - 1) / RS_TILE);
  if (!S.wrapped.reserve(sizeof(T) * N * n) || !S.mask.reserve(sizeof(uint32_t) * n) ||
      !S.ncopy.reserve(sizeof(int) * (n + 1)) || !S.keys[0].reserve(sizeof(uint32_t) * cap) ||
      !S.keys[1].reserve(sizeof(uint32_t) * cap) || !S.vals[0].reserve(sizeof(uint32_t) * cap) ||
      !S.vals[1].reserve(sizeof(uint32_t) * cap) || !S.px.reserve(sizeof(T) * cap) || !S.py.reserve(sizeof(T) * cap) ||
      !S.pz.reserve(sizeof(T) * cap) || !S.off.reserve(std::is_same<T, float>::value ? 16 : sizeof(float4) * cap) || !S.code.reserve(sizeof(int) * cap) ||
      !S.xq.reserve(std::is_same<T, float>::value ? sizeof(float4) * cap : 16) ||
      !S.rs_hist.reserve(sizeof(int) * (1024 * (int64_t)ntiles + 1)))
    return ERR_NOMEM;
  const int gn = grid_for(n);
  const DevGeom<T>* gtab = h.batch.gtab.as<DevGeom<T>>();
  const int* psys = h.batch.psys.as<int>();
  const int* cbase = h.batch.cbase_d.as<int>();
  int* n_dev = S.copy_off.as<int>() + n;  // total number of copies, on the device
  int st = OK;
  if (!batch) {
    // wrap, images, copy offsets and keys in one launch (tile status words and ticket zeroed first)
    const int we_tiles = (int)((n + WE_TILE - 1) / WE_TILE);
    DevBuf& sb = h.scan.level[0];
    if (!sb.reserve((size_t)(we_tiles + 2) * sizeof(unsigned long long))) return ERR_NOMEM;
    unsigned long long* status = sb.as<unsigned long long>();
    CLM_CUDA_TRY(h, cudaMemsetAsync(status, 0, (size_t)(we_tiles + 1) * sizeof(unsigned long long), h.stream));
    unsigned* ticket = reinterpret_cast<unsigned*>(status + we_tiles);
    if (N == 3)
      k_wrap_emit<T, 3><<<we_tiles, WE_BLOCK, 0, h.stream>>>(dg, S.x.as<T>(), (int)n, S.wrapped.as<T>(), (int)cap,
                                                            S.keys[0].as<uint32_t>(), S.vals[0].as<uint32_t>(), n_dev,
                                                            status, ticket, we_tiles, err);
    else
      k_wrap_emit<T, 2><<<we_tiles, WE_BLOCK, 0, h.stream>>>(dg, S.x.as<T>(), (int)n, S.wrapped.as<T>(), (int)cap,
                                                            S.keys[0].as<uint32_t>(), S.vals[0].as<uint32_t>(), n_dev,
                                                            status, ticket, we_tiles, err);
    CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches++;
  } else {
    if (N == 3)
      k_wrap_count_b<T, 3><<<gn, kBlock, 0, h.stream>>>(gtab, psys, S.x.as<T>(), (int)n, S.wrapped.as<T>(),
                                                       S.mask.as<uint32_t>(), S.ncopy.as<int>(), h.batch.sys_err.as<int>());
    else
      k_wrap_count_b<T, 2><<<gn, kBlock, 0, h.stream>>>(gtab, psys, S.x.as<T>(), (int)n, S.wrapped.as<T>(),
                                                       S.mask.as<uint32_t>(), S.ncopy.as<int>(), h.batch.sys_err.as<int>());
    CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches++;
    st = scan_exclusive(h, S.ncopy.as<int>(), S.copy_off.as<int>(), n, n_dev);
    if (st) return st;
    if (N == 3)
      k_emit_b<T, 3><<<gn, kBlock, 0, h.stream>>>(gtab, psys, cbase, S.wrapped.as<T>(), S.mask.as<uint32_t>(),
                                                 S.ncopy.as<int>(), S.copy_off.as<int>(), (int)n, (int)cap,
                                                 S.keys[0].as<uint32_t>(), S.vals[0].as<uint32_t>(), err);
    else
      k_emit_b<T, 2><<<gn, kBlock, 0, h.stream>>>(gtab, psys, cbase, S.wrapped.as<T>(), S.mask.as<uint32_t>(),
                                                 S.ncopy.as<int>(), S.copy_off.as<int>(), (int)n, (int)cap,
                                                 S.keys[0].as<uint32_t>(), S.vals[0].as<uint32_t>(), err);
    CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches++;
  }
  // stable LSD radix sort by cell (the global cell for batches): the fewest passes of at most 10-bit digits,
  // digits as small as that allows
  int bits = 1;
  while (((int64_t)1 << bits) < ncells) bits++;
  const int passes = (bits + 9) / 10;
  const int dbits = std::max(8, (bits + passes - 1) / passes);
  int cur = 0;
  for (int pss = 0; pss < passes; pss++) {
    const int shift = dbits * pss;
    const int64_t hn = ((int64_t)1 << dbits) * ntiles;
    auto hist = (dbits == 8) ? k_rs_hist<8> : (dbits == 9) ? k_rs_hist<9> : k_rs_hist<10>;
    hist<<<ntiles, kBlock, 0, h.stream>>>(S.keys[cur].as<uint32_t>(), n_dev, (int)cap, shift, S.rs_hist.as<int>(), ntiles);
    CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches++;
    st = scan_exclusive(h, S.rs_hist.as<int>(), S.rs_hist.as<int>(), hn, S.rs_hist.as<int>() + hn);
    if (st) return st;
    auto scat = (dbits == 8) ? k_rs_scatter<8> : (dbits == 9) ? k_rs_scatter<9> : k_rs_scatter<10>;
    scat<<<ntiles, kBlock, 0, h.stream>>>(S.keys[cur].as<uint32_t>(), S.vals[cur].as<uint32_t>(),
                                          S.keys[1 - cur].as<uint32_t>(), S.vals[1 - cur].as<uint32_t>(), n_dev, (int)cap,
                                          shift, S.rs_hist.as<int>(), ntiles);
    CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches++;
    cur = 1 - cur;
  }
  // gather coordinates in cell order; cell offsets from the sorted keys
  const int gc = grid_for(cap + 1);  // copies, plus one thread that closes cell_start
  if (!batch) {
    if (N == 3)
      k_gather<T, 3><<<gc, kBlock, 0, h.stream>>>(dg, S.wrapped.as<T>(), S.keys[cur].as<uint32_t>(),
                                                 S.vals[cur].as<uint32_t>(), n_dev, (int)cap, (int)n, S.px.as<T>(),
                                                 S.py.as<T>(), S.pz.as<T>(), S.off.as<float4>(), S.xq.as<float4>(),
                                                 S.code.as<int>(), S.cell_flags.as<int>(), (int)ncells,
                                                 S.cell_start.as<int>(), err);
    else
      k_gather<T, 2><<<gc, kBlock, 0, h.stream>>>(dg, S.wrapped.as<T>(), S.keys[cur].as<uint32_t>(),
                                                 S.vals[cur].as<uint32_t>(), n_dev, (int)cap, (int)n, S.px.as<T>(),
                                                 S.py.as<T>(), S.pz.as<T>(), S.off.as<float4>(), S.xq.as<float4>(),
                                                 S.code.as<int>(), S.cell_flags.as<int>(), (int)ncells,
                                                 S.cell_start.as<int>(), err);
    CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches++;
    // cells with real particles, in linear order; their number stays on the device (real_scan[ncells])
    const int ct = (int)((ncells + SCAN_TILE - 1) / SCAN_TILE);
    DevBuf& sb = h.scan.level[0];
    if (!sb.reserve((size_t)(ct + 2) * sizeof(unsigned long long))) return ERR_NOMEM;
    unsigned long long* status = sb.as<unsigned long long>();
    CLM_CUDA_TRY(h, cudaMemsetAsync(status, 0, (size_t)(ct + 1) * sizeof(unsigned long long), h.stream));
    k_compact_1pass<<<ct, kBlock, 0, h.stream>>>(S.cell_flags.as<int>(), (int)ncells, S.real_list.as<int>(),
                                                 S.real_scan.as<int>() + ncells, status,
                                                 reinterpret_cast<unsigned*>(status + ct), ct, err);
    CLM_CUDA_TRY(h, cudaGetLastError());
    h.launches++;
    return OK;
  }
  if (N == 3)
    k_gather_b<T, 3><<<gc, kBlock, 0, h.stream>>>(gtab, psys, cbase, S.wrapped.as<T>(), S.keys[cur].as<uint32_t>(),
                                                 S.vals[cur].as<uint32_t>(), n_dev, (int)cap, (int)n, S.px.as<T>(),
                                                 S.py.as<T>(), S.pz.as<T>(), S.off.as<float4>(), S.xq.as<float4>(),
                                                 S.code.as<int>(), S.cell_flags.as<int>(), (int)ncells,
                                                 S.cell_start.as<int>(), err);
  else
    k_gather_b<T, 2><<<gc, kBlock, 0, h.stream>>>(gtab, psys, cbase, S.wrapped.as<T>(), S.keys[cur].as<uint32_t>(),
                                                 S.vals[cur].as<uint32_t>(), n_dev, (int)cap, (int)n, S.px.as<T>(),
                                                 S.py.as<T>(), S.pz.as<T>(), S.off.as<float4>(), S.xq.as<float4>(),
                                                 S.code.as<int>(), S.cell_flags.as<int>(), (int)ncells,
                                                 S.cell_start.as<int>(), err);
  CLM_CUDA_TRY(h, cudaGetLastError());
  h.launches++;
  // cells with real particles, in linear order; batches also read the per-cell scan (the items of each
  // system); their number stays on the device (real_scan[ncells])
  st = scan_exclusive(h, S.cell_flags.as<int>(), S.real_scan.as<int>(), ncells, S.real_scan.as<int>() + ncells);
  if (st) return st;
  k_compact<<<grid_for(ncells), kBlock, 0, h.stream>>>(S.cell_flags.as<int>(), S.real_scan.as<int>(), (int)ncells,
                                                       S.real_list.as<int>());
  CLM_CUDA_TRY(h, cudaGetLastError());
  h.launches++;
  return OK;
}

// Reads the device totals of the last build of every set (after the caller synchronized the stream
// through `staged`, which the caller filled with enqueue_build_totals) and checks the error word.
int enqueue_build_totals(Handle& h) {
  for (int s = 0; s < h.nsets; s++) {
    SetData& S = h.sets[s];
    if (!S.pending) continue;
    // the number of copies: the copy-offset scan's total, or (counting build) the last cell start
    const int* copies = S.counted ? S.cell_start.as<int>() + S.ncells : S.copy_off.as<int>() + S.n;
    CLM_CUDA_TRY(h, cudaMemcpyAsync(h.pinned + 32 + 2 * s, copies, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    CLM_CUDA_TRY(h, cudaMemcpyAsync(h.pinned + 33 + 2 * s, S.real_scan.as<int>() + S.ncells, sizeof(int),
                                    cudaMemcpyDeviceToHost, h.stream));
    if (S.counted)
      CLM_CUDA_TRY(h, cudaMemcpyAsync(h.pinned + 44 + s, S.copy_off.as<int>() + S.n + 1, sizeof(int),
                                      cudaMemcpyDeviceToHost, h.stream));
  }
  CLM_CUDA_TRY(h, cudaMemcpyAsync(h.pinned + 40, h.err.p, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
  return OK;
}

int check_build_totals(Handle& h, bool* overflow) {
  *overflow = false;
  const int errw = h.pinned[40];
  if (errw & DERR_NAN) {
    for (int s = 0; s < h.nsets; s++) h.sets[s].dirty = true;
    h.last_error = "Invalid coordinates found (NaN) in the particle positions.";
    return ERR_NAN;
  }
  for (int s = 0; s < h.nsets; s++) {
    SetData& S = h.sets[s];
    if (!S.pending) continue;
    if (h.pinned[32 + 2 * s] < 0) {  // the 32-bit copy-offset scan wrapped: more than 2^31 - 1 copies
      S.pending = false;
      S.dirty = true;
      h.last_error = "too many particle copies for one set (particles and their periodic images exceed 2^31 - 1)";
      return ERR_ARG;
    }
    S.n_copies = h.pinned[32 + 2 * s];
    S.n_real_cells = h.pinned[33 + 2 * s];
    if (S.counted && h.pinned[44 + s] > kRadixAbovePerCell) S.prefer_radix = true;
    if (S.counted && (errw & DERR_TILE_OVERFLOW)) {
      // a tile had more copies than its staging slots: more slots per particle, and build again
      S.tile_mult = std::min(27, 2 * S.tile_mult);
      S.dirty = true;
      *overflow = true;
    }
    S.pending = false;
    if (S.n_copies > S.cap_used || (errw & DERR_COPY_OVERFLOW)) {
      S.copy_cap = S.n_copies + S.n_copies / 8 + 1024;
      S.dirty = true;
      *overflow = true;
    } else if (S.n_copies > S.copy_cap) {
      S.copy_cap = S.n_copies;
    }
  }
  if (errw & DERR_SCAN) {
    h.last_error = "cell-list build: a scan tile gave up waiting for an earlier tile";
    return ERR_INTERNAL;
  }
  if (!*overflow && (errw & DERR_CELL_RANGE)) {
    h.last_error = "cell-list build consistency check failed (particle outside the computing box)";
    return ERR_INTERNAL;
  }
  return OK;
}

template void fill_devgeom<float>(const Geometry<float>&, int, DevGeom<float>&);
template void fill_devgeom<double>(const Geometry<double>&, int, DevGeom<double>&);
template int build_set<float>(Handle&, int, const Geometry<float>&);
template int build_set<double>(Handle&, int, const Geometry<double>&);
template int set_limits<float>(Handle&, float*, float*);
template int set_limits<double>(Handle&, double*, double*);

}  // namespace clm
