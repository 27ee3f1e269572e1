/*
 * celllistmap_gb300.h — C ABI of libcelllist_cuda.so, the GB300 (sm_103a)
 * cutoff-pair engine: cell-list construction and the cell-pair map with a
 * registry of built-in pair operators.
 *
 * Every function returns an int32 status (CLM_OK = 0).  A handle owns all the
 * device buffers it uses; host pointers passed in are read during the call and
 * not retained.  One handle = one CUDA stream = one host thread at a time;
 * different handles are independent.
 *
 * The entry points replace these calls of CellListMap.jl (paths are relative to
 * the CellListMap.jl source tree):
 *   Box(unitcell, cutoff; lcell)          src/internals/Box.jl:191-203, 330-335, 374-377
 *   CellList / UpdateCellList!            src/internals/CellLists.jl:511-521, 590-605, 644-927, 1094-1204
 *   _pairwise!(f, output, box, cl)        src/internals/self.jl:28-45, src/internals/cross.jl:8-25
 *   pairwise!(f, sys)                     src/API/pairwise.jl:48-63
 *   neighborlist / neighborlist!          src/API/neighborlist.jl:217-231, 314-340
 * with `f` restricted to the built-in operators enumerated by clm_op_id.
 */
#ifndef CELLLISTMAP_GB300_H
#define CELLLISTMAP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct clm_handle_s* clm_handle;

/* Status codes.  The Julia/Python front ends map them back to the reference's
 * exception types (ArgumentError, DimensionMismatch). */
enum clm_status {
  CLM_OK = 0,
  CLM_ERR_ARG = 1,             /* invalid argument (ArgumentError) */
  CLM_ERR_CELL_TOO_SMALL = 2,  /* unit cell check failed, src/internals/Box.jl:243,597-607 */
  CLM_ERR_NAN = 3,             /* NaN coordinates, src/internals/CellOperations.jl:6-21 */
  CLM_ERR_DIM = 4,             /* dimension mismatch, src/internals/CellLists.jl:740-751 */
  CLM_ERR_CUDA = 5,            /* a CUDA runtime call failed */
  CLM_ERR_CAPACITY = 6,        /* output buffer too small; the required size is reported */
  CLM_ERR_STATE = 7,           /* call out of order (e.g. run before build) */
  CLM_ERR_TIMEOUT = 8,         /* a bounded device-side wait gave up */
  CLM_ERR_NOMEM = 9,           /* device allocation failed */
  CLM_ERR_LCELL = 10,          /* lcell < 1, src/internals/Box.jl:192 */
  CLM_ERR_NONPERIODIC_CELL = 11, /* unit-cell update on a non-periodic system, src/API/updating.jl:30-45 */
  CLM_ERR_INTERNAL = 12        /* a device-side consistency check failed */
};

enum clm_dtype { CLM_F32 = 0, CLM_F64 = 1 };

/* Box kinds: OrthorhombicCell, TriclinicCell, NonPeriodicCell (src/internals/Box.jl:5-9) */
enum clm_cell_kind { CLM_ORTHO = 0, CLM_TRICLINIC = 1, CLM_NONPERIODIC = 2 };

/* Built-in pair operators.  Each reproduces one closure pattern of the
 * reference (file:line of the pattern in the comments). */
enum clm_op_id {
  CLM_OP_NL = 1,             /* push_pair!: (i, j, d), src/internals/neighborlist.jl:67-76 */
  CLM_OP_COUNT = 2,          /* number of pairs, test/modules/Testing.jl:135-141 */
  CLM_OP_SUM_D2 = 3,         /* output += d2, src/API/ParticleSystem.jl:110-118 */
  CLM_OP_SUM_D = 4,          /* output += d, test/modules/Testing.jl:22 */
  CLM_OP_SUM_INV_D = 5,      /* output += 1/d */
  CLM_OP_SOFT_ENERGY = 6,    /* u += (c - d)^2, test/examples/packmol.jl:49-55 */
  CLM_OP_SOFT_FORCES = 7,    /* energy and forces of (c - d)^2 */
  CLM_OP_LJ_ENERGY = 8,      /* u += eps*(c12 (s/d)^12 - c6 (s/d)^6), test/applications/namd/ParticleSystem_vs_NAMD.jl:15-18 */
  CLM_OP_LJ_FORCES = 9,      /* energy and forces of the same, per-type eps/sigma tables optional */
  CLM_OP_MINDIST = 10,       /* argmin d, test/examples/nearest_neighbor.jl:9-16,43 */
  CLM_OP_RHIST = 11,         /* radial histogram with per-bin velocity accumulator, test/examples/pairwise_velocities.jl:17-24 */
  CLM_OP_INV_D_FORCES = 12,  /* energy 1/d with gradient accumulation, docs/src/ParticleSystem/single_set_compound.md:79-86 */
  CLM_OP_LJ_ADJOINT = 13,    /* LJ energy, forces and the adjoint of the energy w.r.t. the cell and the per-type
                                eps/sigma (no reference counterpart: the reference differentiates closures with
                                ForwardDiff, test/examples/generic_types.jl:10-20,102) */
  CLM_OP_WEIGHTED_INV_D = 14 /* u -= c w_i w_j / d and forces df = (c w_i w_j / d^2 / d)(x_i - x_j), f_i -= df,
                                f_j += df: the gravitational potential and force examples with w = mass,
                                c = 9.8 (test/examples/gravitational_potential.jl:30-33,
                                test/examples/gravitational_force.jl:37-46); Coulomb sums with w = charge */
};

/* Precision forms of the map (see clm_set_precision). */
enum clm_precision {
  CLM_PREC_EXACT = 0,  /* input dtype end to end; results bit-exact with the reference's arithmetic */
  CLM_PREC_SPLIT = 1   /* FP32 pair arithmetic on cell-relative offsets, FP64 re-test of pairs near the cutoff */
};

/* Operator parameters (clm_run's op_params).  Unused fields are ignored. */
typedef struct {
  double p[8];               /* SOFT: p[0] = c (0 => cutoff).  LJ: p[0] = eps, p[1] = sigma, p[2] = c12, p[3] = c6.
                                WEIGHTED_INV_D: p[0] = c */
  int32_t ntypes;            /* LJ: number of particle types (0 => single eps/sigma) */
  int32_t nbins;             /* RHIST: number of bins */
  const int32_t* types_x;    /* LJ: type of each x particle (host or device, see params_on_device) */
  const int32_t* types_y;    /* LJ cross: type of each y particle */
  const double* eps_table;   /* LJ: ntypes x ntypes row-major */
  const double* sig_table;   /* LJ: ntypes x ntypes row-major */
  const double* vel_x;       /* RHIST: velocities of x, n x dim, in the handle's dtype */
  const double* vel_y;       /* RHIST cross: velocities of y */
  const double* bins;        /* RHIST: nbins+1 ascending edges */
  int32_t params_on_device;  /* 1 if the pointers above are device pointers */
  int32_t reserved;
  const double* weights_x;   /* WEIGHTED_INV_D: weight of each x particle (p[0] = c) */
  const double* weights_y;   /* WEIGHTED_INV_D cross: weight of each y particle */
} clm_op_params;

/* Outputs of clm_run.  Pointers may be host or device (out_on_device).  Only
 * the fields the operator produces are written. */
typedef struct {
  double scalar;             /* energies / sums (host, always written when produced) */
  int64_t count;             /* pair count (COUNT, NL) */
  int64_t min_i, min_j;      /* MINDIST: pair with the smallest distance (index_base applied) */
  double min_d;
  void* forces_x;            /* n_x x dim in the handle's dtype */
  void* forces_y;            /* n_y x dim (cross) */
  int64_t* hist_count;       /* nbins */
  double* hist_sum;          /* nbins */
  int32_t out_on_device;
  int32_t index_base;        /* 0 or 1 for MINDIST indices */
  double* adjoint;           /* LJ_ADJOINT (host): virial W = sum g dx dx^T (3x3 row-major, original frame;
                                dU/dM = W M^-T for the cell matrix M with scaled coordinates fixed), then
                                dU/deps and dU/dsigma per type pair (a <= b, row-major upper triangle; one
                                entry without types).  Length 9 + 2 * ntypes (ntypes + 1) / 2 (or 11). */
} clm_outputs;

/* Handle lifecycle.  nsets = 1 (self pairs) or 2 (x-y cross pairs).
 * Replaces ParticleSystem(...) state: src/API/ParticleSystem.jl:142-202. */
int32_t clm_create(int32_t dtype, int32_t dim, int32_t nsets, clm_handle* h);
int32_t clm_destroy(clm_handle h);

/* Bind the handle to a CUDA stream (cudaStream_t passed as void*; NULL = the
 * handle's own stream). */
int32_t clm_set_stream(clm_handle h, void* stream);

/* Box(unitcell, cutoff; lcell) — src/internals/Box.jl:191-270, update_box 395-423.
 * M: column-major dim x dim unit cell (columns are lattice vectors); for
 * CLM_ORTHO only the diagonal is used; ignored for CLM_NONPERIODIC (the box is
 * derived from the positions at each build, src/internals/ParticleSystem.jl:158-164). */
int32_t clm_set_box(clm_handle h, const double* M, int32_t cell_kind, double cutoff, int32_t lcell);

/* Positions of set `set` (0 = x, 1 = y): n points, dim x n column-major (the
 * memory layout of a Julia Vector{SVector} / Matrix(dim, n)), in the handle's
 * dtype.  is_device = 1 if xyz is a device pointer.  Marks the set dirty
 * (ParticleSystemPositions.updated, src/API/ParticleSystemPositions.jl:14-22). */
int32_t clm_set_positions(clm_handle h, int32_t set, const void* xyz, int64_t n, int32_t is_device);

/* UpdateCellList! for every dirty set — src/internals/CellLists.jl:727-927,
 * 1180-1204; non-periodic: src/internals/NonPeriodicCells.jl:93-251. */
int32_t clm_build(clm_handle h);

/* Select the precision form of clm_run (CLM_PREC_EXACT or CLM_PREC_SPLIT).  In the split form pair sets,
 * counts and histogram bins stay those of the exact form; a Float64 radial histogram whose positive bin edges
 * come closer to 0 than the split form's FP32 distance error window (about sqrt(dim) (3 lcell + 5) cell side
 * 2^-12) runs in the exact form. */
int32_t clm_set_precision(clm_handle h, int32_t precision);

/* _pairwise!(op, output, box, cl) — src/internals/self.jl:28-184,
 * src/internals/cross.jl:8-129 — for one built-in operator.  Builds first if a
 * set is dirty (UpdateParticleSystem!, src/internals/ParticleSystem.jl:129-224). */
int32_t clm_run(clm_handle h, int32_t op_id, const clm_op_params* params, clm_outputs* out);

/* Neighbour list of the last CLM_OP_NL run: the number of pairs, then the
 * pairs (unordered, as in src/API/neighborlist.jl:229-230).  d has the
 * handle's dtype.  index_base 1 gives Julia indices. */
int32_t clm_nl_count(clm_handle h, int64_t* n);
int32_t clm_nl_fetch(clm_handle h, int64_t* i, int64_t* j, void* d, int64_t cap, int32_t index_base,
                     int32_t out_on_device);

/* Box fields as computed by the library (for Box mirrors and parity checks):
 * nc[dim], cell_size[dim], computing box min/max[dim], aligned unit cell,
 * rotation and inverse rotation (column-major dim x dim), cutoff. */
int32_t clm_get_box(clm_handle h, int64_t* nc, double* cell_size, double* cbmin, double* cbmax, double* aligned,
                    double* rotation, double* inv_rotation, double* cutoff);

/* CellList summary of set `set` after a build: real particles, particles in the
 * computing box including images, cells with particles, cells with real
 * particles (src/internals/CellLists.jl:115-137). */
int32_t clm_get_celllist_info(clm_handle h, int32_t set, int64_t* n_real, int64_t* n_particles,
                              int64_t* n_cells_with_particles, int64_t* n_cells_with_real);

/* The built cell list of set `set`, copies in cell order: linear cell index
 * (0-based, x fastest), particle index (index_base applied), real flag and
 * coordinates (n_particles x dim, handle dtype).  Host buffers. */
int32_t clm_fetch_celllist(clm_handle h, int32_t set, int64_t cap, int64_t* cell, int64_t* index, int8_t* real,
                           void* coords, int32_t index_base);

/* Timing of the last build and run (device milliseconds, CUDA events). */
int32_t clm_last_timings(clm_handle h, float* build_ms, float* map_ms);

/* Allocation-free pair reductions, for callers that cannot call cudaMalloc where they evaluate
 * (under an application-owned device pool, in a real-time loop that must not enter the CUDA
 * allocator).  No counterpart in the reference.  Supports CLM_OP_COUNT, CLM_OP_SUM_D2, CLM_OP_SUM_D,
 * CLM_OP_SUM_INV_D, CLM_OP_SOFT_ENERGY, CLM_OP_LJ_ENERGY (no type tables) and CLM_OP_MINDIST on a
 * handle whose cell lists are already built (clm_build; returns CLM_ERR_STATE otherwise, since
 * building allocates).  Per-block partials live in a static 128 KiB + 256 B device array (4096 block
 * slots, held by every GPU that loads the library until exit); a launch needing more slots returns
 * CLM_ERR_CAPACITY.  The first call on a device looks up the array's device address, so make it
 * before any stream capture.  Calls share the array: calls that overlap on the GPU race.  Call with
 * the handle's device current.  The call waits for its result (stream synchronization, host read). */
int32_t clm_run_noalloc(clm_handle h, int32_t op_id, const clm_op_params* params, clm_outputs* out);

/* LJ energy, forces and adjoint in one call: clm_run(h, CLM_OP_LJ_ADJOINT, params, out).  The
 * reference has no such entry point (it differentiates its map with ForwardDiff dual numbers,
 * test/examples/generic_types.jl:10-20,102); out->forces_x and out->adjoint are required. */
int32_t clm_lj_adjoint(clm_handle h, const clm_op_params* params, clm_outputs* out);

/* ---------------------------------------------------------------- batches of independent systems
 * Many periodic systems of uneven size in one handle: one cell list over a global cell index, one
 * launch per kernel for all systems, and optionally the whole step (build + operators) replayed
 * as a CUDA graph.  The reference handles one system per ParticleSystem (src/API/ParticleSystem.jl:
 * 142-202); a batch is the loop `for sys in systems; pairwise!(f, sys); end` in one call.
 * Positions: clm_set_positions(h, 0, xyz, n_total, is_device) with the systems concatenated. */
typedef struct {
  double* scalar;         /* nsys: the operator's sum per system (COUNT: the count); NaN for a failed system */
  int64_t* count;         /* nsys: pairs per system (COUNT, NL) */
  void* forces;           /* n_total x dim, handle dtype (force operators) */
  int32_t out_on_device;  /* 1 if scalar/count/forces are device pointers */
  int32_t reserved;
} clm_batch_outputs;

/* A handle for batches (set 0 only).  clm_set_box/clm_build/clm_run refuse it (CLM_ERR_STATE). */
int32_t clm_batched_create(int32_t dtype, int32_t dim, clm_handle* h);

/* nsys systems; offsets[nsys+1] delimit each system's particles in the concatenated positions;
 * cells: nsys unit cells, dim x dim column-major each (CLM_TRICLINIC), or dim sides each
 * (CLM_ORTHO); one cutoff and lcell for all.  A system whose cell fails the reference's check
 * (Box.jl:243, plane distance > 2 cutoff) gets status CLM_ERR_CELL_TOO_SMALL and is skipped. */
int32_t clm_batched_set_systems(clm_handle h, int64_t nsys, const int64_t* offsets, const double* cells,
                                int32_t cell_kind, double cutoff, int32_t lcell);

/* One step: build the cell lists of all systems, then run `nops` operators (NL, COUNT, SUM_*,
 * SOFT_ENERGY, LJ_ENERGY, SOFT_FORCES, LJ_FORCES, INV_D_FORCES; no type tables), outs[k] receiving
 * the results of ops[k].  The neighbour list (at most one NL op per step) is read with clm_nl_count /
 * clm_nl_fetch (global particle indices).  With the graph on, the first call runs the step directly
 * and records it; later calls with the same operators, parameters and sizes replay the recording. */
int32_t clm_batched_run(clm_handle h, int32_t nops, const int32_t* ops, const clm_op_params* params,
                        clm_batch_outputs* outs);

/* Per-system status of the last step (CLM_OK, CLM_ERR_CELL_TOO_SMALL, CLM_ERR_NAN). */
int32_t clm_batched_status(clm_handle h, int32_t* status, int64_t nsys);

/* Replay steps as a CUDA graph (1) or launch them one by one (0, the default). */
int32_t clm_batched_set_graph(clm_handle h, int32_t enable);

/* Cell-tile and block shape: lcell (cells per cutoff), parts per cell, resident blocks per SM
 * divided by grid_div.  Any value <= 0 keeps the current one. */
int32_t clm_batched_set_config(clm_handle h, int32_t lcell, int32_t cell_split, int32_t grid_div);

/* Autotuner: times every candidate (lcell 1..3, parts per cell 1..2, grid_div 1..2) on `reps`
 * steps of the given operators with the current positions, keeps the fastest, and returns it in
 * config[3] (lcell, cell_split, grid_div) with its median step time in best_ms. */
int32_t clm_batched_autotune(clm_handle h, int32_t nops, const int32_t* ops, const clm_op_params* params,
                             int32_t reps, int32_t* config, float* best_ms);

/* Device time of the last step (build + operators, CUDA events) and kernels it launched. */
int32_t clm_batched_last_step(clm_handle h, float* step_ms, int64_t* launches);

/* Number of CUDA kernels this handle has launched so far (cumulative). */
int32_t clm_stats(clm_handle h, int64_t* kernel_launches);

/* Device (and pinned host) allocations made by the library in this process so far: count and bytes.
 * Buffers grow only, so repeated steps with unchanged sizes allocate nothing — the GPU counterpart of
 * the reference's allocation tests for update!/neighborlist! (test/API/neighborlists.jl:114-177). */
int32_t clm_device_allocations(int64_t* count, int64_t* bytes);

/* Human-readable description of the last error on this handle. */
int32_t clm_last_error(clm_handle h, char* buf, size_t n);

/* Library version string. */
const char* clm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CELLLISTMAP_GB300_H */
