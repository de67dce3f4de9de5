// pbf_internal.cuh — constants, device math and launch wrappers shared by the
// translation units of libpbf.  Internal: the public boundary is include/pbf.h.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include "../../include/pbf.h"

namespace pbf {

// A named NVTX range over one C-ABI call, for profilers: the kernels a call
// launches (graph launches included) fall inside it, so `ncu --nvtx
// --nvtx-include "pbf_step/"` captures the steps alone.  NVTX is header-only;
// with no tool attached a push or pop is a no-op.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// fluids/helper.h:4 — the reference's truncated pi, used by its host-side
// kernel coefficients (getPoly6 / getSpikyGrad constructors).
constexpr double kRefPi = 3.14159265359;

// The box of one scene and where its cells sit in the global cell numbering.
struct SceneGeom {
  float llim[3], ulim[3];
  float lo[3], hi[3];      // wall clamp bounds: llim + lim_eps, ulim - lim_eps (rounded once from double)
  int dims[3];             // cells per axis
  int cell_base;           // global id of the scene's cell 0
};

// Everything a pass needs, computed once per step on the host and passed by
// value.  Coefficients follow the reference's host-side set-up bit for bit
// (fluids/Simulator.cu:77-98, :129, :187-188, :235).
struct StepConsts {
  float h, h2;
  float poly6_coef;        // 315 / (64 pi h^9), getPoly6 ctor
  float spiky_coef;        // -45 / (pi h^6), getSpikyGrad ctor
  float spiky_coef_rho0;   // spiky_coef / pho0 (lambda pass gradients are grad W / pho0)
  float pho0, inv_pho0;
  float lambda_eps;
  float coef_corr;         // -k_corr / W(delta_q)^n_corr
  float n_corr;
  int npow;                // n_corr as a small positive integer, or -1
  float keps2;             // kernel_eps^2: spiky gradient is zero for |r| < kernel_eps
  float max_dp;
  float vort_eps;          // vorticity confinement strength (0: off)
  float k_b;               // k_boundaryDensity
  float c_xsph;
  float dt, inv_dt;
  float g[3];              // gravity vector = -g * up
  int cells;               // cells of all scenes
  int dense_grid;          // blocks of the dense neighbour kernels (a multiple of the SM count)
  int dense_window;        // candidates above which a warp takes the dense kernel
  int dense_all;           // 1: every warp takes the dense kernel; 0: never; -1: by particle count
  int order;               // 1: the passes take particles in current-cell order (bucketed); 0: grid order
  int stage_sparse;        // slots a sparse-kernel block may stage in shared memory (0: none)
  int stage_dense;         // slots a dense-kernel block may stage in shared memory (0: none)
  int queue_sparse;        // hit-queue chunks per thread of the sparse / dense kernel (1: none)
  int queue_dense;
  int dense_split;         // warps of the dense kernel sharing one item's windows: 1, 2, 4 or 8
  int dense_interleave;    // 1: those warps take every dense_split-th chunk; 0: contiguous parts
  SceneGeom geom;          // the box of a single-scene step
};

// Where a particle's box comes from: the single scene in StepConsts, or a
// table of scenes indexed by a per-particle scene id.  Scenes occupy
// contiguous particle ranges, before and after the cell sort alike, so one
// id array serves both orders.
struct Geometry {
  const SceneGeom* scenes;  // nullptr: single scene
  const uint16_t* sid;      // [n] scene of each particle slot
};

__device__ __forceinline__ SceneGeom geom_of(const StepConsts& c, const Geometry& G, int i) {
  return G.scenes ? G.scenes[G.sid[i]] : c.geom;
}

// Cell coordinate along one axis: getGridxyz / getGridId (fluids/Simulator.cu:30-36,
// :65-71): IEEE (p - llim) / h, truncating conversion (saturating, NaN -> 0),
// clamped into [0, dim - 1].
__device__ __forceinline__ int cell_coord(float p, float llim, float h, int dim) {
  int v = __float2int_rz(__fdiv_rn(__fsub_rn(p, llim), h));
  return min(max(v, 0), dim - 1);
}

__device__ __forceinline__ int3 cell_of(const StepConsts& c, const SceneGeom& g, float4 p) {
  return make_int3(cell_coord(p.x, g.llim[0], c.h, g.dims[0]),
                   cell_coord(p.y, g.llim[1], c.h, g.dims[1]),
                   cell_coord(p.z, g.llim[2], c.h, g.dims[2]));
}

// xyzToId (fluids/Simulator.cu:44-53): x-major, z fastest; offset to the scene's cells.
__device__ __forceinline__ int cell_index(const SceneGeom& g, int x, int y, int z) {
  return g.cell_base + (x * g.dims[1] + y) * g.dims[2] + z;
}

// |a - b|^2 with the fused multiply-adds nvcc forms for the reference's
// d.x*d.x + d.y*d.y + d.z*d.z.
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
  return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

// W(r^2) for r^2 < h^2 (getPoly6::operator(), fluids/Simulator.cu:84-89).
__device__ __forceinline__ float poly6_inside(const StepConsts& c, float r2) {
  float d = c.h2 - r2;
  return c.poly6_coef * d * d * d;
}

// w^n for the s_corr term (the reference calls powf, fluids/Simulator_kernel.cuh:165).
__device__ __forceinline__ float pow_corr(const StepConsts& c, float w) {
  switch (c.npow) {
    case 1: return w;
    case 2: return w * w;
    case 3: return w * w * w;
    case 4: { float w2 = w * w; return w2 * w2; }
    default: return powf(w, c.n_corr);
  }
}

// DensityBoundary (fluids/Simulator.cu:139-161), evaluated only when
// k_boundaryDensity != 0.
__device__ __forceinline__ float density_at(float d, float h) {
  const float k = (float)(2.0 * kRefPi / 3.0);
  if (d > h) return 0.f;
  if (d <= 0.f) return k;
  return k * (h - d) * (h - d) * (h + d);
}

__device__ __forceinline__ float boundary_density(const StepConsts& c, const SceneGeom& g, float4 p) {
  return density_at(g.ulim[0] - p.x, c.h) + density_at(p.x - g.llim[0], c.h) +
         density_at(g.ulim[1] - p.y, c.h) + density_at(p.y - g.llim[1], c.h) +
         density_at(g.ulim[2] - p.z, c.h) + density_at(p.z - g.llim[2], c.h);
}

// ---- launch wrappers (grid.cu) ------------------------------------------------

// Scratch of the neighbour grid build, all device pointers owned by the solver.
struct GridScratch {
  uint32_t* keys_a;     // [max_particles]
  uint32_t* keys_b;     // [max_particles]
  uint32_t* vals_a;     // [max_particles]
  uint32_t* vals_b;     // [max_particles]
  uint32_t* cell_count; // [max_cells + 1]
  uint32_t* cell_start; // [max_cells + 1]  exclusive prefix of cell counts
  uint32_t* radix_counts;   // [256 * max_sort_tiles]
  uint32_t* scan_partials;  // [kMaxScanPartials]
  const uint32_t* keys_sorted;  // set by build_grid: cell id of each sorted slot (inside keys_a/b)
};

constexpr int kScanTile = 2048;
constexpr int kMaxScanPartials = 8192;
constexpr int kSortTile = 2048;

int sort_tiles(int n);
size_t radix_counts_len(int max_particles);

// Hash (optionally predicting x* = x + dt (v + dt g) first), count cells,
// stable radix sort by cell id, exclusive prefix of counts.
//   pos/vel != null: predict from them;  xstar != null: hash xstar directly.
// On return (stream order): *perm_out points at the sorted-slot -> input index
// array (inside scratch), scratch.cell_start holds cells + 1 prefix entries.
// keys_copy (optional, n entries) receives the unsorted cell ids.
cudaError_t build_grid(const StepConsts& c, const Geometry& G, const float4* pos, const float4* vel,
                       const float4* xstar, int n, GridScratch& s, const uint32_t** perm_out,
                       uint32_t* keys_copy, cudaStream_t stream);

// start/end per cell in the reference's format (0/0 for empty cells).
cudaError_t export_ranges(const StepConsts& c, const uint32_t* cell_start, uint32_t* start,
                          uint32_t* end, cudaStream_t stream);

// ---- launch wrappers (solver.cu) ----------------------------------------------

struct SolverScratch {
  float4* xs;          // sorted x (positions at t)
  float4* xa;          // predicted / iterated positions, ping
  float4* xb;          // pong
  uint32_t* iid_s;     // sorted iid
  float* lambda;
  float* rho;
  uint32_t* flags;     // [kNumFlags] per-step flags and dense-list counters, zeroed by reorder
  uint32_t* dense;     // [dense_list_len(max_particles)] work slots handed to the dense kernels
  uint32_t* masks;     // [kMaskWords][mask_stride] the lambda pass's neighbour masks
  int mask_stride;     // >= particles
  uint32_t* cell_flags;         // [max_cells + 1] CellFlag bits per cell, zeroed by reorder
  const uint32_t* keys_sorted;  // the grid's sorted cell ids (set before the passes)
  const uint32_t* cell_start;   // the grid's cell prefix (set before the passes)
  // group tables of the cells holding >= kGroupCell particles (one slot each);
  // slot s of population p owns entries [grp_off[s], grp_off[s] + p) of the
  // pools of max_particles entries and [2 grp_off[s], 2 grp_off[s] + 2 p) of
  // each hash table part
  int grp_pool;        // pool entries (max_particles)
  int* grp_cell;       // [group_slots] cell of each slot
  int* grp_off;        // [group_slots] first pool entry of each slot
  int* grp_n;          // [group_slots] groups in the slot's current table; -1: not grouped
  int* grp_rep;        // [max_particles] pool: sorted slot of each group's first particle
  int* grp_cnt;        // [max_particles] pool: particles of each group
  float4* grp_pos;     // [max_particles] pool: the group's position
  float4* grp_sum;     // [max_particles] pool: pass sums of the group (see solver.cu)
  float4* grp_aux;     // [max_particles] pool: velocity of the group's first particle (xsph)
  int* grp_id;         // [max_particles] hash entry of each particle of a grouped cell
  int* grp_hash;       // [4][2 max_particles] hash tables: owner, count, first particle, rank
                       // (owner, count and first are 0 between passes)
  unsigned* grp_max;   // [max_particles] pool: largest deviation of a group (0 between passes)
  unsigned long long* grp_acc;  // [3 max_particles] pool: fixed-point sums (0 between passes)
  int* grp_list;       // [max_particles] pool: hash entries a slot's pass claimed
  int* grp_list_n;     // [group_slots] entries claimed (0 between passes)
  int* grp_done;       // [group_slots] work items finished (0 between passes)
  int* grp_zero;       // [group_slots] every deviation of the pass's sums is zero
  int* grp_item_off;   // [group_slots] first work item of each slot
  int* grp_item_slot;  // [group_items] slot of each work item
  // work lists of the lambda and delta_p passes (see solver.cu): the
  // particles that compute, and for each follower its group's first particle
  int* work_list;      // [max_particles]
  int* work_follow;    // [max_particles] -1, or the sorted slot whose results particle i takes
  int* work_blocks;    // [work_blocks_len(max_particles)] per-block counts, then offsets
  // current-cell order (StepConsts::order): the computing particles of a pass
  // bucketed by the cell they are in now
  uint32_t* bcnt;      // [max_cells + 1] particles per current cell
  uint32_t* bstart;    // [max_cells + 1] exclusive prefix of bcnt
  uint2* bent;         // [max_particles] (current cell, rank in it) of each computing particle
  int* bucket;         // [max_particles] the computing particles, bucket by bucket
  uint32_t* bpart;     // [kMaxScanPartials] scan partials
};

// Lambda and delta_p results are the same for every particle of a position
// group (same position: same window, same candidates in the same order; a
// co-located particle adds W(0) to rho and, at r < kernel_eps, no gradient,
// exactly as the particle itself does), so those passes run once per group,
// on its first particle, and copy the results to the others (the followers).
// The computing particles are listed in cell order per iteration.
constexpr int kWorkThreads = 1024;
constexpr size_t work_blocks_len(int max_particles) { return (size_t)max_particles / kWorkThreads + 2; }

// Bits of SolverScratch::cell_flags: the stale cell of a particle whose
// value can poison a neighbour's sum the way the reference's IEEE arithmetic
// does.  A particle takes the per-candidate exact path only when its own
// values or a flagged cell of its window call for it.
enum CellFlag : uint32_t {
  kCellLambdaNonFinite = 1u,
  kCellRhoNotPositive = 2u,  // rho <= 0 or NaN
  kCellVelNonFinite = 4u,
};
// Bits kCellSlotShift.. of cell_flags hold 1 + the group slot of a cell that
// holds >= kGroupCell particles (0: none), set once per step by reorder.
constexpr int kCellSlotShift = 8;

// Group tables.  Particles piled into one cell often sit at bitwise-identical
// positions (clamped into a box corner, or collapsed onto one point by the
// tensile term).  For every cell holding at least kGroupCell particles, each
// pass first groups its particles by the values that enter a pair term
// non-linearly (position; position and density for XSPH; delta_p reuses the
// lambda pass's groups) in a hash table with room for every particle, orders
// the groups by their first particle, and a window containing the cell
// visits each group once with its multiplicity instead of its particles.
// The pair terms are linear in lambda_j (delta_p) and v_j (XSPH): a group
// carries the sum of its members' values, accumulated exactly in fixed point
// (integer atomics, so the sum does not depend on the order).  This is the
// reference's sum with its terms grouped: results differ from it by
// rounding only.
constexpr int kGroupCell = 512;
// PBF_GROUP_CHUNK (a build-time tuning macro): particles of a grouped cell per
// work item of the group-table kernels.
#ifndef PBF_GROUP_CHUNK
#define PBF_GROUP_CHUNK 8192
#endif
constexpr int kGroupChunk = PBF_GROUP_CHUNK;
inline size_t group_slots(int max_particles) { return (size_t)max_particles / kGroupCell + 1; }
inline size_t group_items(int max_particles) {
  return (size_t)max_particles / kGroupChunk + group_slots(max_particles) + 1;
}

// Neighbour masks a particle keeps between the lambda and delta_p passes of
// one iteration: one 32-bit mask per chunk of 32 consecutive candidates.
constexpr int kMaskWords = 16;

// Words of SolverScratch::flags.  The two step flags are raised by a pass
// when a later pass must take its exact (slow) path to reproduce the
// reference's IEEE results (almost always zero).  The two counters are the
// lengths of the dense lists, used alternately by consecutive passes.
enum StepFlag {
  kFlagLambdaNonFinite = 0,  // some lambda_i is NaN/inf: delta_p must see it through zero gradients
  kFlagXsphExact = 1,        // some rho_i <= 0 or non-finite, or some velocity non-finite
  kDenseCount0 = 2,
  kDenseCount1 = 3,
  kGroupCount = 4,           // cells with a group slot (set by reorder)
  kGroupPool = 5,            // group pool entries handed out (set by reorder)
  kGroupItems = 6,           // group work items (set by reorder)
  kWorkCount = 7,            // particles on the current iteration's work list
  kWorkDone = 8,             // blocks of the work-list count finished (0 between uses)
  kWorkIdentity = 9,         // 1: no grouped cell this step, the passes take every particle in order
  kBucketCount = 10,         // particles in the current buckets
  kItemCount0 = 11,          // dense-kernel batches handed out, by pass parity (work queue)
  kItemCount1 = 12,
  kNumFlags = 13
};

// One more word after the step flags, cleared only when the host reads it:
// device-side errors (ErrorBit) recorded by any step since.
constexpr int kErrorWord = kNumFlags;
constexpr int kFlagWords = kNumFlags + 1;
enum ErrorBit : uint32_t {
  kErrStageTimeout = 1u,     // a shared-memory staging copy did not complete in time
};

// Largest stage (slots, 16 bytes each) a neighbour-pass block may ask for;
// the staged pass kernels allow that much dynamic shared memory beside their
// hit queue (set_pass_kernel_attributes).
constexpr int kStageMax = 4096;
cudaError_t set_pass_kernel_attributes();

// Entries of the dense list: one per particle.
constexpr size_t dense_list_len(int max_particles) { return (size_t)max_particles + 1; }

// Gather pos/vel/iid into cell order and recompute x* (bit-identical to the hash).
cudaError_t reorder(const StepConsts& c, const uint32_t* perm, const float4* pos, const float4* vel,
                    const uint32_t* iid, int n, SolverScratch& s, cudaStream_t stream);

// Each neighbour pass is two launches: the sparse kernel over all particles,
// then the dense kernel over the warps the sparse kernel handed on.  `pass`
// numbers the passes of a step (0, 1, 2, ...) and picks the dense counter.

// lambda_i and rho_i of every particle at positions X.
cudaError_t launch_lambda(const StepConsts& c, const Geometry& G, const float4* X, const uint32_t* cs, int n,
                          const SolverScratch& s, int pass, cudaStream_t stream);
// One Jacobi position update X -> T.
cudaError_t launch_delta_p(const StepConsts& c, const Geometry& G, const float4* X, const uint32_t* cs, int n,
                           const SolverScratch& s, int pass, float4* T, cudaStream_t stream);
// Last position update: x_final -> npos, (x_final - x) / dt -> vel, and the
// permuted inputs -> pos, iid.
cudaError_t launch_delta_p_final(const StepConsts& c, const Geometry& G, const float4* X, const uint32_t* cs, int n,
                                 const SolverScratch& s, int pass, float4* pos, float4* npos,
                                 float4* vel, uint32_t* iid, cudaStream_t stream);
// XSPH: nvel = vel + c sum_j 2 (v_j - v_i) W / (rho_i + rho_j).
cudaError_t launch_xsph(const StepConsts& c, const Geometry& G, const float4* X, const float4* V, const uint32_t* cs,
                        int n, const SolverScratch& s, int pass, float4* NV, cudaStream_t stream);

// Candidates above which a warp takes the dense kernel, and the particle
// count below which every warp does (defaults; pbf_autotune can override).
constexpr int kDefaultDenseWindow = 512;
// Blocks of the dense kernel per SM (its grid is this many times the SM count).
#ifndef PBF_DENSE_BLOCKS_PER_SM
#define PBF_DENSE_BLOCKS_PER_SM 4
#endif
constexpr int kDenseBlocksPerSm = PBF_DENSE_BLOCKS_PER_SM;
constexpr int kDenseAllBelow = 131072;
// Slots a block of the sparse / dense pass kernel stages in shared memory
// (defaults; 0: no staging; pbf_autotune can override, up to kStageMax).
constexpr int kDefaultStageSparse = 0;
constexpr int kDefaultStageDense = 0;
// Hit-queue capacities (chunks per thread; 1: the pair body right after each
// chunk) and the dense kernel's warps per item (defaults; pbf_autotune can
// override, queues up to kMaxQueue* chunks).
constexpr int kMaxQueueSparse = 16;
constexpr int kMaxQueueDense = 8;
constexpr int kDefaultQueueSparse = 1;
constexpr int kDefaultQueueDense = 1;
constexpr int kDefaultDenseSplit = 8;
constexpr int kDefaultDenseInterleave = 0;

// Vorticity confinement after XSPH, on its output NV (positions X = npos):
// omega_i = sum_j (u_j - u_i) x g_ij and eta_i = sum_j |omega_j| g_ij over
// the neighbours j != i with kernel_eps <= r < h, g_ij the spiky gradient
// grad W(x_i - x_j); then u_i += dt eps (eta_i / |eta_i|) x omega_i (Macklin
// and Mueller 2013, eqs. 15-16).  Scratch: s.xb holds omega (free after the
// last position update).
cudaError_t launch_vorticity(const StepConsts& c, const Geometry& G, const float4* X, const uint32_t* cs, int n,
                             const SolverScratch& s, float4* NV, cudaStream_t stream);
constexpr int kVorticityLaunches = 2;

// Kernel launches of one neighbour pass of n particles (sparse kernel unless
// every warp goes dense, dense kernel).
int pass_launches(const StepConsts& c, int n);
// Group-table, work-list and follower launches of one step of n particles at
// niter iterations.
int group_launches(const StepConsts& c, int n, int niter);

// ---- reverse pass (adjoint.cu) ------------------------------------------------------

constexpr int kMaxTapeIters = 64;

// The positions entering every iteration and the final ones of a taped step
// (X[0] = x*, X[niter] = npos), and every iteration's lambda.
struct BackwardTape {
  int niter;
  float4* X[kMaxTapeIters + 1];
  float* lambda[kMaxTapeIters];
};

struct BackwardArgs {
  StepConsts c;
  Geometry G;
  const uint32_t* cs;
  int n;
  const float4* xs;      // sorted input positions
  const float* rho;      // rho of the last lambda pass
  const float4* XK;      // final positions (set by backward)
  const float4* g_npos;  // adjoints of the outputs (set by backward)
  const float4* g_nvel;
  float4* gx;       // adjoint of the current positions
  float4* gx_next;  // adjoint being built for the earlier positions
  float4* gx0;      // velocity-update part of the sorted inputs' adjoint
  float* grho;      // adjoint of the last rho (from XSPH)
  float4* pbar;     // adjoint of the delta_p sums / pho0 ... / pho0
  float* lbar;      // adjoint of lambda
  float4* gs;       // G_i (xyz) and Sbar_i (w)
  float* rtot;      // adjoint of rho_i incl. the constraint's
  float* wall_part; // [blocks][6] per-block wall adjoints
  const float4* X0; // predicted positions (the grid's positions; set by backward)
  unsigned long long* gcell;  // packed grid cell of each particle (cell of X0)
  unsigned long long* kcell;  // packed cell of the current positions
  float4* fix;      // scattered adjoints of non-reciprocal pairs: xyz positions, w lambda / rho
  float4* fixv;     // scattered velocity adjoints of non-reciprocal pairs (XSPH)
  // The scattered terms are summed exactly, in any order (adjoint.cu): listed,
  // then added per target as 64-bit fixed point scaled by the target's largest
  // term; fix / fixv above take only terms beyond the list's capacity.
  int2* sc_key;               // [sc_cap] (target particle, 0: fix / 1: fixv)
  float4* sc_val;             // [sc_cap] the term (fixv: w unused)
  unsigned long long* sc_acc; // [7][sc_stride] fixed-point sums (fix xyzw, fixv xyz); 0 between folds
  unsigned* sc_max;           // [7][sc_stride] largest finite |term| (float bits); 0 between folds
  unsigned* sc_cnt;           // [2][sc_stride] terms per target (fix, fixv); 0 between folds
  unsigned* sc_nonfin;        // [sc_stride] non-finite terms, 3 bits per component; 0 between folds
  unsigned* sc_ctr;           // [2] terms listed, terms beyond the capacity; listed is 0 between folds
  int sc_cap;
  int sc_stride;
  int lanes;        // lanes per particle below kWarpPerParticleBelow particles: 8, 16 or 32
};

// Bytes of the reverse pass's exact-scatter scratch for up to np particles
// (list capacity kScatterPerParticle terms per particle).
constexpr int kScatterPerParticle = 8;
inline size_t scatter_bytes(size_t np) {
  const size_t cap = np * kScatterPerParticle;
  return cap * (sizeof(int2) + sizeof(float4)) + np * (7 * 8 + 7 * 4 + 2 * 4 + 4) + 64;
}

// Poly6 density (mass 1, radius h) of the particles at the nodes of a
// dims[0] x dims[1] x dims[2] lattice of cell centres spanning [lo, hi], and
// its adjoint w.r.t. the positions (both gather-only).
cudaError_t density_grid(const float4* pos, int n, const float lo[3], const float hi[3],
                         const int dims[3], float h, float* grid, cudaStream_t stream);
cudaError_t density_grid_backward(const float4* pos, int n, const float lo[3], const float hi[3],
                                  const int dims[3], float h, const float* g_grid, float4* g_pos,
                                  cudaStream_t stream);

// The reverse pass of the taped step: adjoints of its outputs (npos, nvel,
// cell order) -> adjoints of its inputs (pos, vel, input order) and of the
// limits (g_lim = ulim xyz, llim xyz).  fix and fixv start at zero and are
// left at zero.
cudaError_t backward(const BackwardArgs& args, const BackwardTape& tape, const uint32_t* perm,
                     const void* g_npos, const void* g_nvel, void* g_pos, void* g_vel, float* g_lim,
                     cudaStream_t stream);

// Exclusive prefix of in[0, len) into out (may alias in): 3 launches,
// partials holds kMaxScanPartials entries.
cudaError_t exclusive_scan(const uint32_t* in, uint32_t* out, int len, uint32_t* partials, cudaStream_t stream);

// Launches (and memset nodes) of one bucketing by current cell; an ordered
// step buckets before every lambda pass and before XSPH.
constexpr int kBucketLaunches = 6;
inline int bucket_launches(const StepConsts& c, int niter) { return c.order ? kBucketLaunches * (niter + 1) : 0; }

// Kernel launches of one build_grid call with n particles and c.cells cells.
int grid_launches(const StepConsts& c, int n);

}  // namespace pbf
