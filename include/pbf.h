/*
 * pbf.h — C ABI of the GB300-native Position Based Fluids step.
 *
 * This is the drop-in boundary for the per-frame simulation path of
 * naeioi/PBF-CUDA's `Simulator` class (fluids/Simulator.h:7-61).  Every entry
 * point takes plain pointers and sizes; device pointers are CUDA global-memory
 * addresses, streams are `cudaStream_t` passed as `void*`.  No call allocates
 * on the caller's behalf except pbf_create, which owns all solver scratch.
 *
 * Differences from the reference interface, all deliberate:
 *  - buffers are device pointers to float4 (x, y, z, w) instead of OpenGL
 *    buffer names of float3 (fluids/Simulator.cpp:20-36); pos.w is a
 *    per-particle payload carried with the particle (to npos.w), velocity w
 *    components are written as 0;
 *  - every call returns a pbf_status instead of exit()ing inside
 *    checkCudaErrors (common/cuda_inc/helper_cuda.h:1000-1014);
 *  - pbf_step is asynchronous on the given stream (the reference synchronises
 *    the device between phases, fluids/Simulator.cpp:44-79);
 *  - gravity acts along -up (the reference hard-codes up = +z,
 *    fluids/Simulator.cu:174).
 */
#ifndef PBF_H_
#define PBF_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBF_ABI_VERSION 4

/* Largest max_particles of a solver, and largest total of a batch: 2^27.
 * The solver's per-particle tables are indexed with 32-bit integers, the
 * largest holding 16 words per particle.  At the limit a solver holds about
 * 37 GB of scratch (~272 B per particle) besides the caller's buffers. */
#define PBF_MAX_PARTICLES 134217728

typedef enum pbf_status {
  PBF_OK = 0,
  PBF_ERR_INVALID_ARG = 1, /* null pointer, n < 0, aliasing buffers, bad params */
  PBF_ERR_CAPACITY = 2,    /* n > max_particles, or the box needs more cells than allocated */
  PBF_ERR_CUDA = 3,        /* a CUDA runtime call failed; see pbf_last_error() */
  PBF_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  PBF_ERR_NOT_READY = 5    /* the solver has no step results yet */
} pbf_status;

/*
 * Solver parameters.  Field names and meaning follow the reference's
 * GUIParams solver fields (fluids/GUIParams.h:6-17); the last four fields
 * make the reference's hard-coded gravity axis and compile-time constants
 * (fluids/helper.h:4-9) explicit.
 */
typedef struct pbf_params {
  int niter;                 /* solver iterations per step            GUIParams::niter */
  float pho0;                /* rest density (mass 1 per particle)    GUIParams::pho0 */
  float g;                   /* gravity magnitude                     GUIParams::g */
  float h;                   /* kernel radius = grid cell size        GUIParams::h */
  float dt;                  /* time step of one pbf_step             GUIParams::dt */
  float lambda_eps;          /* constraint relaxation epsilon         GUIParams::lambda_eps */
  float delta_q;             /* s_corr reference distance             GUIParams::delta_q */
  float k_corr;              /* s_corr strength                       GUIParams::k_corr */
  float n_corr;              /* s_corr exponent                       GUIParams::n_corr */
  float k_boundaryDensity;   /* wall density weight                   GUIParams::k_boundaryDensity */
  float c_XSPH;              /* XSPH viscosity                        GUIParams::c_XSPH */
  float up[3];               /* gravity acts along -up; reference: (0,0,1) */
  float lim_eps;             /* wall clamp inset; reference LIM_EPS = 1e-3 */
  float kernel_eps;          /* spiky-gradient cutoff; reference KERNAL_EPS = 1e-4 */
  float max_dp;              /* per-component delta_p clamp; reference MAX_DP = 0.1 */
  float vorticity_eps;       /* vorticity confinement strength; 0 (default): off, as the
                                reference, which has none (README.md:14 lists it as missing) */
} pbf_params;

typedef struct pbf_solver pbf_solver;

/* Reference defaults (fluids/FluidSystem.cpp:15-25, fluids/helper.h:4-9). */
void pbf_params_default(pbf_params* out);

const char* pbf_status_string(pbf_status s);
/* Message of the last failing call on this host thread ("" if none). */
const char* pbf_last_error(void);
int pbf_abi_version(void);

/*
 * Replaces Simulator::Simulator(const GUIParams&, float3 ulim, float3 llim)
 * (fluids/Simulator.h:10-26).  Allocates scratch for up to max_particles
 * particles and for a cell grid of 4x the cells of [llim, ulim] at cell size
 * h (the reference allocates 4 * prod((ulim - llim) / 0.1) cells,
 * fluids/Simulator.h:13-14).  Must be called with the target device current.
 * max_particles in [0, PBF_MAX_PARTICLES], else PBF_ERR_INVALID_ARG (< 0) or
 * PBF_ERR_CAPACITY (above the limit), before any CUDA call.
 */
pbf_status pbf_create(const pbf_params* params, const float ulim[3], const float llim[3],
                      int max_particles, pbf_solver** out);

/* Replaces Simulator::~Simulator (fluids/Simulator.h:27-34). Accepts NULL. */
pbf_status pbf_destroy(pbf_solver* s);

/* Replace Simulator::loadParams / saveParams (fluids/Simulator.cpp:101-130):
 * the reference copies from/to the GUIParams singleton; here the caller owns
 * the struct.  Takes effect at the next pbf_step. */
pbf_status pbf_set_params(pbf_solver* s, const pbf_params* params);
pbf_status pbf_get_params(const pbf_solver* s, pbf_params* out);

/* Replaces Simulator::setLim(ulim, llim) (fluids/Simulator.cpp:132-136).
 * PBF_ERR_CAPACITY if the new box needs more cells than were allocated. */
pbf_status pbf_set_limits(pbf_solver* s, const float ulim[3], const float llim[3]);
pbf_status pbf_get_limits(const pbf_solver* s, float ulim[3], float llim[3]);

/*
 * Replaces Simulator::step(pos, npos, vel, nvel, iid, nparticle)
 * (fluids/Simulator.h:37, fluids/Simulator.cpp:10-99).  One time step dt.
 * Same contract as the reference:
 *   in : pos, vel, iid       state at t (any order)
 *   out: pos, iid            permuted in place into cell order (stable sort by
 *                            cell id of the predicted position)
 *        vel                 (npos - pos) / dt, before XSPH, in cell order
 *        npos, nvel          state at t + dt, in cell order
 * All five buffers hold n entries (float4, except iid), must be distinct and
 * 16-byte aligned.  Asynchronous on `stream` (a cudaStream_t, NULL = legacy
 * default stream).  A handle is not thread-safe: one step in flight per handle.
 */
pbf_status pbf_step(pbf_solver* s, void* pos, void* npos, void* vel, void* nvel,
                    uint32_t* iid, int n, void* stream);

/*
 * Density rho_i of the last step's final lambda pass (fluids/Simulator_kernel.cuh:123-124),
 * in the cell order of that step, copied into the device buffer rho (n floats).
 * Used for the density-constraint error statistics.
 */
pbf_status pbf_get_density(const pbf_solver* s, float* rho, int n, void* stream);

/*
 * The neighbour grid of the reference (fluids/Simulator.cu:178-211) for the
 * given predicted positions xstar (device, n float4), exported in the
 * reference's formats:
 *   keys  [n]      cell id of each particle, input order (getGridId)
 *   perm  [n]      input index of the k-th particle in cell order (stable)
 *   start [cells]  first sorted index of each cell, 0 if empty (computeGridRange)
 *   end   [cells]  one past the last sorted index, 0 if empty
 *   dims  [3]      host out: cells per axis, ceil((ulim - llim) / h)
 * cells = dims[0]*dims[1]*dims[2]; start/end must hold that many entries
 * (query dims first with start = end = NULL).  Uses the solver's limits and h.
 */
pbf_status pbf_build_grid(pbf_solver* s, const void* xstar, int n, uint32_t* keys,
                          uint32_t* perm, uint32_t* start, uint32_t* end, int dims[3],
                          void* stream);

/*
 * Per-phase device times of the last pbf_step, from CUDA events recorded on
 * the step's stream while profiling is enabled.  Replaces the reference's
 * Logger phase timing (fluids/Logger.cpp:27-45, fluids/Simulator.cpp:44-79),
 * which brackets phases with cudaDeviceSynchronize; here nothing synchronises
 * until pbf_profile_read, which waits for the step's last event.
 */
typedef struct pbf_step_profile {
  float grid_ms;      /* predict + hash + cell counts + radix sort */
  float reorder_ms;   /* gather into cell order */
  float lambda_ms;    /* all lambda passes */
  float delta_p_ms;   /* all position-correction passes (+ velocity update) */
  float xsph_ms;      /* XSPH pass */
  float total_ms;     /* whole step */
  int iterations;     /* solver iterations timed (up to 64) */
  int launches;       /* kernels launched by the step (also without profiling) */
  int grid_launches;  /* of which in the grid build */
} pbf_step_profile;

pbf_status pbf_profile_enable(pbf_solver* s, int on);
pbf_status pbf_profile_read(pbf_solver* s, pbf_step_profile* out);

/*
 * Whether pbf_step runs as a CUDA graph (default: on).  The step's launches
 * are captured on an internal stream, the solver's executable graph is
 * updated in place (new wall positions only change kernel arguments) and
 * launched on the caller's stream; off, the kernels are launched one by one.
 * No counterpart in the reference, which launches eagerly and synchronises.
 */
pbf_status pbf_use_graphs(pbf_solver* s, int on);

/*
 * Reverse pass (adjoint) of steps, for differentiating through the solver.
 * No counterpart in the reference.  pbf_tape_enable(s, depth) with depth > 0
 * turns the tape on as an empty stack of up to `depth` taped steps (at most
 * 1024; 0 turns it off): every following pbf_step pushes what its reverse
 * pass needs (positions entering each solver iteration and the final ones,
 * each iteration's lambda, the sorted inputs, the last density, the sort
 * permutation and the cell prefix: about (niter + 1) * 16 + niter * 4 + 28
 * bytes per particle plus 4 per cell, allocated here), and fails with
 * PBF_ERR_CAPACITY when the stack is full.  pbf_backward pops the most
 * recent taped step: it takes the adjoints of that step's outputs npos and
 * nvel (device, n float4, the step's output cell order) and writes the
 * adjoints of its inputs pos and vel (device, n float4, the step's input
 * order) and of the box limits (g_lim: device, 6 floats: ulim xyz then llim
 * xyz, through the wall clamp).  The neighbour sets and clamp states of the
 * forward are held fixed; k_boundaryDensity must be 0.  A rollout is
 * differentiated by taping a run of steps and popping them in reverse order
 * (checkpointing: re-run a segment from a saved state with the tape on).
 */
pbf_status pbf_tape_enable(pbf_solver* s, int depth);
pbf_status pbf_backward(pbf_solver* s, const void* g_npos, const void* g_nvel, void* g_pos,
                        void* g_vel, float* g_lim, void* stream);

/*
 * Poly6 density (mass 1, radius h) of n particles (device float4) at the
 * centres of a dims[0] x dims[1] x dims[2] lattice of cells spanning
 * [lo, hi] (device grid, x slowest), and the adjoint of that map: g_grid
 * (device, one float per node) -> g_pos (device, n float4).  Both are
 * gathers.  The loss of the inverse problem; no counterpart in the reference.
 * PBF_ERR_INVALID_ARG unless lo < hi (finite), h > 0 (finite) and dims >= 1
 * with fewer than 2^31 nodes.
 */
pbf_status pbf_density_grid(const void* pos, int n, const float lo[3], const float hi[3],
                            const int dims[3], float h, float* grid, void* stream);
pbf_status pbf_density_grid_backward(const void* pos, int n, const float lo[3], const float hi[3],
                                     const int dims[3], float h, const float* g_grid, void* g_pos,
                                     void* stream);

/*
 * Batched ensemble: many independent scenes of uneven particle counts, each
 * with its own box, advanced together, one launch per pass for all scenes.
 * No counterpart in the reference (one Simulator per scene there).
 * Particle arrays hold the scenes back to back: scene s occupies slots
 * [offset_s, offset_s + counts[s]), offset_s = counts[0] + ... + counts[s-1].
 * Every scene follows pbf_step's contract within its own range (stable cell
 * order, outputs, vel = (npos - pos) / dt); scenes never exchange particles.
 * All scenes share one parameter set.  At most 65535 scenes.
 */
typedef struct pbf_batch pbf_batch;

/* ulim/llim: 3 * nscenes floats; counts: nscenes particle counts, summing to
 * at most PBF_MAX_PARTICLES (else PBF_ERR_CAPACITY).  Reserves 4x the cells
 * of the initial boxes, like pbf_create. */
pbf_status pbf_batch_create(const pbf_params* params, int nscenes, const float* ulim, const float* llim,
                            const int* counts, pbf_batch** out);
pbf_status pbf_batch_destroy(pbf_batch* b);
/* Moves the walls of one scene (Simulator::setLim of that scene). */
pbf_status pbf_batch_set_limits(pbf_batch* b, int scene, const float ulim[3], const float llim[3]);
/* One step of every scene; the five buffers hold sum(counts) entries. */
pbf_status pbf_batch_step(pbf_batch* b, void* pos, void* npos, void* vel, void* nvel, uint32_t* iid,
                          void* stream);
/* rho of the last step's final lambda pass for all particles (device, sum(counts) floats). */
pbf_status pbf_batch_get_density(const pbf_batch* b, float* rho, void* stream);
pbf_status pbf_batch_use_graphs(pbf_batch* b, int on);

/*
 * Autotuning (no counterpart in the reference).  Times a few choices of how
 * the neighbour passes split their work -- the window size above which a
 * particle's window goes to the dense kernel (a block of 8 warps splitting
 * the windows of 32 particles), whether every particle does, the order in
 * which the passes take particles (the cell order of the grid, or the cell
 * each particle is in at that iteration), how many warps of the dense kernel
 * split a batch's windows, how many neighbour chunks a thread queues before
 * running their pair terms, and how many candidate positions a block of each
 * pass kernel may stage in shared memory (bulk asynchronous copies of the
 * column runs its particles' windows share, read there instead of through
 * L1) -- by running `steps` steps per choice from copies of the
 * caller's state (pos, vel, iid: device, n entries; they are not modified),
 * and keeps the fastest for the solver's following steps.  The window and
 * dense choices change the order in which window sums are added, so results
 * differ by rounding only, and so does the dense split; the particle order,
 * the queues and the staging change nothing (each particle's sums are the
 * same whichever warp computes them, in whichever loop, from whichever copy
 * of the positions).  The trial steps are not taped.  The cell
 * size stays h: with the reference's stale grid, another cell size would
 * change which neighbours a step sees.
 */
typedef struct pbf_tuning {
  int dense_window;   /* window entries above which a particle takes the dense kernel */
  int dense_all;      /* 1: every particle takes the dense kernel */
  float ms_per_step;  /* the chosen configuration's time per step */
  float ms_default;   /* the default configuration's time per step */
  int order;          /* 1: current-cell order (the default); 0: grid order */
  int bwd_lanes;      /* pbf_backward, steps under 131072 particles: lanes per particle, 8, 16
                         or 32 (0: the default, 32); not timed by pbf_autotune */
  int stage_sparse;   /* slots (16 bytes each) a block of the one-thread-per-particle kernel
                         copies into shared memory when its particles share one column of
                         cells (0: none; at most 4096) */
  int stage_dense;    /* the same for a block of the dense kernel */
  int queue_sparse;   /* neighbour chunks of 32 candidates whose hits a thread of the
                         one-thread-per-particle kernel queues before running their pair terms
                         in one loop (1: each chunk's right away; at most 16) */
  int queue_dense;    /* the same for the dense kernel (at most 8) */
  int dense_split;    /* warps of the dense kernel that split one batch of 32 particles'
                         windows: 1, 2, 4 or 8 (a block of 8 warps takes 8 / dense_split
                         batches at a time) */
  int dense_interleave; /* 1: those warps take every dense_split-th chunk of 32 candidates of a
                           window; 0: one contiguous part each (-1: the default, 0) */
} pbf_tuning;

pbf_status pbf_autotune(pbf_solver* s, const void* pos, const void* vel, const uint32_t* iid, int n, int steps,
                        pbf_tuning* out, void* stream);
pbf_status pbf_batch_autotune(pbf_batch* b, const void* pos, const void* vel, const uint32_t* iid, int steps,
                              pbf_tuning* out, void* stream);
/* The choices of the following steps, set directly (e.g. a choice an earlier
 * pbf_autotune returned): dense_window >= 32 candidates, or 0 for the
 * default; dense_all 1 (every particle dense), 0 (by window) or -1 (the
 * default: every particle dense below 131072 particles); order 1, 0 or -1
 * (the default, 1); bwd_lanes 0 (the default), 8, 16 or 32; stage_sparse and
 * stage_dense 0 (off) to 4096 slots, or -1 (the default); queue_sparse 1-16,
 * queue_dense 1-8 and dense_split 1, 2, 4 or 8, or 0 (the defaults: 1, 1,
 * 8); dense_interleave 0, 1 or -1 (the default, 0).  ms fields are ignored on set and 0 on get. */
pbf_status pbf_set_tuning(pbf_solver* s, const pbf_tuning* t);
pbf_status pbf_get_tuning(const pbf_solver* s, pbf_tuning* t);
/* The same for a batch (bwd_lanes is ignored: a batch has no reverse pass). */
pbf_status pbf_batch_set_tuning(pbf_batch* b, const pbf_tuning* t);
pbf_status pbf_batch_get_tuning(const pbf_batch* b, pbf_tuning* t);

/*
 * Errors the solver's kernels recorded on the device since the last call.
 * Waits for the solver's work on `stream` (device, as for pbf_step), then
 * returns PBF_ERR_TIMEOUT if a bounded device-side wait gave up since -- a
 * block's copy of candidate positions into shared memory that did not
 * complete; that block then read global memory instead, so the steps'
 * results are unchanged -- else PBF_OK, and clears the record.  No
 * counterpart in the reference, which does not check kernel errors.
 */
pbf_status pbf_check_device(pbf_solver* s, void* stream);
pbf_status pbf_batch_check_device(pbf_batch* b, void* stream);

/*
 * One step, same contract and results as pbf_step (bit for bit, with the
 * default tuning), for callers that cannot allocate device memory (no
 * pbf_solver, so no pbf_create).  It has no counterpart in the reference.  It
 * calls no cudaMalloc or cudaFree: its scratch is a fixed array of about
 * 11.6 MB inside this library's device image, held by every GPU that loads
 * the library until the process exits.
 * Limits: n <= 32768 particles and a box of at most 131072 cells at cell size
 * h; larger calls return PBF_ERR_CAPACITY.  The first call on each device
 * looks up the array's device address (set-up), so make it before any stream
 * capture; the address is looked up again when the device's context has
 * changed since (after cudaDeviceReset, for one).  Every call shares the
 * array: calls that overlap on the GPU race, so serialise them.
 */
pbf_status pbf_step_noalloc(const pbf_params* params, const float ulim[3], const float llim[3],
                            void* pos, void* npos, void* vel, void* nvel, uint32_t* iid, int n,
                            void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PBF_H_ */
