// api.cu — the C ABI of include/pbf.h: solver object, parameter handling,
// argument checks and the phase sequence of one step.
//
// Phase sequence of pbf_step, as Simulator::step (fluids/Simulator.cpp:10-99):
//   advect + buildGridHash  -> grid.cu  (predict, hash, counts, radix sort)
//   (gather into cell order) -> solver.cu reorder
//   niter x correctDensity   -> solver.cu lambda / delta_p (Jacobi ping-pong)
//   updateVelocity           -> fused into the last delta_p pass
//   correctVelocity (XSPH)   -> solver.cu xsph
// All of it is enqueued on the caller's stream without host synchronisation.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "pbf_internal.cuh"

// The kernels index per-particle tables with int: the neighbour masks
// (kMaskWords words per particle) and the group hash (8 ints per particle)
// are the largest.
static_assert((long long)pbf::kMaskWords * PBF_MAX_PARTICLES - 1 <= 2147483647LL,
              "mask index overflows int at PBF_MAX_PARTICLES");
static_assert(8LL * PBF_MAX_PARTICLES - 1 <= 2147483647LL, "group hash index overflows int at PBF_MAX_PARTICLES");

// Executable graphs of recent steps.  A step's launches depend only on its
// constants (box, cells, coefficients, tuning), its buffers, its particle
// count and its iterations, so a step whose key matches a cached graph's
// replays that graph: no stream capture, no graph update.  A static box with
// the reference's tic-toc buffers settles on two graphs.
struct StepKey {
  pbf::StepConsts c;
  const void* bufs[5];
  int n, niter;
};

struct GraphCache {
  static constexpr int kEntries = 4;
  struct Entry {
    StepKey key;
    bool valid = false;
    cudaGraphExec_t exec = nullptr;
    const uint32_t* keys_sorted = nullptr;  // host-side results of the capture, restored on replay
    const uint32_t* perm = nullptr;
  } e[kEntries];
  int next = 0;
  void clear() {
    for (Entry& x : e) {
      if (x.exec) cudaGraphExecDestroy(x.exec);
      x = Entry();
    }
    next = 0;
  }
};

// Executable graphs of recent reverse passes.  A reverse pass's launches
// depend only on its arguments (the taped step's constants and record, the
// scratch, the lanes) and the caller's adjoint buffers, so a call whose key
// matches a cached graph replays it.  A checkpointed rollout reverses the same
// tape slots into the same buffers segment after segment, so its calls hit.
struct BackwardKey {
  pbf::BackwardArgs a;
  pbf::BackwardTape t;
  const void* perm;
  const void* bufs[5];
};

struct BackwardCache {
  static constexpr int kEntries = 48;
  struct Entry {
    BackwardKey key;
    bool valid = false;
    cudaGraphExec_t exec = nullptr;
  } e[kEntries];
  int next = 0;
  void clear() {
    for (Entry& x : e) {
      if (x.exec) cudaGraphExecDestroy(x.exec);
      x = Entry();
    }
    next = 0;
  }
};

StepKey make_key(const pbf::StepConsts& c, void* pos, void* npos, void* vel, void* nvel, void* iid, int n,
                 int niter) {
  StepKey k;
  std::memset(&k, 0, sizeof(k));  // padding included: keys compare as bytes
  k.c = c;
  const void* b[5] = {pos, npos, vel, nvel, iid};
  for (int a = 0; a < 5; ++a) k.bufs[a] = b[a];
  k.n = n;
  k.niter = niter;
  return k;
}

// Phase boundaries recorded by pbf_step when profiling is on.
enum { kEvStart, kEvGrid, kEvReorder, kEvXsphStart, kEvEnd, kEvFixed };
constexpr int kMaxProfiledIters = 64;

// Taped steps a solver's tape can hold (pbf_tape_enable).
constexpr int kMaxTapeDepth = 1024;

struct pbf_solver {
  pbf_params params;
  float ulim[3], llim[3];
  int max_particles;
  int max_cells;
  int device;
  int num_sms;
  int last_n;  // particles of the last completed step (for pbf_get_density)
  pbf::GridScratch grid;
  pbf::SolverScratch sol;
  // profiling (Logger equivalent, fluids/Logger.cpp:27-45): CUDA events
  bool profile;
  cudaEvent_t ev[kEvFixed];
  cudaEvent_t ev_it[3 * kMaxProfiledIters];  // per iteration: lambda start, delta_p start, delta_p end
  int prof_iters;       // iterations recorded by the last profiled step (0: none)
  int last_launches;    // kernels launched by the last pbf_step
  int last_grid_launches;
  // CUDA graph of the step: captured on cap_stream, updated in place each step
  // (profiled or taped steps), or replayed from the cache
  bool use_graph;
  cudaStream_t cap_stream;
  cudaGraphExec_t exec;
  GraphCache cache;
  BackwardCache bw_cache;  // graphs of reverse passes (pbf_backward)
  // the tape (pbf_tape_enable): a stack of taped steps, each record holding
  // what the step's reverse pass needs, and the reverse pass's scratch
  int tape_depth;            // records the stack holds; 0: tape off
  int tape_top;              // records on the stack
  int tape_cap;              // records allocated
  int tape_iters;            // iterations a record holds
  size_t tape_rec;           // bytes per record
  unsigned char* tape_mem;   // tape_cap records
  struct TapeMeta {
    pbf::StepConsts c;
    int n;
    int niter;
  } tape_meta[kMaxTapeDepth];
  float4* bw4;               // 7 * max_particles: gx, gx_next, gx0, pbar, gs, fix, fixv
  unsigned char* bw_sc;      // the reverse pass's exact-scatter scratch (scatter_bytes)
  float* bw1;                // 4 * max_particles: grho, lbar, rtot (+ spare)
  unsigned long long* bw8;   // 2 * max_particles: packed grid cells, packed current cells
  float* wall_part;          // 6 * blocks
  const uint32_t* last_perm;
  // dense-kernel and order choices (pbf_autotune); tune_window 0 / tune_order -1: the defaults
  int tune_window;
  int tune_all;
  int tune_order;
  int tune_bwd_lanes;  // 0: the default (32)
  int tune_stage_sparse;  // staged slots per sparse / dense block; -1: the defaults
  int tune_stage_dense;
  int tune_queue_sparse;  // hit-queue chunks per sparse / dense thread; 0: the defaults
  int tune_queue_dense;
  int tune_split;         // dense warps per item; 0: the default
  int tune_interleave;    // dense warps take interleaved chunks; -1: the default
};

namespace {

thread_local char g_err[512] = "";

pbf_status fail(pbf_status s, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
pbf_status fail(pbf_status s, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return s;
}

pbf_status cuda_fail(cudaError_t e, const char* what) {
  return fail(PBF_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

#define PBF_CUDA(call, what)                         \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

// Reads and clears a device error word (kErrorWord) after the work queued on
// `stream`: PBF_ERR_TIMEOUT if a bounded device wait gave up.
pbf_status check_device_word(uint32_t* word, cudaStream_t stream, const char* what) {
  uint32_t bits = 0u;
  PBF_CUDA(cudaMemcpyAsync(&bits, word, sizeof(bits), cudaMemcpyDeviceToHost, stream), what);
  PBF_CUDA(cudaStreamSynchronize(stream), what);
  if (bits == 0u) return PBF_OK;
  PBF_CUDA(cudaMemsetAsync(word, 0, sizeof(uint32_t), stream), what);
  PBF_CUDA(cudaStreamSynchronize(stream), what);
  if (bits & pbf::kErrStageTimeout)
    return fail(PBF_ERR_TIMEOUT, "%s: a shared-memory staging copy did not complete in time (the pass read "
                                 "global memory instead)", what);
  return fail(PBF_ERR_CUDA, "%s: device error bits 0x%x", what, bits);
}

bool finite_f(float v) { return std::isfinite(v); }

pbf_status check_params(const pbf_params* p) {
  if (!p) return fail(PBF_ERR_INVALID_ARG, "params is NULL");
  if (p->niter < 1) return fail(PBF_ERR_INVALID_ARG, "niter must be >= 1 (got %d)", p->niter);
  const float vals[] = {p->pho0, p->g, p->h, p->dt, p->lambda_eps, p->delta_q, p->k_corr,
                        p->n_corr, p->k_boundaryDensity, p->c_XSPH, p->up[0], p->up[1],
                        p->up[2], p->lim_eps, p->kernel_eps, p->max_dp, p->vorticity_eps};
  for (float v : vals)
    if (!finite_f(v)) return fail(PBF_ERR_INVALID_ARG, "params hold a non-finite value");
  if (!(p->h > 0.f)) return fail(PBF_ERR_INVALID_ARG, "h must be > 0");
  if (!(p->dt > 0.f)) return fail(PBF_ERR_INVALID_ARG, "dt must be > 0");
  if (!(p->pho0 > 0.f)) return fail(PBF_ERR_INVALID_ARG, "pho0 must be > 0");
  if (p->max_dp < 0.f || p->lim_eps < 0.f || p->kernel_eps < 0.f || p->vorticity_eps < 0.f)
    return fail(PBF_ERR_INVALID_ARG, "max_dp, lim_eps, kernel_eps and vorticity_eps must be >= 0");
  return PBF_OK;
}

// Cells per axis as the reference computes them: (int)ceilf((ulim - llim) / h)
// in float (fluids/Simulator.cu:187-188), at least 1.
pbf_status grid_dims(const float ulim[3], const float llim[3], float h, int dims[3],
                     long long* cells) {
  long long c = 1;
  for (int a = 0; a < 3; ++a) {
    if (!finite_f(ulim[a]) || !finite_f(llim[a]))
      return fail(PBF_ERR_INVALID_ARG, "limits must be finite");
    if (!(ulim[a] > llim[a])) return fail(PBF_ERR_INVALID_ARG, "ulim must exceed llim on every axis");
    const float d = ceilf((ulim[a] - llim[a]) / h);
    if (!(d < 1e9f)) return fail(PBF_ERR_CAPACITY, "grid too large");
    dims[a] = d < 1.f ? 1 : (int)d;
    c *= dims[a];
  }
  *cells = c;
  return PBF_OK;
}

// A float parameter as the double it was typed as: the shortest decimal that
// rounds to it.  The reference's LIM_EPS is the double literal 1e-3
// (fluids/helper.h:5), and the float field 1e-3f promotes back to exactly 1e-3.
double promote_decimal(float f) {
  char buf[32];
  for (int prec = 1; prec <= 9; ++prec) {
    snprintf(buf, sizeof(buf), "%.*g", prec, (double)f);
    const double d = strtod(buf, nullptr);
    if ((float)d == f) return d;
  }
  return (double)f;
}

// A scene's box: limits, clamp bounds (double arithmetic with LIM_EPS, as the
// reference's min/max against ulim.x - LIM_EPS, fluids/Simulator_kernel.cuh:190-192),
// cells per axis and its first global cell id.
pbf::SceneGeom make_geom(const pbf_params& p, const float ulim[3], const float llim[3],
                         const int dims[3], int cell_base) {
  pbf::SceneGeom g;
  std::memset(&g, 0, sizeof(g));
  for (int a = 0; a < 3; ++a) {
    g.lo[a] = (float)((double)llim[a] + promote_decimal(p.lim_eps));
    g.hi[a] = (float)((double)ulim[a] - promote_decimal(p.lim_eps));
    g.llim[a] = llim[a];
    g.ulim[a] = ulim[a];
    g.dims[a] = dims[a];
  }
  g.cell_base = cell_base;
  return g;
}

// The reference's host-side coefficients, bit for bit (see pbf_internal.cuh).
pbf::StepConsts make_consts(const pbf_params& p, const float ulim[3], const float llim[3],
                            const int dims[3], int num_sms) {
  pbf::StepConsts c;
  std::memset(&c, 0, sizeof(c));
  const float h = p.h;
  c.h = h;
  c.h2 = h * h;
  // Host code is compiled with -ffp-contract=off, so these float expressions
  // round after every operation, as the reference's host code does.
  {
    const float ih = 1.f / h;
    const float ih3 = ih * ih * ih;
    const float ih9 = ih3 * ih3 * ih3;
    c.poly6_coef = (float)((double)(315.f * ih9) / (64.0 * pbf::kRefPi));
  }
  {
    float h6 = h * h;
    h6 = h6 * h6 * h6;
    c.spiky_coef = (float)(-45.0 / (pbf::kRefPi * (double)h6));
  }
  c.pho0 = p.pho0;
  c.inv_pho0 = 1.f / p.pho0;
  c.spiky_coef_rho0 = c.spiky_coef / p.pho0;
  c.lambda_eps = p.lambda_eps;
  {
    const float dq2 = p.delta_q * p.delta_q;
    float wdq = 0.f;
    if (dq2 < c.h2) {
      const float d = c.h2 - dq2;
      wdq = c.poly6_coef * d * d * d;
    }
    c.coef_corr = -p.k_corr / powf(wdq, p.n_corr);
  }
  c.n_corr = p.n_corr;
  c.npow = -1;
  for (int k = 1; k <= 4; ++k)
    if (p.n_corr == (float)k) c.npow = k;
  c.keps2 = p.kernel_eps * p.kernel_eps;
  c.max_dp = p.max_dp;
  c.vort_eps = p.vorticity_eps;
  c.k_b = p.k_boundaryDensity;
  c.c_xsph = p.c_XSPH;
  c.dt = p.dt;
  c.inv_dt = 1.f / p.dt;
  for (int a = 0; a < 3; ++a) c.g[a] = -p.g * p.up[a];
  c.geom = make_geom(p, ulim, llim, dims, 0);
  c.cells = dims[0] * dims[1] * dims[2];
  c.dense_grid = pbf::kDenseBlocksPerSm * (num_sms > 0 ? num_sms : 1);
  c.dense_window = pbf::kDefaultDenseWindow;
  c.dense_all = -1;
  c.order = 1;
  c.stage_sparse = pbf::kDefaultStageSparse;
  c.stage_dense = pbf::kDefaultStageDense;
  c.queue_sparse = pbf::kDefaultQueueSparse;
  c.queue_dense = pbf::kDefaultQueueDense;
  c.dense_split = pbf::kDefaultDenseSplit;
  c.dense_interleave = pbf::kDefaultDenseInterleave;
  return c;
}

// Streaming multiprocessors of the current device (1 if it cannot be queried).
int current_sms() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return sms;
}

template <typename T>
cudaError_t alloc(T** p, size_t count) {
  return cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
}

// Layout of one tape record (256-byte aligned parts): positions entering each
// iteration and the final ones X[0..iters], each iteration's lambda, the
// sorted inputs, the last lambda pass's density, the sort permutation and the
// grid's cell prefix.
struct TapeLayout {
  size_t x, l, xs, rho, perm, cs, bytes;
  TapeLayout(size_t np, size_t cells1, int iters) {
    auto up = [](size_t v) { return (v + 255) / 256 * 256; };
    x = 0;
    l = x + up(sizeof(float4) * np * (iters + 1));
    xs = l + up(sizeof(float) * np * iters);
    rho = xs + up(sizeof(float4) * np);
    perm = rho + up(sizeof(float) * np);
    cs = perm + up(sizeof(uint32_t) * np);
    bytes = cs + up(sizeof(uint32_t) * cells1);
  }
};

// Group tables for up to max_particles particles (pbf_internal.cuh).
cudaError_t alloc_groups(pbf::SolverScratch& sol, int max_particles) {
  const size_t slots = pbf::group_slots(max_particles);
  const size_t entries = (size_t)max_particles;
  sol.grp_pool = max_particles;
  cudaError_t e = alloc(&sol.grp_cell, slots);
  if (e == cudaSuccess) e = alloc(&sol.grp_off, slots);
  if (e == cudaSuccess) e = alloc(&sol.grp_n, slots);
  if (e == cudaSuccess) e = alloc(&sol.grp_rep, entries);
  if (e == cudaSuccess) e = alloc(&sol.grp_cnt, entries);
  if (e == cudaSuccess) e = alloc(&sol.grp_pos, entries);
  if (e == cudaSuccess) e = alloc(&sol.grp_sum, entries);
  if (e == cudaSuccess) e = alloc(&sol.grp_aux, entries);
  if (e == cudaSuccess) e = alloc(&sol.grp_id, entries);
  if (e == cudaSuccess) e = alloc(&sol.grp_hash, 8 * entries);
  if (e == cudaSuccess) e = alloc(&sol.grp_max, entries);
  if (e == cudaSuccess) e = alloc(&sol.grp_acc, 3 * entries);
  if (e == cudaSuccess) e = alloc(&sol.grp_list, entries);
  if (e == cudaSuccess) e = alloc(&sol.grp_list_n, slots);
  if (e == cudaSuccess) e = alloc(&sol.grp_done, slots);
  if (e == cudaSuccess) e = alloc(&sol.grp_zero, slots);
  if (e == cudaSuccess) e = alloc(&sol.grp_item_off, slots);
  if (e == cudaSuccess) e = alloc(&sol.grp_item_slot, pbf::group_items(max_particles));
  if (e == cudaSuccess) e = alloc(&sol.work_list, (size_t)max_particles + 1);
  if (e == cudaSuccess) e = alloc(&sol.work_follow, (size_t)max_particles + 1);
  if (e == cudaSuccess) e = alloc(&sol.work_blocks, pbf::work_blocks_len(max_particles));
  // what the group kernels expect to find at zero
  if (e == cudaSuccess) e = cudaMemset(sol.grp_hash, 0, sizeof(int) * 8 * entries);
  if (e == cudaSuccess) e = cudaMemset(sol.grp_max, 0, sizeof(unsigned) * entries);
  if (e == cudaSuccess) e = cudaMemset(sol.grp_acc, 0, sizeof(unsigned long long) * 3 * entries);
  if (e == cudaSuccess) e = cudaMemset(sol.grp_list_n, 0, sizeof(int) * slots);
  if (e == cudaSuccess) e = cudaMemset(sol.grp_done, 0, sizeof(int) * slots);
  return e;
}

// Current-cell buckets (StepConsts::order) for up to np particles and nc - 1 cells.
cudaError_t alloc_buckets(pbf::SolverScratch& sol, size_t np, size_t nc) {
  cudaError_t e = alloc(&sol.bcnt, nc);
  if (e == cudaSuccess) e = alloc(&sol.bstart, nc);
  if (e == cudaSuccess) e = alloc(&sol.bent, np);
  if (e == cudaSuccess) e = alloc(&sol.bucket, np);
  if (e == cudaSuccess) e = alloc(&sol.bpart, (size_t)pbf::kMaxScanPartials);
  return e;
}

void free_all(pbf_solver* s) {
  void* ptrs[] = {s->grid.keys_a, s->grid.keys_b, s->grid.vals_a, s->grid.vals_b,
                  s->grid.cell_count, s->grid.cell_start, s->grid.radix_counts,
                  s->grid.scan_partials, s->sol.xs, s->sol.xa, s->sol.xb, s->sol.iid_s,
                  s->sol.lambda, s->sol.rho, s->sol.flags, s->sol.dense, s->sol.masks,
                  s->sol.cell_flags, s->sol.grp_cell, s->sol.grp_off, s->sol.grp_n, s->sol.grp_rep, s->sol.grp_cnt,
                  s->sol.grp_pos, s->sol.grp_sum, s->sol.grp_aux, s->sol.grp_id, s->sol.grp_hash,
                  s->sol.grp_max, s->sol.grp_acc, s->sol.grp_list, s->sol.grp_list_n, s->sol.grp_done,
                  s->sol.grp_zero, s->sol.grp_item_off, s->sol.grp_item_slot, s->sol.work_list,
                  s->sol.work_follow, s->sol.work_blocks, s->sol.bcnt, s->sol.bstart, s->sol.bent,
                  s->sol.bucket, s->sol.bpart};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (cudaEvent_t& e : s->ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t& e : s->ev_it)
    if (e) cudaEventDestroy(e);
  if (s->exec) cudaGraphExecDestroy(s->exec);
  s->cache.clear();
  s->bw_cache.clear();
  if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
  void* tape[] = {s->tape_mem, s->bw4, s->bw1, s->bw8, s->wall_part, s->bw_sc};
  for (void* p : tape)
    if (p) cudaFree(p);
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// The parts of the reverse pass's exact-scatter scratch (pbf::scatter_bytes(np) bytes at base).
void scatter_layout(unsigned char* base, size_t np, pbf::BackwardArgs& a) {
  const size_t cap = np * pbf::kScatterPerParticle;
  unsigned char* p = base;
  a.sc_val = (float4*)p;
  p += sizeof(float4) * cap;
  a.sc_acc = (unsigned long long*)p;
  p += sizeof(unsigned long long) * 7 * np;
  a.sc_key = (int2*)p;
  p += sizeof(int2) * cap;
  a.sc_max = (unsigned*)p;
  p += sizeof(unsigned) * 7 * np;
  a.sc_cnt = (unsigned*)p;
  p += sizeof(unsigned) * 2 * np;
  a.sc_nonfin = (unsigned*)p;
  p += sizeof(unsigned) * np;
  a.sc_ctr = (unsigned*)p;
  a.sc_cap = (int)cap;
  a.sc_stride = (int)np;
}

}  // namespace

extern "C" {

void pbf_params_default(pbf_params* out) {
  if (!out) return;
  std::memset(out, 0, sizeof(*out));
  out->niter = 4;
  out->pho0 = 8000.f;
  out->g = 9.8f;
  out->h = .1f;
  out->dt = 0.0083f;
  out->lambda_eps = 1000.f;
  out->delta_q = (float)(0.3 * out->h);
  out->k_corr = 0.001f;
  out->n_corr = 4.f;
  out->k_boundaryDensity = 0.f;
  out->c_XSPH = 0.5f;
  out->up[0] = 0.f;
  out->up[1] = 0.f;
  out->up[2] = 1.f;
  out->lim_eps = 1e-3f;
  out->kernel_eps = 1e-4f;
  out->max_dp = 0.1f;
  out->vorticity_eps = 0.f;
}

const char* pbf_status_string(pbf_status s) {
  switch (s) {
    case PBF_OK: return "ok";
    case PBF_ERR_INVALID_ARG: return "invalid argument";
    case PBF_ERR_CAPACITY: return "capacity exceeded";
    case PBF_ERR_CUDA: return "CUDA error";
    case PBF_ERR_TIMEOUT: return "device wait timed out";
    case PBF_ERR_NOT_READY: return "no step results yet";
  }
  return "unknown status";
}

const char* pbf_last_error(void) { return g_err; }

int pbf_abi_version(void) { return PBF_ABI_VERSION; }

pbf_status pbf_create(const pbf_params* params, const float ulim[3], const float llim[3],
                      int max_particles, pbf_solver** out) {
  g_err[0] = 0;
  if (!out) return fail(PBF_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (!ulim || !llim) return fail(PBF_ERR_INVALID_ARG, "limits are NULL");
  if (max_particles < 0) return fail(PBF_ERR_INVALID_ARG, "max_particles < 0");
  if (max_particles > PBF_MAX_PARTICLES)
    return fail(PBF_ERR_CAPACITY, "max_particles = %d exceeds %d", max_particles, PBF_MAX_PARTICLES);
  pbf_status st = check_params(params);
  if (st != PBF_OK) return st;
  int dims[3];
  long long cells;
  if ((st = grid_dims(ulim, llim, params->h, dims, &cells)) != PBF_OK) return st;
  // 4x the initial box's cells, like the reference's ngrid (fluids/Simulator.h:13-14),
  // so a moving wall can widen the box.
  long long max_cells = 4 * cells;
  const long long scan_cap = (long long)pbf::kScanTile * pbf::kMaxScanPartials - 1;
  if (max_cells > scan_cap) max_cells = cells;
  if (max_cells > scan_cap) return fail(PBF_ERR_CAPACITY, "box needs %lld cells, limit %lld", cells, scan_cap);

  // value-initialised: every pointer, handle and count zero, the graph cache empty
  pbf_solver* s = new (std::nothrow) pbf_solver();
  if (!s) return fail(PBF_ERR_CAPACITY, "host allocation failed");
  s->tune_all = -1;
  s->tune_order = -1;
  s->tune_stage_sparse = -1;
  s->tune_stage_dense = -1;
  s->tune_interleave = -1;
  s->params = *params;
  std::memcpy(s->ulim, ulim, sizeof(s->ulim));
  std::memcpy(s->llim, llim, sizeof(s->llim));
  s->max_particles = max_particles;
  s->max_cells = (int)max_cells;
  cudaError_t e = cudaGetDevice(&s->device);
  const size_t np = (size_t)max_particles;
  const size_t nc = (size_t)max_cells + 1;
  if (e == cudaSuccess) e = alloc(&s->grid.keys_a, np);
  if (e == cudaSuccess) e = alloc(&s->grid.keys_b, np);
  if (e == cudaSuccess) e = alloc(&s->grid.vals_a, np);
  if (e == cudaSuccess) e = alloc(&s->grid.vals_b, np);
  if (e == cudaSuccess) e = alloc(&s->grid.cell_count, nc);
  if (e == cudaSuccess) e = alloc(&s->grid.cell_start, nc);
  if (e == cudaSuccess) e = alloc(&s->grid.radix_counts, pbf::radix_counts_len(max_particles));
  if (e == cudaSuccess) e = alloc(&s->grid.scan_partials, (size_t)pbf::kMaxScanPartials);
  if (e == cudaSuccess) e = alloc(&s->sol.xs, np);
  if (e == cudaSuccess) e = alloc(&s->sol.xa, np);
  if (e == cudaSuccess) e = alloc(&s->sol.xb, np);
  if (e == cudaSuccess) e = alloc(&s->sol.iid_s, np);
  if (e == cudaSuccess) e = alloc(&s->sol.lambda, np);
  if (e == cudaSuccess) e = alloc(&s->sol.rho, np);
  if (e == cudaSuccess) e = alloc(&s->sol.flags, (size_t)pbf::kFlagWords);
  if (e == cudaSuccess) e = cudaMemset(s->sol.flags, 0, sizeof(uint32_t) * pbf::kFlagWords);
  if (e == cudaSuccess) e = alloc(&s->sol.dense, pbf::dense_list_len(max_particles));
  if (e == cudaSuccess) e = alloc(&s->sol.masks, (size_t)pbf::kMaskWords * np);
  s->sol.mask_stride = (int)np;
  if (e == cudaSuccess) e = alloc(&s->sol.cell_flags, nc);
  if (e == cudaSuccess) e = alloc_groups(s->sol, max_particles);
  if (e == cudaSuccess) e = alloc_buckets(s->sol, np, nc);
  if (e == cudaSuccess) s->num_sms = current_sms();
  if (e == cudaSuccess) e = pbf::set_pass_kernel_attributes();
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking);
  s->use_graph = true;
  if (e != cudaSuccess) {
    free_all(s);
    delete s;
    cudaGetLastError();
    return cuda_fail(e, "pbf_create: cudaMalloc");
  }
  *out = s;
  return PBF_OK;
}

pbf_status pbf_destroy(pbf_solver* s) {
  if (!s) return PBF_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != s->device) cudaSetDevice(s->device);
  free_all(s);
  if (prev >= 0 && prev != s->device) cudaSetDevice(prev);
  delete s;
  return PBF_OK;
}

pbf_status pbf_set_params(pbf_solver* s, const pbf_params* params) {
  if (!s) return fail(PBF_ERR_INVALID_ARG, "solver is NULL");
  pbf_status st = check_params(params);
  if (st != PBF_OK) return st;
  int dims[3];
  long long cells;
  if ((st = grid_dims(s->ulim, s->llim, params->h, dims, &cells)) != PBF_OK) return st;
  if (cells > s->max_cells)
    return fail(PBF_ERR_CAPACITY, "h = %g needs %lld cells, %d allocated", params->h, cells, s->max_cells);
  s->params = *params;
  return PBF_OK;
}

pbf_status pbf_get_params(const pbf_solver* s, pbf_params* out) {
  if (!s || !out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
  *out = s->params;
  return PBF_OK;
}

pbf_status pbf_set_limits(pbf_solver* s, const float ulim[3], const float llim[3]) {
  if (!s || !ulim || !llim) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
  int dims[3];
  long long cells;
  pbf_status st = grid_dims(ulim, llim, s->params.h, dims, &cells);
  if (st != PBF_OK) return st;
  if (cells > s->max_cells)
    return fail(PBF_ERR_CAPACITY, "box needs %lld cells, %d allocated", cells, s->max_cells);
  std::memcpy(s->ulim, ulim, sizeof(s->ulim));
  std::memcpy(s->llim, llim, sizeof(s->llim));
  return PBF_OK;
}

pbf_status pbf_get_limits(const pbf_solver* s, float ulim[3], float llim[3]) {
  if (!s || !ulim || !llim) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
  std::memcpy(ulim, s->ulim, sizeof(s->ulim));
  std::memcpy(llim, s->llim, sizeof(s->llim));
  return PBF_OK;
}

}  // extern "C"

namespace {

// One step's launches: constants, geometry, scratch, and the profiling
// events (null when the step is not profiled).
struct StepPlan {
  pbf::StepConsts c;
  pbf::Geometry G;
  pbf::GridScratch* grid;
  pbf::SolverScratch* sol;
  int niter;
  cudaEvent_t* ev;     // [kEvFixed] or null
  cudaEvent_t* ev_it;  // [3 * kMaxProfiledIters] or null
  unsigned char* tape;  // the tape record this step fills (null: not taped)
  size_t tape_x, tape_l, tape_xs, tape_rho, tape_perm, tape_cs;  // its parts (byte offsets)
  int tape_stride;     // particles per part slot
  const uint32_t** perm_out;  // receives the step's sort permutation
};

// Enqueues one step on stream st_ (a capturing stream when building the graph).
pbf_status enqueue_step(const StepPlan& P, void* pos, void* npos, void* vel, void* nvel,
                        uint32_t* iid, int n, cudaStream_t st_) {
  const pbf::StepConsts& c = P.c;
  const pbf::Geometry& G = P.G;
  const int niter = P.niter;
  const int piters = niter < kMaxProfiledIters ? niter : kMaxProfiledIters;
  const bool prof = P.ev != nullptr;
  // Under stream capture the record must be External to become an
  // event-record node of the graph (a plain record would only order the
  // capture); outside capture the flag is not allowed.
  cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
  if (prof) PBF_CUDA(cudaStreamIsCapturing(st_, &cap_status), "pbf_step: capture status");
  const unsigned ev_flags = cap_status == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : 0u;
#define PBF_EV(e) \
  if (prof) PBF_CUDA(cudaEventRecordWithFlags((e), st_, ev_flags), "pbf_step: event")
  PBF_EV(P.ev[kEvStart]);
  // advect + buildGridHash (fluids/Simulator.cpp:46-53)
  const uint32_t* perm = nullptr;
  PBF_CUDA(pbf::build_grid(c, G, (const float4*)pos, (const float4*)vel, nullptr, n, *P.grid, &perm,
                           nullptr, st_),
           "pbf_step: grid");
  PBF_EV(P.ev[kEvGrid]);
  if (P.perm_out) *P.perm_out = perm;
  P.sol->keys_sorted = P.grid->keys_sorted;
  P.sol->cell_start = P.grid->cell_start;
  PBF_CUDA(pbf::reorder(c, perm, (const float4*)pos, (const float4*)vel, iid, n, *P.sol, st_),
           "pbf_step: reorder");
  PBF_EV(P.ev[kEvReorder]);
  const size_t ts = (size_t)P.tape_stride;
  float4* tape_x = P.tape ? (float4*)(P.tape + P.tape_x) : nullptr;
  float* tape_l = P.tape ? (float*)(P.tape + P.tape_l) : nullptr;
#define PBF_TAPE(dst, src, bytes) \
  if (P.tape) PBF_CUDA(cudaMemcpyAsync((dst), (src), (bytes), cudaMemcpyDeviceToDevice, st_), "pbf_step: tape")
  PBF_TAPE(tape_x, P.sol->xa, sizeof(float4) * n);
  // niter x correctDensity (fluids/Simulator.cpp:55-60), Jacobi ping-pong;
  // updateVelocity fused into the last position update (fluids/Simulator.cpp:62-66)
  const uint32_t* cs = P.grid->cell_start;
  const pbf::SolverScratch& sol = *P.sol;
  float4* X = sol.xa;
  float4* T = sol.xb;
  for (int it = 0; it < niter; ++it) {
    if (it < piters) PBF_EV(P.ev_it[3 * it]);
    PBF_CUDA(pbf::launch_lambda(c, G, X, cs, n, sol, 2 * it, st_), "pbf_step: lambda");
    PBF_TAPE(tape_l + ts * it, sol.lambda, sizeof(float) * n);
    if (it < piters) PBF_EV(P.ev_it[3 * it + 1]);
    if (it + 1 < niter) {
      PBF_CUDA(pbf::launch_delta_p(c, G, X, cs, n, sol, 2 * it + 1, T, st_), "pbf_step: delta_p");
      PBF_TAPE(tape_x + ts * (it + 1), T, sizeof(float4) * n);
      float4* t = X;
      X = T;
      T = t;
    } else {
      PBF_CUDA(pbf::launch_delta_p_final(c, G, X, cs, n, sol, 2 * it + 1, (float4*)pos,
                                         (float4*)npos, (float4*)vel, iid, st_),
               "pbf_step: delta_p");
      PBF_TAPE(tape_x + ts * (it + 1), npos, sizeof(float4) * n);
    }
    if (it < piters) PBF_EV(P.ev_it[3 * it + 2]);
  }
  // correctVelocity: XSPH (fluids/Simulator.cpp:68-71)
  PBF_EV(P.ev[kEvXsphStart]);
  PBF_CUDA(pbf::launch_xsph(c, G, (const float4*)npos, (const float4*)vel, cs, n, sol, 2 * niter,
                            (float4*)nvel, st_),
           "pbf_step: xsph");
  if (c.vort_eps > 0.f)
    PBF_CUDA(pbf::launch_vorticity(c, G, (const float4*)npos, cs, n, sol, (float4*)nvel, st_),
             "pbf_step: vorticity");
  PBF_EV(P.ev[kEvEnd]);
  // the rest of the record: sorted inputs, last density, permutation, cell prefix
  PBF_TAPE(P.tape + P.tape_xs, P.sol->xs, sizeof(float4) * n);
  PBF_TAPE(P.tape + P.tape_rho, P.sol->rho, sizeof(float) * n);
  PBF_TAPE(P.tape + P.tape_perm, perm, sizeof(uint32_t) * n);
  PBF_TAPE(P.tape + P.tape_cs, P.grid->cell_start, sizeof(uint32_t) * (c.cells + 1));
#undef PBF_EV
#undef PBF_TAPE
  return PBF_OK;
}

// Captures the step into a graph, updates the executable graph `exec` in
// place (kernel arguments change every step as the walls move; the topology
// does not) or re-instantiates it, and launches it on st_.
pbf_status launch_step_graph(const StepPlan& P, cudaStream_t cap, cudaGraphExec_t* exec, void* pos,
                             void* npos, void* vel, void* nvel, uint32_t* iid, int n,
                             cudaStream_t st_) {
  PBF_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), "pbf_step: begin capture");
  const pbf_status est = enqueue_step(P, pos, npos, vel, nvel, iid, n, cap);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(cap, &g);
  if (est != PBF_OK) {
    if (g) cudaGraphDestroy(g);
    return est;
  }
  if (ce != cudaSuccess) return cuda_fail(ce, "pbf_step: end capture");
  if (*exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(*exec, g, &info) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphExecDestroy(*exec);
      *exec = nullptr;
    }
  }
  if (!*exec) {
    const cudaError_t ie = cudaGraphInstantiate(exec, g, 0);
    if (ie != cudaSuccess) {
      cudaGraphDestroy(g);
      *exec = nullptr;
      return cuda_fail(ie, "pbf_step: graph instantiate");
    }
  }
  cudaGraphDestroy(g);
  PBF_CUDA(cudaGraphLaunch(*exec, st_), "pbf_step: graph launch");
  return PBF_OK;
}

// Replays the cached graph of a step with this key, or captures the step into
// a cache entry (the oldest) and launches it.
pbf_status launch_cached(const StepPlan& P, GraphCache& cache, cudaStream_t cap, void* pos, void* npos,
                         void* vel, void* nvel, uint32_t* iid, int n, cudaStream_t st_) {
  const StepKey key = make_key(P.c, pos, npos, vel, nvel, iid, n, P.niter);
  for (GraphCache::Entry& x : cache.e) {
    if (x.valid && std::memcmp(&x.key, &key, sizeof(key)) == 0) {
      P.grid->keys_sorted = x.keys_sorted;
      P.sol->keys_sorted = x.keys_sorted;
      P.sol->cell_start = P.grid->cell_start;
      if (P.perm_out) *P.perm_out = x.perm;
      PBF_CUDA(cudaGraphLaunch(x.exec, st_), "pbf_step: graph launch");
      return PBF_OK;
    }
  }
  GraphCache::Entry& x = cache.e[cache.next];
  cache.next = (cache.next + 1) % GraphCache::kEntries;
  x.valid = false;
  const uint32_t* perm = nullptr;
  StepPlan Q = P;
  Q.perm_out = &perm;
  const pbf_status st = launch_step_graph(Q, cap, &x.exec, pos, npos, vel, nvel, iid, n, st_);
  if (st != PBF_OK) return st;
  if (P.perm_out) *P.perm_out = perm;
  x.key = key;
  x.keys_sorted = P.grid->keys_sorted;
  x.perm = perm;
  x.valid = true;
  return PBF_OK;
}

}  // namespace

extern "C" {

pbf_status pbf_step(pbf_solver* s, void* pos, void* npos, void* vel, void* nvel, uint32_t* iid,
                    int n, void* stream) {
  const pbf::NvtxRange range("pbf_step");
  if (!s) return fail(PBF_ERR_INVALID_ARG, "solver is NULL");
  if (n < 0) return fail(PBF_ERR_INVALID_ARG, "n < 0");
  if (n > s->max_particles)
    return fail(PBF_ERR_CAPACITY, "n = %d exceeds max_particles = %d", n, s->max_particles);
  if (n == 0) return PBF_OK;
  const void* bufs[5] = {pos, npos, vel, nvel, iid};
  for (int a = 0; a < 5; ++a) {
    if (!bufs[a]) return fail(PBF_ERR_INVALID_ARG, "buffer %d is NULL", a);
    if (!aligned16(bufs[a]) && a < 4) return fail(PBF_ERR_INVALID_ARG, "buffer %d not 16-byte aligned", a);
    for (int b = 0; b < a; ++b)
      if (bufs[a] == bufs[b]) return fail(PBF_ERR_INVALID_ARG, "buffers %d and %d alias", b, a);
  }
  int dims[3];
  long long cells;
  pbf_status st = grid_dims(s->ulim, s->llim, s->params.h, dims, &cells);
  if (st != PBF_OK) return st;
  if (cells > s->max_cells) return fail(PBF_ERR_CAPACITY, "box needs %lld cells", cells);
  cudaStream_t st_ = (cudaStream_t)stream;
  const bool prof = s->profile;
  s->prof_iters = 0;
  StepPlan P;
  P.c = make_consts(s->params, s->ulim, s->llim, dims, s->num_sms);
  if (s->tune_window > 0) P.c.dense_window = s->tune_window;
  P.c.dense_all = s->tune_all;
  if (s->tune_order >= 0) P.c.order = s->tune_order;
  if (s->tune_stage_sparse >= 0) P.c.stage_sparse = s->tune_stage_sparse;
  if (s->tune_stage_dense >= 0) P.c.stage_dense = s->tune_stage_dense;
  if (s->tune_queue_sparse > 0) P.c.queue_sparse = s->tune_queue_sparse;
  if (s->tune_queue_dense > 0) P.c.queue_dense = s->tune_queue_dense;
  if (s->tune_split > 0) P.c.dense_split = s->tune_split;
  if (s->tune_interleave >= 0) P.c.dense_interleave = s->tune_interleave;
  P.G = pbf::Geometry{nullptr, nullptr};
  P.grid = &s->grid;
  P.sol = &s->sol;
  P.niter = s->params.niter;
  P.ev = prof ? s->ev : nullptr;
  P.ev_it = prof ? s->ev_it : nullptr;
  const bool taping = s->tape_depth > 0;
  if (taping && s->params.niter > s->tape_iters)
    return fail(PBF_ERR_CAPACITY, "tape records hold %d iterations, params ask for %d (re-enable the tape)",
                s->tape_iters, s->params.niter);
  if (taping && (s->params.k_boundaryDensity != 0.f || s->params.vorticity_eps != 0.f))
    return fail(PBF_ERR_INVALID_ARG, "the reverse pass needs k_boundaryDensity == 0 and vorticity_eps == 0");
  if (taping && s->tape_top >= s->tape_depth)
    return fail(PBF_ERR_CAPACITY, "the tape holds %d taped steps: run pbf_backward or re-enable the tape",
                s->tape_depth);
  const TapeLayout tl((size_t)s->max_particles, (size_t)s->max_cells + 1, s->tape_iters);
  P.tape = taping ? s->tape_mem + tl.bytes * (size_t)s->tape_top : nullptr;
  P.tape_x = tl.x, P.tape_l = tl.l, P.tape_xs = tl.xs, P.tape_rho = tl.rho, P.tape_perm = tl.perm;
  P.tape_cs = tl.cs;
  P.tape_stride = s->max_particles;
  P.perm_out = &s->last_perm;
  const pbf::StepConsts& c = P.c;
  if (!s->use_graph)
    st = enqueue_step(P, pos, npos, vel, nvel, iid, n, st_);
  else if (prof || taping)  // event and tape nodes are the step's own: capture it
    st = launch_step_graph(P, s->cap_stream, &s->exec, pos, npos, vel, nvel, iid, n, st_);
  else
    st = launch_cached(P, s->cache, s->cap_stream, pos, npos, vel, nvel, iid, n, st_);
  if (st != PBF_OK) return st;
  const int niter = s->params.niter;
  s->last_grid_launches = pbf::grid_launches(c, n);
  s->last_launches = s->last_grid_launches + 1 + pbf::pass_launches(c, n) * (2 * niter + 1) +
                     pbf::group_launches(c, n, niter) + pbf::bucket_launches(c, niter) +
                     (c.vort_eps > 0.f ? pbf::kVorticityLaunches : 0);
  if (prof) s->prof_iters = niter < kMaxProfiledIters ? niter : kMaxProfiledIters;
  s->last_n = n;
  if (taping) {
    s->tape_meta[s->tape_top] = {c, n, niter};
    ++s->tape_top;
  }
  return PBF_OK;
}

pbf_status pbf_tape_enable(pbf_solver* s, int depth) {
  if (!s) return fail(PBF_ERR_INVALID_ARG, "solver is NULL");
  s->tape_top = 0;
  if (depth <= 0) {
    s->tape_depth = 0;
    return PBF_OK;
  }
  s->tape_depth = 0;
  if (s->params.k_boundaryDensity != 0.f || s->params.vorticity_eps != 0.f)
    return fail(PBF_ERR_INVALID_ARG, "the reverse pass needs k_boundaryDensity == 0 and vorticity_eps == 0");
  if (depth > kMaxTapeDepth) return fail(PBF_ERR_CAPACITY, "at most %d taped steps", kMaxTapeDepth);
  const int iters = s->params.niter;
  if (iters > pbf::kMaxTapeIters) return fail(PBF_ERR_CAPACITY, "at most %d taped iterations", pbf::kMaxTapeIters);
  const size_t np = (size_t)(s->max_particles > 0 ? s->max_particles : 1);
  if (!s->bw4) {
    const size_t blocks = (np * 32 + 127) / 128;  // the reverse kernels' blocks at 32 lanes per particle
    cudaError_t e = alloc(&s->bw4, np * 7);
    if (e == cudaSuccess) e = alloc(&s->bw1, np * 4);
    if (e == cudaSuccess) e = alloc(&s->bw8, np * 2);
    if (e == cudaSuccess) e = cudaMemset(s->bw4 + 5 * np, 0, sizeof(float4) * 2 * np);
    if (e == cudaSuccess) e = alloc(&s->wall_part, blocks * 6);
    // the exact-scatter scratch starts (and is left by every fold) at zero
    if (e == cudaSuccess) e = alloc(&s->bw_sc, pbf::scatter_bytes(np));
    if (e == cudaSuccess) e = cudaMemset(s->bw_sc, 0, pbf::scatter_bytes(np));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cuda_fail(e, "pbf_tape_enable");
    }
  }
  if (depth > s->tape_cap || iters > s->tape_iters) {
    s->bw_cache.clear();  // its graphs point into the old records
    if (s->tape_mem) cudaFree(s->tape_mem);
    s->tape_mem = nullptr;
    s->tape_cap = 0;
    const int it = iters > s->tape_iters ? iters : s->tape_iters;
    const int cap = depth > s->tape_cap ? depth : s->tape_cap;
    const TapeLayout tl(np, (size_t)s->max_cells + 1, it);
    cudaError_t e = alloc(&s->tape_mem, tl.bytes * (size_t)cap);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cuda_fail(e, "pbf_tape_enable");
    }
    s->tape_iters = it;
    s->tape_cap = cap;
  }
  s->tape_depth = depth;
  return PBF_OK;
}

pbf_status pbf_backward(pbf_solver* s, const void* g_npos, const void* g_nvel, void* g_pos,
                        void* g_vel, float* g_lim, void* stream) {
  const pbf::NvtxRange range("pbf_backward");
  if (!s) return fail(PBF_ERR_INVALID_ARG, "solver is NULL");
  if (s->tape_top <= 0) return fail(PBF_ERR_NOT_READY, "no taped step to reverse");
  if (!g_npos || !g_nvel || !g_pos || !g_vel || !g_lim) return fail(PBF_ERR_INVALID_ARG, "NULL buffer");
  const int slot = s->tape_top - 1;
  const pbf_solver::TapeMeta& m = s->tape_meta[slot];
  const size_t np = (size_t)s->max_particles;
  const TapeLayout tl(np, (size_t)s->max_cells + 1, s->tape_iters);
  unsigned char* rec = s->tape_mem + tl.bytes * (size_t)slot;
  pbf::BackwardArgs a;
  std::memset(&a, 0, sizeof(a));
  a.c = m.c;
  a.G = pbf::Geometry{nullptr, nullptr};
  a.cs = (const uint32_t*)(rec + tl.cs);
  a.n = m.n;
  a.xs = (const float4*)(rec + tl.xs);
  a.rho = (const float*)(rec + tl.rho);
  a.gx = s->bw4;
  a.gx_next = s->bw4 + np;
  a.gx0 = s->bw4 + 2 * np;
  a.pbar = s->bw4 + 3 * np;
  a.gs = s->bw4 + 4 * np;
  a.grho = s->bw1;
  a.lbar = s->bw1 + np;
  a.rtot = s->bw1 + 2 * np;
  a.fix = s->bw4 + 5 * np;
  a.fixv = s->bw4 + 6 * np;
  scatter_layout(s->bw_sc, np, a);
  a.lanes = s->tune_bwd_lanes > 0 ? s->tune_bwd_lanes : 32;
  a.gcell = s->bw8;
  a.kcell = s->bw8 + np;
  a.wall_part = s->wall_part;
  pbf::BackwardTape t;
  std::memset(&t, 0, sizeof(t));  // unused slots included: keys compare as bytes
  t.niter = m.niter;
  float4* X = (float4*)(rec + tl.x);
  float* L = (float*)(rec + tl.l);
  for (int k = 0; k <= t.niter; ++k) t.X[k] = X + np * k;
  for (int k = 0; k < t.niter; ++k) t.lambda[k] = L + np * k;
  const uint32_t* perm = (const uint32_t*)(rec + tl.perm);
  cudaStream_t st_ = (cudaStream_t)stream;
  if (!s->use_graph) {
    PBF_CUDA(pbf::backward(a, t, perm, g_npos, g_nvel, g_pos, g_vel, g_lim, st_), "pbf_backward");
    s->tape_top = slot;
    return PBF_OK;
  }
  // as one CUDA graph: replayed from the cache, or captured into its oldest entry
  BackwardKey key;
  std::memset(&key, 0, sizeof(key));
  key.a = a;
  key.t = t;
  key.perm = perm;
  const void* bufs[5] = {g_npos, g_nvel, g_pos, g_vel, g_lim};
  for (int k = 0; k < 5; ++k) key.bufs[k] = bufs[k];
  for (BackwardCache::Entry& x : s->bw_cache.e) {
    if (x.valid && std::memcmp(&x.key, &key, sizeof(key)) == 0) {
      PBF_CUDA(cudaGraphLaunch(x.exec, st_), "pbf_backward: graph launch");
      s->tape_top = slot;
      return PBF_OK;
    }
  }
  BackwardCache::Entry& x = s->bw_cache.e[s->bw_cache.next];
  s->bw_cache.next = (s->bw_cache.next + 1) % BackwardCache::kEntries;
  x.valid = false;
  PBF_CUDA(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal), "pbf_backward: begin capture");
  const cudaError_t be = pbf::backward(a, t, perm, g_npos, g_nvel, g_pos, g_vel, g_lim, s->cap_stream);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(s->cap_stream, &g);
  if (be != cudaSuccess || ce != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_fail(be != cudaSuccess ? be : ce, "pbf_backward: capture");
  }
  if (x.exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(x.exec, g, &info) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphExecDestroy(x.exec);
      x.exec = nullptr;
    }
  }
  if (!x.exec) {
    const cudaError_t ie = cudaGraphInstantiate(&x.exec, g, 0);
    if (ie != cudaSuccess) {
      cudaGraphDestroy(g);
      x.exec = nullptr;
      return cuda_fail(ie, "pbf_backward: graph instantiate");
    }
  }
  cudaGraphDestroy(g);
  PBF_CUDA(cudaGraphLaunch(x.exec, st_), "pbf_backward: graph launch");
  x.key = key;
  x.valid = true;
  s->tape_top = slot;
  return PBF_OK;
}

pbf_status pbf_use_graphs(pbf_solver* s, int on) {
  if (!s) return fail(PBF_ERR_INVALID_ARG, "solver is NULL");
  s->use_graph = on != 0;
  return PBF_OK;
}

pbf_status pbf_profile_enable(pbf_solver* s, int on) {
  if (!s) return fail(PBF_ERR_INVALID_ARG, "solver is NULL");
  if (on && !s->ev[0]) {
    for (cudaEvent_t& e : s->ev) PBF_CUDA(cudaEventCreate(&e), "pbf_profile_enable");
    for (cudaEvent_t& e : s->ev_it) PBF_CUDA(cudaEventCreate(&e), "pbf_profile_enable");
  }
  s->profile = on != 0;
  return PBF_OK;
}

pbf_status pbf_profile_read(pbf_solver* s, pbf_step_profile* out) {
  if (!s || !out) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
  std::memset(out, 0, sizeof(*out));
  out->launches = s->last_launches;
  out->grid_launches = s->last_grid_launches;
  if (s->prof_iters == 0) return fail(PBF_ERR_NOT_READY, "no profiled step recorded");
  PBF_CUDA(cudaEventSynchronize(s->ev[kEvEnd]), "pbf_profile_read");
  float ms = 0.f;
  PBF_CUDA(cudaEventElapsedTime(&ms, s->ev[kEvStart], s->ev[kEvGrid]), "pbf_profile_read");
  out->grid_ms = ms;
  PBF_CUDA(cudaEventElapsedTime(&ms, s->ev[kEvGrid], s->ev[kEvReorder]), "pbf_profile_read");
  out->reorder_ms = ms;
  for (int it = 0; it < s->prof_iters; ++it) {
    PBF_CUDA(cudaEventElapsedTime(&ms, s->ev_it[3 * it], s->ev_it[3 * it + 1]), "pbf_profile_read");
    out->lambda_ms += ms;
    PBF_CUDA(cudaEventElapsedTime(&ms, s->ev_it[3 * it + 1], s->ev_it[3 * it + 2]), "pbf_profile_read");
    out->delta_p_ms += ms;
  }
  PBF_CUDA(cudaEventElapsedTime(&ms, s->ev[kEvXsphStart], s->ev[kEvEnd]), "pbf_profile_read");
  out->xsph_ms = ms;
  PBF_CUDA(cudaEventElapsedTime(&ms, s->ev[kEvStart], s->ev[kEvEnd]), "pbf_profile_read");
  out->total_ms = ms;
  out->iterations = s->prof_iters;
  return PBF_OK;
}

pbf_status pbf_get_density(const pbf_solver* s, float* rho, int n, void* stream) {
  if (!s || !rho) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
  if (s->last_n == 0) return fail(PBF_ERR_NOT_READY, "no step has run");
  if (n < 0 || n > s->last_n) return fail(PBF_ERR_INVALID_ARG, "n outside [0, %d]", s->last_n);
  PBF_CUDA(cudaMemcpyAsync(rho, s->sol.rho, sizeof(float) * n, cudaMemcpyDeviceToDevice,
                           (cudaStream_t)stream),
           "pbf_get_density");
  return PBF_OK;
}

pbf_status pbf_build_grid(pbf_solver* s, const void* xstar, int n, uint32_t* keys, uint32_t* perm,
                          uint32_t* start, uint32_t* end, int dims[3], void* stream) {
  const pbf::NvtxRange range("pbf_build_grid");
  if (!s || !dims) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
  long long cells;
  pbf_status st = grid_dims(s->ulim, s->llim, s->params.h, dims, &cells);
  if (st != PBF_OK) return st;
  if (!start && !end && !keys && !perm) return PBF_OK;  // dims query
  if (cells > s->max_cells) return fail(PBF_ERR_CAPACITY, "box needs %lld cells", cells);
  if (n < 0 || n > s->max_particles) return fail(PBF_ERR_CAPACITY, "n outside [0, max_particles]");
  if (!start || !end) return fail(PBF_ERR_INVALID_ARG, "start/end are NULL");
  if (n > 0 && (!xstar || !keys || !perm)) return fail(PBF_ERR_INVALID_ARG, "NULL buffer");
  const pbf::StepConsts c = make_consts(s->params, s->ulim, s->llim, dims, s->num_sms);
  cudaStream_t st_ = (cudaStream_t)stream;
  if (n == 0) {
    PBF_CUDA(cudaMemsetAsync(start, 0, sizeof(uint32_t) * cells, st_), "pbf_build_grid");
    PBF_CUDA(cudaMemsetAsync(end, 0, sizeof(uint32_t) * cells, st_), "pbf_build_grid");
    return PBF_OK;
  }
  const uint32_t* p = nullptr;
  PBF_CUDA(pbf::build_grid(c, pbf::Geometry{nullptr, nullptr}, nullptr, nullptr, (const float4*)xstar, n,
                           s->grid, &p, keys, st_),
           "pbf_build_grid");
  PBF_CUDA(cudaMemcpyAsync(perm, p, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st_),
           "pbf_build_grid: perm");
  PBF_CUDA(pbf::export_ranges(c, s->grid.cell_start, start, end, st_), "pbf_build_grid: ranges");
  return PBF_OK;
}

}  // extern "C"

// ---- helpers for other translation units of the library ---------------------------

namespace pbf {

pbf_status set_error(pbf_status s, const char* msg) { return fail(s, "%s", msg); }

pbf_status set_cuda_error(cudaError_t e, const char* what) { return cuda_fail(e, what); }

pbf_status validate_step_setup(const pbf_params* params, const float ulim[3], const float llim[3],
                               long long max_cells, StepConsts* out) {
  pbf_status st = check_params(params);
  if (st != PBF_OK) return st;
  if (!ulim || !llim) return fail(PBF_ERR_INVALID_ARG, "limits are NULL");
  int dims[3];
  long long cells;
  if ((st = grid_dims(ulim, llim, params->h, dims, &cells)) != PBF_OK) return st;
  if (cells > max_cells)
    return fail(PBF_ERR_CAPACITY, "box needs %lld cells, the limit is %lld", cells, max_cells);
  *out = make_consts(*params, ulim, llim, dims, current_sms());
  return PBF_OK;
}

pbf_status validate_step_buffers(const void* pos, const void* npos, const void* vel, const void* nvel,
                                 const void* iid) {
  const void* bufs[5] = {pos, npos, vel, nvel, iid};
  for (int a = 0; a < 5; ++a) {
    if (!bufs[a]) return fail(PBF_ERR_INVALID_ARG, "buffer %d is NULL", a);
    if (!aligned16(bufs[a]) && a < 4) return fail(PBF_ERR_INVALID_ARG, "buffer %d not 16-byte aligned", a);
    for (int b = 0; b < a; ++b)
      if (bufs[a] == bufs[b]) return fail(PBF_ERR_INVALID_ARG, "buffers %d and %d alias", b, a);
  }
  return PBF_OK;
}

}  // namespace pbf

// ---- batched ensemble ---------------------------------------------------------------

struct pbf_batch {
  pbf_params params;
  int nscenes;
  int n;          // particles of all scenes
  int max_cells;  // cells reserved for all scenes together
  int num_sms;
  int device;
  int last_n;
  std::vector<float> ulim, llim;  // 3 * nscenes
  std::vector<int> counts;
  std::vector<pbf::SceneGeom> geom;  // host copy of the scene table
  pbf::SceneGeom* d_geom;
  uint16_t* d_sid;
  pbf::GridScratch grid;
  pbf::SolverScratch sol;
  bool use_graph;
  cudaStream_t cap_stream;
  cudaGraphExec_t exec;
  GraphCache cache;
  std::vector<pbf::SceneGeom> geom_dev;  // the scene table as last uploaded
  int tune_window = 0;  // dense-kernel, order and staging choices (pbf_batch_autotune); 0 / -1: the defaults
  int tune_all = -1;
  int tune_order = -1;
  int tune_stage_sparse = -1;
  int tune_stage_dense = -1;
  int tune_queue_sparse = 0;
  int tune_queue_dense = 0;
  int tune_split = 0;
  int tune_interleave = -1;
};

namespace {

void batch_free(pbf_batch* b) {
  void* ptrs[] = {b->grid.keys_a, b->grid.keys_b, b->grid.vals_a, b->grid.vals_b,
                  b->grid.cell_count, b->grid.cell_start, b->grid.radix_counts,
                  b->grid.scan_partials, b->sol.xs, b->sol.xa, b->sol.xb, b->sol.iid_s,
                  b->sol.lambda, b->sol.rho, b->sol.flags, b->sol.dense, b->sol.masks,
                  b->sol.cell_flags, b->sol.grp_cell, b->sol.grp_off, b->sol.grp_n, b->sol.grp_rep, b->sol.grp_cnt,
                  b->sol.grp_pos, b->sol.grp_sum, b->sol.grp_aux, b->sol.grp_id, b->sol.grp_hash,
                  b->sol.grp_max, b->sol.grp_acc, b->sol.grp_list, b->sol.grp_list_n, b->sol.grp_done,
                  b->sol.grp_zero, b->sol.grp_item_off, b->sol.grp_item_slot, b->sol.work_list,
                  b->sol.work_follow, b->sol.work_blocks, b->sol.bcnt, b->sol.bstart, b->sol.bent,
                  b->sol.bucket, b->sol.bpart, b->d_geom, b->d_sid};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->cache.clear();
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
}

// Rebuilds the host scene table from the current limits; returns the total cells.
pbf_status batch_tables(pbf_batch* b, long long* total_cells) {
  long long base = 0;
  for (int k = 0; k < b->nscenes; ++k) {
    int dims[3];
    long long cells;
    pbf_status st = grid_dims(&b->ulim[3 * k], &b->llim[3 * k], b->params.h, dims, &cells);
    if (st != PBF_OK) return st;
    if (base + cells > 2147483647LL) return fail(PBF_ERR_CAPACITY, "too many cells");
    b->geom[k] = make_geom(b->params, &b->ulim[3 * k], &b->llim[3 * k], dims, (int)base);
    base += cells;
  }
  *total_cells = base;
  return PBF_OK;
}

}  // namespace

extern "C" {

pbf_status pbf_batch_create(const pbf_params* params, int nscenes, const float* ulim, const float* llim,
                            const int* counts, pbf_batch** out) {
  g_err[0] = 0;
  if (!out) return fail(PBF_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  if (!ulim || !llim || !counts) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
  if (nscenes < 1 || nscenes > 65535) return fail(PBF_ERR_INVALID_ARG, "nscenes must be in [1, 65535]");
  pbf_status st = check_params(params);
  if (st != PBF_OK) return st;
  long long n = 0;
  for (int k = 0; k < nscenes; ++k) {
    if (counts[k] < 0) return fail(PBF_ERR_INVALID_ARG, "counts[%d] < 0", k);
    n += counts[k];
  }
  if (n > PBF_MAX_PARTICLES) return fail(PBF_ERR_CAPACITY, "%lld particles exceed %d", n, PBF_MAX_PARTICLES);
  pbf_batch* b = new (std::nothrow) pbf_batch();
  if (!b) return fail(PBF_ERR_CAPACITY, "host allocation failed");
  b->params = *params;
  b->nscenes = nscenes;
  b->n = (int)n;
  b->ulim.assign(ulim, ulim + 3 * nscenes);
  b->llim.assign(llim, llim + 3 * nscenes);
  b->counts.assign(counts, counts + nscenes);
  b->geom.resize(nscenes);
  long long cells;
  if ((st = batch_tables(b, &cells)) != PBF_OK) {
    delete b;
    return st;
  }
  long long max_cells = 4 * cells;
  const long long scan_cap = (long long)pbf::kScanTile * pbf::kMaxScanPartials - 1;
  if (max_cells > scan_cap) max_cells = cells;
  if (max_cells > scan_cap) {
    delete b;
    return fail(PBF_ERR_CAPACITY, "scenes need %lld cells, limit %lld", cells, scan_cap);
  }
  b->max_cells = (int)max_cells;
  cudaError_t e = cudaGetDevice(&b->device);
  const size_t np = (size_t)(n > 0 ? n : 1), nc = (size_t)max_cells + 1;
  if (e == cudaSuccess) e = alloc(&b->grid.keys_a, np);
  if (e == cudaSuccess) e = alloc(&b->grid.keys_b, np);
  if (e == cudaSuccess) e = alloc(&b->grid.vals_a, np);
  if (e == cudaSuccess) e = alloc(&b->grid.vals_b, np);
  if (e == cudaSuccess) e = alloc(&b->grid.cell_count, nc);
  if (e == cudaSuccess) e = alloc(&b->grid.cell_start, nc);
  if (e == cudaSuccess) e = alloc(&b->grid.radix_counts, pbf::radix_counts_len((int)np));
  if (e == cudaSuccess) e = alloc(&b->grid.scan_partials, (size_t)pbf::kMaxScanPartials);
  if (e == cudaSuccess) e = alloc(&b->sol.xs, np);
  if (e == cudaSuccess) e = alloc(&b->sol.xa, np);
  if (e == cudaSuccess) e = alloc(&b->sol.xb, np);
  if (e == cudaSuccess) e = alloc(&b->sol.iid_s, np);
  if (e == cudaSuccess) e = alloc(&b->sol.lambda, np);
  if (e == cudaSuccess) e = alloc(&b->sol.rho, np);
  if (e == cudaSuccess) e = alloc(&b->sol.flags, (size_t)pbf::kFlagWords);
  if (e == cudaSuccess) e = cudaMemset(b->sol.flags, 0, sizeof(uint32_t) * pbf::kFlagWords);
  if (e == cudaSuccess) e = alloc(&b->sol.dense, pbf::dense_list_len((int)np));
  if (e == cudaSuccess) e = alloc(&b->sol.masks, (size_t)pbf::kMaskWords * np);
  b->sol.mask_stride = (int)np;
  if (e == cudaSuccess) e = alloc(&b->sol.cell_flags, nc);
  if (e == cudaSuccess) e = alloc_groups(b->sol, (int)np);
  if (e == cudaSuccess) e = alloc_buckets(b->sol, np, nc);
  if (e == cudaSuccess) e = alloc(&b->d_geom, (size_t)nscenes);
  if (e == cudaSuccess) e = alloc(&b->d_sid, np);
  if (e == cudaSuccess) {
    std::vector<uint16_t> sid(np, 0);
    size_t k = 0;
    for (int sc = 0; sc < nscenes; ++sc)
      for (int j = 0; j < counts[sc]; ++j) sid[k++] = (uint16_t)sc;
    e = cudaMemcpy(b->d_sid, sid.data(), sizeof(uint16_t) * np, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = pbf::set_pass_kernel_attributes();
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    batch_free(b);
    delete b;
    cudaGetLastError();
    return cuda_fail(e, "pbf_batch_create");
  }
  b->num_sms = current_sms();
  b->use_graph = true;
  *out = b;
  return PBF_OK;
}

pbf_status pbf_batch_destroy(pbf_batch* b) {
  if (!b) return PBF_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != b->device) cudaSetDevice(b->device);
  batch_free(b);
  if (prev >= 0 && prev != b->device) cudaSetDevice(prev);
  delete b;
  return PBF_OK;
}

pbf_status pbf_batch_set_limits(pbf_batch* b, int scene, const float ulim[3], const float llim[3]) {
  if (!b || !ulim || !llim) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
  if (scene < 0 || scene >= b->nscenes) return fail(PBF_ERR_INVALID_ARG, "scene %d out of range", scene);
  const std::vector<float> old_u(b->ulim.begin() + 3 * scene, b->ulim.begin() + 3 * scene + 3);
  const std::vector<float> old_l(b->llim.begin() + 3 * scene, b->llim.begin() + 3 * scene + 3);
  std::memcpy(&b->ulim[3 * scene], ulim, sizeof(float) * 3);
  std::memcpy(&b->llim[3 * scene], llim, sizeof(float) * 3);
  long long cells;
  pbf_status st = batch_tables(b, &cells);
  if (st == PBF_OK && cells > b->max_cells)
    st = fail(PBF_ERR_CAPACITY, "scenes need %lld cells, %d reserved", cells, b->max_cells);
  if (st != PBF_OK) {
    std::memcpy(&b->ulim[3 * scene], old_u.data(), sizeof(float) * 3);
    std::memcpy(&b->llim[3 * scene], old_l.data(), sizeof(float) * 3);
    long long ignored;
    batch_tables(b, &ignored);
  }
  return st;
}

pbf_status pbf_batch_step(pbf_batch* b, void* pos, void* npos, void* vel, void* nvel, uint32_t* iid,
                          void* stream) {
  const pbf::NvtxRange range("pbf_batch_step");
  if (!b) return fail(PBF_ERR_INVALID_ARG, "batch is NULL");
  const int n = b->n;
  if (n == 0) return PBF_OK;
  if (pbf::validate_step_buffers(pos, npos, vel, nvel, iid) != PBF_OK) return PBF_ERR_INVALID_ARG;
  long long cells;
  pbf_status st = batch_tables(b, &cells);
  if (st != PBF_OK) return st;
  if (cells > b->max_cells) return fail(PBF_ERR_CAPACITY, "scenes need %lld cells", cells);
  cudaStream_t st_ = (cudaStream_t)stream;
  // the scene table stays on the device; when a wall moved it goes in stream
  // order ahead of the step (pageable source: staged before the call returns,
  // so the host copy may change afterwards)
  const size_t table = sizeof(pbf::SceneGeom) * b->nscenes;
  if (b->geom_dev.size() != b->geom.size() || std::memcmp(b->geom_dev.data(), b->geom.data(), table) != 0) {
    PBF_CUDA(cudaMemcpyAsync(b->d_geom, b->geom.data(), table, cudaMemcpyHostToDevice, st_),
             "pbf_batch_step: scene table");
    b->geom_dev = b->geom;
  }
  StepPlan P;
  int unit_dims[3] = {1, 1, 1};
  P.c = make_consts(b->params, &b->ulim[0], &b->llim[0], unit_dims, b->num_sms);
  P.c.cells = (int)cells;
  if (b->tune_window > 0) P.c.dense_window = b->tune_window;
  P.c.dense_all = b->tune_all;
  if (b->tune_order >= 0) P.c.order = b->tune_order;
  if (b->tune_stage_sparse >= 0) P.c.stage_sparse = b->tune_stage_sparse;
  if (b->tune_stage_dense >= 0) P.c.stage_dense = b->tune_stage_dense;
  if (b->tune_queue_sparse > 0) P.c.queue_sparse = b->tune_queue_sparse;
  if (b->tune_queue_dense > 0) P.c.queue_dense = b->tune_queue_dense;
  if (b->tune_split > 0) P.c.dense_split = b->tune_split;
  if (b->tune_interleave >= 0) P.c.dense_interleave = b->tune_interleave;
  P.G = pbf::Geometry{b->d_geom, b->d_sid};
  P.grid = &b->grid;
  P.sol = &b->sol;
  P.niter = b->params.niter;
  P.ev = nullptr;
  P.ev_it = nullptr;
  P.tape = nullptr;
  P.tape_x = P.tape_l = P.tape_xs = P.tape_rho = P.tape_perm = P.tape_cs = 0;
  P.tape_stride = 0;
  P.perm_out = nullptr;
  st = b->use_graph ? launch_cached(P, b->cache, b->cap_stream, pos, npos, vel, nvel, iid, n, st_)
                    : enqueue_step(P, pos, npos, vel, nvel, iid, n, st_);
  if (st != PBF_OK) return st;
  b->last_n = n;
  return PBF_OK;
}

pbf_status pbf_batch_get_density(const pbf_batch* b, float* rho, void* stream) {
  if (!b || !rho) return fail(PBF_ERR_INVALID_ARG, "NULL argument");
  if (b->last_n == 0) return fail(PBF_ERR_NOT_READY, "no step has run");
  PBF_CUDA(cudaMemcpyAsync(rho, b->sol.rho, sizeof(float) * b->n, cudaMemcpyDeviceToDevice,
                           (cudaStream_t)stream),
           "pbf_batch_get_density");
  return PBF_OK;
}

pbf_status pbf_batch_use_graphs(pbf_batch* b, int on) {
  if (!b) return fail(PBF_ERR_INVALID_ARG, "batch is NULL");
  b->use_graph = on != 0;
  return PBF_OK;
}

}  // extern "C"

// ---- density grid (the inverse problem's loss) ---------------------------------------

namespace {

// lo < hi finite, h > 0 finite, dims >= 1 with fewer than 2^31 nodes (the
// kernels index nodes with int).
pbf_status check_lattice(const float lo[3], const float hi[3], const int dims[3], float h) {
  if (!(h > 0.f) || !std::isfinite(h)) return fail(PBF_ERR_INVALID_ARG, "h must be finite and > 0");
  for (int a = 0; a < 3; ++a)
    if (!(lo[a] < hi[a]) || !std::isfinite(lo[a]) || !std::isfinite(hi[a]))
      return fail(PBF_ERR_INVALID_ARG, "lo must be below hi, both finite");
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return fail(PBF_ERR_INVALID_ARG, "dims must be >= 1");
  if ((long long)dims[0] * dims[1] * dims[2] > 2147483647LL)
    return fail(PBF_ERR_INVALID_ARG, "dims hold 2^31 or more nodes");
  return PBF_OK;
}

}  // namespace

extern "C" {

pbf_status pbf_density_grid(const void* pos, int n, const float lo[3], const float hi[3],
                            const int dims[3], float h, float* grid, void* stream) {
  const pbf::NvtxRange range("pbf_density_grid");
  if ((!pos && n > 0) || !lo || !hi || !dims || !grid || n < 0)
    return fail(PBF_ERR_INVALID_ARG, "NULL argument or n < 0");
  if (pbf_status st = check_lattice(lo, hi, dims, h); st != PBF_OK) return st;
  PBF_CUDA(pbf::density_grid((const float4*)pos, n, lo, hi, dims, h, grid, (cudaStream_t)stream),
           "pbf_density_grid");
  return PBF_OK;
}

pbf_status pbf_density_grid_backward(const void* pos, int n, const float lo[3], const float hi[3],
                                     const int dims[3], float h, const float* g_grid, void* g_pos,
                                     void* stream) {
  const pbf::NvtxRange range("pbf_density_grid_backward");
  if ((!pos && n > 0) || !lo || !hi || !dims || !g_grid || (!g_pos && n > 0) || n < 0)
    return fail(PBF_ERR_INVALID_ARG, "NULL argument or n < 0");
  if (pbf_status st = check_lattice(lo, hi, dims, h); st != PBF_OK) return st;
  PBF_CUDA(pbf::density_grid_backward((const float4*)pos, n, lo, hi, dims, h, g_grid, (float4*)g_pos,
                                      (cudaStream_t)stream),
           "pbf_density_grid_backward");
  return PBF_OK;
}

}  // extern "C"

// ---- autotuning ------------------------------------------------------------------------

namespace {

// Candidate choices timed by pbf_autotune / pbf_batch_autotune.
constexpr int kTuneWindows[] = {64, 128, 256, 512, 1024, 2048};
constexpr int kTuneSplits[] = {1, 2, 4, 8};
constexpr int kTuneInterleave[] = {0, 1};
constexpr int kTuneQueueSparse[] = {1, 10, 16};
constexpr int kTuneQueueDense[] = {1, 4, 8};
constexpr int kTuneStageSparse[] = {0, 1024, 2048};
constexpr int kTuneStageDense[] = {0, 1536, 3072};

// One configuration of the neighbour passes (the fields of pbf_tuning that
// pbf_autotune times).
struct TuneChoice {
  int window, all, order, split, queue_sparse, queue_dense, stage_sparse, stage_dense, interleave;
  bool operator==(const TuneChoice& o) const {
    return window == o.window && all == o.all && order == o.order && split == o.split &&
           queue_sparse == o.queue_sparse && queue_dense == o.queue_dense && stage_sparse == o.stage_sparse &&
           stage_dense == o.stage_dense && interleave == o.interleave;
  }
};

TuneChoice default_choice(int n) {
  return TuneChoice{pbf::kDefaultDenseWindow, n < pbf::kDenseAllBelow ? 1 : 0, 1, pbf::kDefaultDenseSplit,
                    pbf::kDefaultQueueSparse, pbf::kDefaultQueueDense, pbf::kDefaultStageSparse,
                    pbf::kDefaultStageDense, pbf::kDefaultDenseInterleave};
}

// The tuning fields a solver or batch keeps (0 / -1: the defaults).
struct TuneState {
  int window = 0, all = -1, order = -1, split = 0, queue_sparse = 0, queue_dense = 0, stage_sparse = -1,
      stage_dense = -1, interleave = -1;
};

template <class T>
TuneState tune_state(const T* h) {
  return TuneState{h->tune_window,       h->tune_all,         h->tune_order,
                   h->tune_split,        h->tune_queue_sparse, h->tune_queue_dense,
                   h->tune_stage_sparse, h->tune_stage_dense,  h->tune_interleave};
}

template <class T>
void set_tune_state(T* h, const TuneState& t) {
  h->tune_window = t.window;
  h->tune_all = t.all;
  h->tune_order = t.order;
  h->tune_split = t.split;
  h->tune_queue_sparse = t.queue_sparse;
  h->tune_queue_dense = t.queue_dense;
  h->tune_stage_sparse = t.stage_sparse;
  h->tune_stage_dense = t.stage_dense;
  h->tune_interleave = t.interleave;
}

TuneState state_of(const TuneChoice& c) {
  return TuneState{c.window,       c.all,          c.order,        c.split,     c.queue_sparse,
                   c.queue_dense,  c.stage_sparse, c.stage_dense,  c.interleave};
}

// pbf_tuning fields of a tune state (defaults resolved).
void fill_tuning(const TuneState& t, pbf_tuning* out) {
  out->dense_window = t.window > 0 ? t.window : pbf::kDefaultDenseWindow;
  out->dense_all = t.all;
  out->order = t.order >= 0 ? t.order : 1;
  out->dense_split = t.split > 0 ? t.split : pbf::kDefaultDenseSplit;
  out->queue_sparse = t.queue_sparse > 0 ? t.queue_sparse : pbf::kDefaultQueueSparse;
  out->queue_dense = t.queue_dense > 0 ? t.queue_dense : pbf::kDefaultQueueDense;
  out->stage_sparse = t.stage_sparse >= 0 ? t.stage_sparse : pbf::kDefaultStageSparse;
  out->stage_dense = t.stage_dense >= 0 ? t.stage_dense : pbf::kDefaultStageDense;
  out->dense_interleave = t.interleave >= 0 ? t.interleave : pbf::kDefaultDenseInterleave;
}

// Runs `steps` steps per candidate on copies of (pos, vel, iid) through
// step(choice, bufs...) and returns the fastest choice: first over the
// window, dense and order choices with the other fields at their defaults,
// then, from the best so far, one field at a time: the dense split, the
// sparse and dense hit queues, the sparse and dense stages.
template <class Step>
pbf_status autotune(int n, const void* pos, const void* vel, const uint32_t* iid, int steps, cudaStream_t st,
                    Step step, pbf_tuning* out) {
  if (!pos || !vel || !iid || !out || n <= 0 || steps < 1)
    return fail(PBF_ERR_INVALID_ARG, "NULL argument, n <= 0 or steps < 1");
  float4 *p[2] = {nullptr, nullptr}, *v[2] = {nullptr, nullptr};
  uint32_t* id = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = alloc(&p[0], (size_t)n);
  if (e == cudaSuccess) e = alloc(&p[1], (size_t)n);
  if (e == cudaSuccess) e = alloc(&v[0], (size_t)n);
  if (e == cudaSuccess) e = alloc(&v[1], (size_t)n);
  if (e == cudaSuccess) e = alloc(&id, (size_t)n);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  pbf_status result = PBF_OK;
  // ms per step of one choice (negative: a failure, recorded in e / result)
  auto time_choice = [&](const TuneChoice& ch) -> float {
    if (e != cudaSuccess || result != PBF_OK) return -1.f;
    e = cudaMemcpyAsync(p[0], pos, sizeof(float4) * n, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v[0], vel, sizeof(float4) * n, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(id, iid, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return -1.f;
    int cur = 0;
    float ms = 0.f;
    for (int k = -1; k < steps && result == PBF_OK; ++k) {  // one untimed step first
      if (k == 0) e = cudaEventRecord(e0, st);
      if (e != cudaSuccess) return -1.f;
      result = step(ch, p[cur], p[1 - cur], v[cur], v[1 - cur], id, st);
      cur = 1 - cur;
    }
    if (result != PBF_OK) return -1.f;
    e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    return e == cudaSuccess ? ms / (float)steps : -1.f;
  };
  const TuneChoice def = default_choice(n);
  float best = -1.f, def_ms = -1.f;
  TuneChoice best_ch = def;
  best_ch.all = -1;
  auto consider = [&](const TuneChoice& ch) {
    const float ms = time_choice(ch);
    if (ms < 0.f) return;
    if (ch == def) def_ms = ms;
    if (best < 0.f || ms < best) {
      best = ms;
      best_ch = ch;
    }
  };
  for (int ord = 1; ord >= 0; --ord)
    for (int all = 0; all <= 1; ++all)
      for (int w : kTuneWindows) {
        if (all == 1 && w != pbf::kDefaultDenseWindow) continue;  // the window plays no part then
        TuneChoice ch = def;
        ch.window = w, ch.all = all, ch.order = ord;
        consider(ch);
      }
  // one field at a time from the best so far (a field already at a
  // candidate's value is not timed again)
  auto sweep = [&](int TuneChoice::*field, const int* vals, int count) {
    const TuneChoice base = best_ch;
    for (int k = 0; k < count; ++k) {
      if (vals[k] == base.*field) continue;
      TuneChoice ch = base;
      ch.*field = vals[k];
      consider(ch);
    }
  };
  sweep(&TuneChoice::split, kTuneSplits, 4);
  if (best_ch.split > 1) sweep(&TuneChoice::interleave, kTuneInterleave, 2);
  if (!best_ch.all) sweep(&TuneChoice::queue_sparse, kTuneQueueSparse, 3);
  sweep(&TuneChoice::queue_dense, kTuneQueueDense, 3);
  if (!best_ch.all) sweep(&TuneChoice::stage_sparse, kTuneStageSparse, 3);
  sweep(&TuneChoice::stage_dense, kTuneStageDense, 3);
  for (void* q : {(void*)p[0], (void*)p[1], (void*)v[0], (void*)v[1], (void*)id})
    if (q) cudaFree(q);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (result != PBF_OK) return result;
  if (e != cudaSuccess) return cuda_fail(e, "pbf_autotune");
  fill_tuning(state_of(best_ch), out);
  out->dense_all = best_ch.all;
  out->bwd_lanes = 0;
  out->ms_per_step = best;
  out->ms_default = def_ms;
  return PBF_OK;
}

pbf_status check_tuning(const pbf_tuning* t) {
  if (t->dense_window != 0 && t->dense_window < 32)
    return fail(PBF_ERR_INVALID_ARG, "dense_window must be 0 (default) or >= 32 (got %d)", t->dense_window);
  if (t->dense_all < -1 || t->dense_all > 1)
    return fail(PBF_ERR_INVALID_ARG, "dense_all must be -1, 0 or 1 (got %d)", t->dense_all);
  if (t->order < -1 || t->order > 1)
    return fail(PBF_ERR_INVALID_ARG, "order must be -1, 0 or 1 (got %d)", t->order);
  if (t->bwd_lanes != 0 && t->bwd_lanes != 8 && t->bwd_lanes != 16 && t->bwd_lanes != 32)
    return fail(PBF_ERR_INVALID_ARG, "bwd_lanes must be 0, 8, 16 or 32 (got %d)", t->bwd_lanes);
  if (t->stage_sparse < -1 || t->stage_sparse > pbf::kStageMax || t->stage_dense < -1 ||
      t->stage_dense > pbf::kStageMax)
    return fail(PBF_ERR_INVALID_ARG, "stage_sparse / stage_dense must be -1 to %d (got %d / %d)", pbf::kStageMax,
                t->stage_sparse, t->stage_dense);
  if (t->queue_sparse < 0 || t->queue_sparse > pbf::kMaxQueueSparse || t->queue_dense < 0 ||
      t->queue_dense > pbf::kMaxQueueDense)
    return fail(PBF_ERR_INVALID_ARG, "queue_sparse must be 0 to %d and queue_dense 0 to %d (got %d / %d)",
                pbf::kMaxQueueSparse, pbf::kMaxQueueDense, t->queue_sparse, t->queue_dense);
  if (t->dense_split != 0 && t->dense_split != 1 && t->dense_split != 2 && t->dense_split != 4 &&
      t->dense_split != 8)
    return fail(PBF_ERR_INVALID_ARG, "dense_split must be 0, 1, 2, 4 or 8 (got %d)", t->dense_split);
  if (t->dense_interleave < -1 || t->dense_interleave > 1)
    return fail(PBF_ERR_INVALID_ARG, "dense_interleave must be -1, 0 or 1 (got %d)", t->dense_interleave);
  return PBF_OK;
}

TuneState state_of(const pbf_tuning* t) {
  return TuneState{t->dense_window, t->dense_all,    t->order,        t->dense_split,     t->queue_sparse,
                   t->queue_dense,  t->stage_sparse, t->stage_dense,  t->dense_interleave};
}

}  // namespace

extern "C" {

pbf_status pbf_autotune(pbf_solver* s, const void* pos, const void* vel, const uint32_t* iid, int n, int steps,
                        pbf_tuning* out, void* stream) {
  const pbf::NvtxRange range("pbf_autotune");
  if (!s) return fail(PBF_ERR_INVALID_ARG, "solver is NULL");
  if (n > s->max_particles) return fail(PBF_ERR_CAPACITY, "n = %d exceeds max_particles = %d", n, s->max_particles);
  const int depth = s->tape_depth, top = s->tape_top;
  s->tape_depth = 0;  // the trial steps are not taped
  const TuneState keep = tune_state(s);
  const pbf_status st = autotune(
      n, pos, vel, iid, steps, (cudaStream_t)stream,
      [&](const TuneChoice& ch, float4* p, float4* np, float4* v, float4* nv, uint32_t* id, cudaStream_t strm) {
        set_tune_state(s, state_of(ch));
        return pbf_step(s, p, np, v, nv, id, n, strm);
      },
      out);
  s->tape_depth = depth;
  s->tape_top = top;
  if (st != PBF_OK) {
    set_tune_state(s, keep);
    return st;
  }
  set_tune_state(s, state_of(out));
  out->bwd_lanes = s->tune_bwd_lanes > 0 ? s->tune_bwd_lanes : 32;  // not timed: kept
  return PBF_OK;
}

pbf_status pbf_set_tuning(pbf_solver* s, const pbf_tuning* t) {
  if (!s || !t) return fail(PBF_ERR_INVALID_ARG, "solver or tuning is NULL");
  if (pbf_status st = check_tuning(t); st != PBF_OK) return st;
  set_tune_state(s, state_of(t));
  s->tune_bwd_lanes = t->bwd_lanes;
  return PBF_OK;
}

pbf_status pbf_get_tuning(const pbf_solver* s, pbf_tuning* t) {
  if (!s || !t) return fail(PBF_ERR_INVALID_ARG, "solver or tuning is NULL");
  fill_tuning(tune_state(s), t);
  t->bwd_lanes = s->tune_bwd_lanes > 0 ? s->tune_bwd_lanes : 32;
  t->ms_per_step = 0.f;
  t->ms_default = 0.f;
  return PBF_OK;
}

pbf_status pbf_batch_set_tuning(pbf_batch* b, const pbf_tuning* t) {
  if (!b || !t) return fail(PBF_ERR_INVALID_ARG, "batch or tuning is NULL");
  if (pbf_status st = check_tuning(t); st != PBF_OK) return st;
  set_tune_state(b, state_of(t));
  return PBF_OK;
}

pbf_status pbf_batch_get_tuning(const pbf_batch* b, pbf_tuning* t) {
  if (!b || !t) return fail(PBF_ERR_INVALID_ARG, "batch or tuning is NULL");
  fill_tuning(tune_state(b), t);
  t->bwd_lanes = 0;
  t->ms_per_step = 0.f;
  t->ms_default = 0.f;
  return PBF_OK;
}

pbf_status pbf_check_device(pbf_solver* s, void* stream) {
  if (!s) return fail(PBF_ERR_INVALID_ARG, "solver is NULL");
  return check_device_word(s->sol.flags + pbf::kErrorWord, (cudaStream_t)stream, "pbf_check_device");
}

pbf_status pbf_batch_check_device(pbf_batch* b, void* stream) {
  if (!b) return fail(PBF_ERR_INVALID_ARG, "batch is NULL");
  return check_device_word(b->sol.flags + pbf::kErrorWord, (cudaStream_t)stream, "pbf_batch_check_device");
}

pbf_status pbf_batch_autotune(pbf_batch* b, const void* pos, const void* vel, const uint32_t* iid, int steps,
                              pbf_tuning* out, void* stream) {
  const pbf::NvtxRange range("pbf_batch_autotune");
  if (!b) return fail(PBF_ERR_INVALID_ARG, "batch is NULL");
  const TuneState keep = tune_state(b);
  const pbf_status st = autotune(
      b->n, pos, vel, iid, steps, (cudaStream_t)stream,
      [&](const TuneChoice& ch, float4* p, float4* np, float4* v, float4* nv, uint32_t* id, cudaStream_t strm) {
        set_tune_state(b, state_of(ch));
        return pbf_batch_step(b, p, np, v, nv, id, strm);
      },
      out);
  if (st != PBF_OK) {
    set_tune_state(b, keep);
    return st;
  }
  set_tune_state(b, state_of(out));
  return PBF_OK;
}

}  // extern "C"
