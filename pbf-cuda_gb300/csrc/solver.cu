// solver.cu — the per-particle passes of one step, in cell order:
//   reorder   gather pos/vel/iid by the sorted permutation, recompute x*
//   lambda    density rho_i and lambda_i        computeLambda  (fluids/Simulator_kernel.cuh:52-129)
//   delta_p   s_corr, clamp, wall clamp         computetpos    (fluids/Simulator_kernel.cuh:131-194)
//             the last iteration also writes v = (x_final - x) / dt and the
//             caller's permuted pos / iid       h_updateVelocity (fluids/Simulator.cu:127-137)
//   xsph      XSPH viscosity                    computeXSPH    (fluids/Simulator_kernel.cuh:196-239)
//
// Every pass is gather-only (no atomics on results, no cross-thread writes),
// so results are deterministic.  Neighbour semantics follow the reference
// exactly: the grid is built once per step from x*, every pass looks up the
// 3x3x3 cells around cell(current x_i) in that (stale) grid.  For each
// (dx, dy) column the three z-consecutive cells are adjacent in cell order,
// so the window is 9 runs of sorted slots, visited in the reference's order
// (dx outer, dy inner, slots ascending; fluids/Simulator_kernel.cuh:78-88).
// Jacobi iterations ping-pong between two position buffers instead of the
// reference's tpos -> npos copy (fluids/Simulator.cu:247-248).
//
// Each pass is two kernels.  The sparse kernel gives every particle one
// thread and walks its window in a compact loop (fluid at rest: ~200
// candidates; a window whose grouped cells -- see pbf_internal.cuh -- bring
// it under dense_window entries is walked group by group).  A particle whose
// window still exceeds dense_window entries (particles piled into a few
// cells) instead appends itself to a dense list; the persistent dense kernel
// takes the list in batches of 32 particles from a counter, splits each
// batch's windows over dense_split warps (each walking one part of every
// lane's window) and adds the parts' partial sums in part order in shared
// memory.  Steps of fewer than kDenseAllBelow particles send every particle
// to the dense kernel by default (one thread per particle would leave most
// SMs idle).  Both orders are fixed, so results stay deterministic; they
// differ from the reference's sequential sums only by rounding.  The walks
// test chunks of 32 candidates into hit masks and run the pair body on the
// hits, optionally through a hit queue; each kernel has a variant that
// stages its block's column runs in shared memory by bulk asynchronous
// copies.  Neither changes any sum.
//
// Particles piled onto one position (a grouped cell's position group) have
// bitwise the same window, position and, within a step, lambda: their lambda
// and delta_p results are equal.  When a step has grouped cells, each lambda
// pass first builds a work list (k_work_mark, k_work_list: one particle per
// position group plus every particle outside the groups, in cell order), the
// two passes run on that list, and k_follow copies each group's results to
// its other members.  With no grouped cell the list is the identity and those
// kernels return at once.
//
// IEEE semantics follow the reference's: its kernels evaluate every
// candidate of the window, so a NaN distance (from a NaN position) poisons
// the sums, a non-finite lambda_j poisons delta_p through a zero gradient,
// and 0 * v / (rho_i + rho_j) is NaN when both densities are zero.  Here the
// candidate test is written NaN-inclusively (!(r2 >= h2), as the reference's
// `if (r2 >= h2) return 0`), and the two poisoning rules that need every
// candidate's lambda / density / velocity run only when a per-step flag says
// such a value exists (StepFlag); otherwise candidates outside the cutoff
// contribute exactly zero and are skipped.
#include <climits>

#include "pbf_internal.cuh"

namespace pbf {

namespace {

constexpr int kSparseThreads = 128;
// PBF_DENSE_WARPS (a build-time tuning macro): warps of a dense-kernel block,
// i.e. the chunks each listed particle's window is split into.
#ifndef PBF_DENSE_WARPS
#define PBF_DENSE_WARPS 8
#endif
constexpr int kDenseWarps = PBF_DENSE_WARPS;   // chunks of a dense item's windows
constexpr int kDenseThreads = 32 * kDenseWarps;
// Below kDenseAllBelow particles one thread per particle leaves most of the
// GPU idle: by default every warp then takes the dense kernel (8 warps per 32
// particles).  StepConsts::dense_window / dense_all override the defaults
// (pbf_autotune).
constexpr int kMaxFields = 6;                   // partial-sum fields of the largest pass
constexpr unsigned kFull = 0xffffffffu;

enum PassKind { kLambda = 0, kDeltaP = 1, kDeltaPFinal = 2, kXsph = 3 };

// Everything any pass kernel needs (passed by value).
struct PassArgs {
  StepConsts c;
  Geometry G;
  const float4* X;        // positions the pass reads (sorted)
  const uint32_t* cs;     // cell prefix, cells + 1 entries
  int n;
  int counter;            // flags word holding this pass's dense-list length
  int next_counter;       // the other one, cleared for the next pass
  int item_counter;       // flags word handing out this pass's dense batches
  int next_item_counter;  // the other one, cleared for the next pass
  int dense_all;          // every warp takes the dense kernel (small n)
  uint32_t* flags;
  uint32_t* dense;
  uint32_t* masks;        // neighbour masks: lambda saves them, delta_p reads them
  int mask_stride;
  uint32_t* cell_flags;   // CellFlag bits per cell
  const uint32_t* skeys;  // stale cell of each sorted slot
  float* lambda;          // lambda: out;  delta_p: in
  float* rho;             // lambda: out;  xsph: in
  float4* T;              // delta_p: out
  const float4* xs;       // delta_p_final: sorted x at t
  const uint32_t* iid_s;  // delta_p_final: sorted iid
  float4* npos;           // delta_p_final: out
  float4* vel;            // delta_p_final: out
  float4* pos;            // delta_p_final: out (permuted inputs)
  uint32_t* iid;          // delta_p_final: out (permuted inputs)
  const float4* V;        // xsph: velocities
  float4* NV;             // xsph: out
  // group tables (the dense kernel visits groups of grouped cells)
  const int* grp_off;
  const int* grp_n;
  const int* grp_cnt;
  const float4* grp_pos;
  const float4* grp_sum;
  const float4* grp_aux;
  // the particles the pass computes: list[0, flags[count_word]) (null: every
  // particle, in order); the work list of the lambda / delta_p passes, or the
  // current-cell buckets.  identity_word >= 0: a flag saying the list is the
  // identity (every particle in order)
  const int* list;
  int count_word;
  int identity_word;
};

// The particle that thread slot t of a pass computes (t < work_count(a)).
__device__ __forceinline__ int work_count(const PassArgs& a) {
  return a.list ? (int)a.flags[a.count_word] : a.n;
}
__device__ __forceinline__ int work_particle(const PassArgs& a, int t) {
  return a.list && !(a.identity_word >= 0 && a.flags[a.identity_word]) ? __ldg(a.list + t) : t;
}

// ---- windows ------------------------------------------------------------------------

// Sorted-slot range [s, e) of cells (x, y, z-1 .. z+1) clipped to the grid.
// cs[cells] == n, so e <= n; the clamps keep even an inconsistent table in range.
__device__ __forceinline__ void column_run(const SceneGeom& g, const uint32_t* __restrict__ cs,
                                           int n, int x, int y, int z, int& s, int& e) {
  const int zlo = max(z - 1, 0), zhi = min(z + 1, g.dims[2] - 1);
  const int base = g.cell_base + (x * g.dims[1] + y) * g.dims[2];
  s = (int)__ldg(cs + base + zlo);
  e = max(min((int)__ldg(cs + base + zhi + 1), n), s);
}

__device__ __forceinline__ int window_total(const SceneGeom& g, const uint32_t* __restrict__ cs,
                                            int n, int3 q) {
  int total = 0;
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      int s, e;
      column_run(g, cs, n, x, y, q.z, s, e);
      total += e - s;
    }
  }
  return total;
}

// Candidates of the window and the chunks of 32 consecutive candidates it
// splits into (per run), from one walk over its runs.
__device__ __forceinline__ int window_total_chunks(const SceneGeom& g, const uint32_t* __restrict__ cs, int n,
                                                   int3 q, int& chunks) {
  int total = 0;
  chunks = 0;
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      int s, e;
      column_run(g, cs, n, x, y, q.z, s, e);
      total += e - s;
      chunks += (e - s + 31) >> 5;
    }
  }
  return total;
}

// Whether a cell of the window carries any of `bits`.
__device__ __forceinline__ bool window_flagged(const SceneGeom& g,
                                               const uint32_t* __restrict__ cell_flags, int3 q,
                                               uint32_t bits) {
  const int zlo = max(q.z - 1, 0), zhi = min(q.z + 1, g.dims[2] - 1);
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      const int base = g.cell_base + (x * g.dims[1] + y) * g.dims[2];
      for (int z = zlo; z <= zhi; ++z)
        if (cell_flags[base + z] & bits) return true;
    }
  }
  return false;
}

// ---- where a pass reads candidate positions ---------------------------------------------
//
// From global memory (X[j], read-only path), or from the block's staged copy
// of its window in shared memory.  Run r = 3 (dx + 1) + (dy + 1) of a window
// is one column of three z-consecutive cells; a block stages, per run, the
// slots of the z-range its particles' runs cover, and slot j of run r sits at
// S[j + D[r]].  Either source gives bitwise the same positions, so a pass's
// sums do not depend on which one it read.
struct FromGlobal {
  const float4* __restrict__ X;
  __device__ __forceinline__ float4 at(int j, int) const { return __ldg(X + j); }
  // hit-queue entry of a chunk starting at slot j of run r, and back
  __device__ __forceinline__ int tag(int j, int) const { return j; }
  __device__ __forceinline__ float4 untag(int t, int bit, int& j) const {
    j = t + bit;
    return __ldg(X + j);
  }
};

struct FromStage {
  const float4* S;  // shared memory: the staged runs
  const int* D;     // shared memory: per run, staged index - slot
  __device__ __forceinline__ float4 at(int j, int r) const { return S[j + D[r]]; }
  // staged index (< 2^16) and run
  __device__ __forceinline__ int tag(int j, int r) const { return (j + D[r]) | (r << 16); }
  __device__ __forceinline__ float4 untag(int t, int bit, int& j) const {
    const int v = (t & 0xffff) + bit;
    j = v - D[t >> 16];
    return S[v];
  }
};

// Every candidate of the window, in order.
template <class P, class Src>
__device__ __forceinline__ void visit_window(const SceneGeom& g, const uint32_t* __restrict__ cs,
                                             int n, int3 q, const Src& src, P& p) {
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      const int r = 3 * (dx + 1) + (dy + 1);
      int s, e;
      column_run(g, cs, n, x, y, q.z, s, e);
      for (int j = s; j < e; ++j) p.visit(src.at(j, r), j);
    }
  }
}

// ---- hit queue ------------------------------------------------------------------------
//
// The masked walks below test a chunk of up to 32 consecutive candidates at a
// time into a bit mask (cheap, every lane busy) and run the pair body on the
// set bits only.  Running the body right after each chunk costs a warp
// max-over-lanes(hits of that chunk) body iterations per chunk; lanes whose
// particle has fewer hits in that chunk idle, chunk after chunk.  Instead each
// thread queues its non-empty chunks (mask + where the chunk starts) in shared
// memory and HitQueue::flush runs the body once per queued hit in one flat
// loop, so the warp pays max-over-lanes of the hits of the whole queued span.
// Hits are visited in the order they were queued -- the window's visiting
// order -- so the sums are bitwise those of visiting each chunk's hits right
// away.  The capacity (chunks queued per thread before a flush) comes from
// the step's tuning (StepConsts::queue_sparse / queue_dense); capacity 1 runs
// each chunk's hits right away, straight from registers.
struct HitQueue {
  uint32_t* mask;  // this thread's column: entry k at mask[k * stride]
  int* base;       // where queued chunk k starts (Src::tag)
  int stride;
  int cap;
  int n = 0;

  __device__ HitQueue(uint32_t* mask_, int* base_, int stride_, int cap_)
      : mask(mask_), base(base_), stride(stride_), cap(cap_) {}
  template <class P, class Src>
  __device__ __forceinline__ void flush(const Src& src, P& p) {
    uint32_t m = 0u;
    int b = 0, k = 0;
    for (;;) {
      if (!m) {
        if (k == n) break;
        m = mask[k * stride];  // every queued mask has a bit set
        b = base[k * stride];
        ++k;
      }
      const int bit = __ffs(m) - 1;
      m &= m - 1u;
      int j;
      const float4 xj = src.untag(b, bit, j);
      p.visit(xj, j);
    }
    n = 0;
  }
  template <class P, class Src>
  __device__ __forceinline__ void push(uint32_t m, int tag, const Src& src, P& p) {
    if (cap == 1) {  // no queue: the chunk's hits right away, straight from registers
      while (m) {
        const int bit = __ffs(m) - 1;
        m &= m - 1u;
        int j;
        const float4 xj = src.untag(tag, bit, j);
        p.visit(xj, j);
      }
      return;
    }
    if (!m) return;
    mask[n * stride] = m;
    base[n * stride] = tag;
    if (++n == cap) flush(src, p);
  }
};

// Hit mask of candidates [jb, jb + min(32, j1 - jb)) of run r (four loads in flight).
template <class P, class Src>
__device__ __forceinline__ uint32_t chunk_mask(const Src& src, int jb, int j1, int r, const P& p) {
  const int m = min(32, j1 - jb);
  uint32_t mask = 0u;
  int k = 0;
  for (; k + 3 < m; k += 4) {
    const float4 a = src.at(jb + k, r), b = src.at(jb + k + 1, r), c2 = src.at(jb + k + 2, r),
                 d = src.at(jb + k + 3, r);
    mask |= (uint32_t)p.hit(a, jb + k) << k;
    mask |= (uint32_t)p.hit(b, jb + k + 1) << (k + 1);
    mask |= (uint32_t)p.hit(c2, jb + k + 2) << (k + 2);
    mask |= (uint32_t)p.hit(d, jb + k + 3) << (k + 3);
  }
  for (; k < m; ++k) mask |= (uint32_t)p.hit(src.at(jb + k, r), jb + k) << k;
  return mask;
}

// Candidates [j0, j1) of run r, in order: with skip_misses (the pass's exact
// rules do not need every candidate) a hit mask per chunk of 32 (four loads in
// flight), its hits queued for p.visit() (the caller flushes hq); else every
// candidate, four loads in flight, after flushing what is queued.  Same result
// as visiting each candidate in turn.
template <class P, class Src>
__device__ __forceinline__ void visit_run(const Src& src, int j0, int j1, int r, P& p, bool skip_misses,
                                          HitQueue& hq) {
  if (skip_misses) {
    for (int jb = j0; jb < j1; jb += 32) hq.push(chunk_mask(src, jb, j1, r, p), src.tag(jb, r), src, p);
  } else {
    hq.flush(src, p);
    int j = j0;
    for (; j + 3 < j1; j += 4) {
      const float4 q0 = src.at(j, r), q1 = src.at(j + 1, r), q2 = src.at(j + 2, r), q3 = src.at(j + 3, r);
      p.visit(q0, j);
      p.visit(q1, j + 1);
      p.visit(q2, j + 2);
      p.visit(q3, j + 3);
    }
    for (; j < j1; ++j) p.visit(src.at(j, r), j);
  }
}

// Every candidate of the window, in order, in two stages per chunk of 32
// consecutive slots of a run: a cheap test p.hit() of each candidate (four
// loads in flight) into a bit mask, then p.visit() on the set bits in
// ascending order, through the hit queue.  p.visit() leaves non-hits
// untouched, so the result is that of visit_window.
//
// save_masks: store chunk k's mask at masks[k * stride + i] (k < kMaskWords;
// i: the particle's mask slot) for the next pass over the same positions.
template <class P, class Src>
__device__ __forceinline__ void visit_window_masked(const SceneGeom& g,
                                                    const uint32_t* __restrict__ cs, int n,
                                                    int3 q, const Src& src, P& p,
                                                    uint32_t* __restrict__ masks, int stride,
                                                    int i, HitQueue& hq) {
  int chunk = 0;
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      const int r = 3 * (dx + 1) + (dy + 1);
      int s, e;
      column_run(g, cs, n, x, y, q.z, s, e);
      for (int j0 = s; j0 < e; j0 += 32) {
        const uint32_t mask = chunk_mask(src, j0, e, r, p);
        if (masks && chunk < kMaskWords) masks[chunk * stride + i] = mask;
        ++chunk;
        hq.push(mask, src.tag(j0, r), src, p);
      }
    }
  }
  hq.flush(src, p);
}

// The window's neighbours from the masks a previous pass over the same
// positions saved (visit_window_masked with save): p.visit() on the set bits,
// in order, through the hit queue.  The saved hits are a superset of p's
// (p.visit re-tests).
// chunks: the window's chunk count (at most kMaskWords); each chunk's mask is
// loaded two chunks ahead of its use, so its latency overlaps the pair work.
template <class P, class Src>
__device__ __forceinline__ void visit_window_saved(const SceneGeom& g,
                                                   const uint32_t* __restrict__ cs, int n, int3 q,
                                                   const Src& src, P& p,
                                                   const uint32_t* __restrict__ masks, int stride,
                                                   int i, int chunks, HitQueue& hq) {
  int chunk = 0;
  uint32_t m0 = chunks > 0 ? __ldg(masks + i) : 0u;
  uint32_t m1 = chunks > 1 ? __ldg(masks + stride + i) : 0u;
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      const int r = 3 * (dx + 1) + (dy + 1);
      int s, e;
      column_run(g, cs, n, x, y, q.z, s, e);
      for (int j0 = s; j0 < e; j0 += 32, ++chunk) {
        const uint32_t m = m0;
        m0 = m1;
        m1 = chunk + 2 < chunks ? __ldg(masks + (chunk + 2) * stride + i) : 0u;
        hq.push(m, src.tag(j0, r), src, p);
      }
    }
  }
  hq.flush(src, p);
}

// Candidates [v_lo, v_hi) of the window (numbered in visiting order), run by
// run through visit_run (hit masks and the hit queue, or every candidate on
// the exact path).  The caller flushes hq.
template <class P, class Src>
__device__ __forceinline__ void visit_window_chunk(const SceneGeom& g, const uint32_t* __restrict__ cs, int n,
                                                   int3 q, const Src& src, P& p, int v_lo, int v_hi, HitQueue& hq) {
  int v0 = 0;
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      const int r = 3 * (dx + 1) + (dy + 1);
      int s, e;
      column_run(g, cs, n, x, y, q.z, s, e);
      const int len = e - s;
      const int a = max(v_lo, v0), b = min(v_hi, v0 + len);
      if (a < b) visit_run(src, s + (a - v0), s + (b - v0), r, p, p.skip_misses(), hq);
      v0 += len;
    }
  }
  hq.flush(src, p);
}

// Part `part` of `parts` (a power of two) of the window, interleaved: the
// window's chunks of up to 32 consecutive candidates (per run, in visiting
// order) are numbered 0, 1, 2, ..., and chunk c belongs to part c mod parts.
// Parts of a window then hold about equal shares of its near and far
// candidates, so the warps that split a window finish together.  The caller
// flushes nothing: hq is flushed here.
template <class P, class Src>
__device__ __forceinline__ void visit_window_strided(const SceneGeom& g, const uint32_t* __restrict__ cs, int n,
                                                     int3 q, const Src& src, P& p, int part, int parts,
                                                     HitQueue& hq) {
  int c0 = 0;  // chunks of the window before this run
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      const int r = 3 * (dx + 1) + (dy + 1);
      int s, e;
      column_run(g, cs, n, x, y, q.z, s, e);
      const int nch = (e - s + 31) >> 5;
      for (int k = (part - c0) & (parts - 1); k < nch; k += parts) {
        const int jb = s + 32 * k;
        visit_run(src, jb, min(jb + 32, e), r, p, p.skip_misses(), hq);
      }
      c0 += nch;
    }
  }
  hq.flush(src, p);
}

// Groups of cell `cell` in the pass's table, or -1 when the cell is visited
// particle by particle.
__device__ __forceinline__ int cell_groups(const PassArgs& a, int cell, int& slot) {
  const uint32_t sl = __ldg(a.cell_flags + cell) >> kCellSlotShift;
  slot = (int)sl - 1;
  return sl ? __ldg(a.grp_n + slot) : -1;
}

// Entries of the window when grouped cells count their groups.
__device__ __forceinline__ int window_total_grouped(const SceneGeom& g, const PassArgs& a, int3 q) {
  const int zlo = max(q.z - 1, 0), zhi = min(q.z + 1, g.dims[2] - 1);
  int total = 0;
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      const int base = g.cell_base + (x * g.dims[1] + y) * g.dims[2];
      for (int z = zlo; z <= zhi; ++z) {
        int slot;
        const int ng = cell_groups(a, base + z, slot);
        if (ng > 0) {
          total += ng;
        } else {
          const int s0 = (int)__ldg(a.cs + base + z);
          total += max(min((int)__ldg(a.cs + base + z + 1), a.n), s0) - s0;
        }
      }
    }
  }
  return total;
}

// Entries [v_lo, v_hi) of the window in visiting order, grouped cells
// contributing their groups (p.visit_group; `own`: i belongs to the cell) and
// the other cells their particles (p.visit).  Without grouped cells this
// visits exactly what visit_window_chunk does, in the same order.
template <class P, class Src>
__device__ __forceinline__ void visit_window_grouped(const SceneGeom& g, const PassArgs& a, int3 q,
                                                     const Src& src, P& p, int v_lo, int v_hi, HitQueue& hq) {
  const int zlo = max(q.z - 1, 0), zhi = min(q.z + 1, g.dims[2] - 1);
  int v0 = 0;
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      const int r = 3 * (dx + 1) + (dy + 1);
      const int base = g.cell_base + (x * g.dims[1] + y) * g.dims[2];
      for (int z = zlo; z <= zhi; ++z) {
        int slot;
        const int ng = cell_groups(a, base + z, slot);
        const int s0 = (int)__ldg(a.cs + base + z);
        const int e0 = max(min((int)__ldg(a.cs + base + z + 1), a.n), s0);
        const int len = ng > 0 ? ng : e0 - s0;
        const int lo = max(v_lo, v0), hi = min(v_hi, v0 + len);
        if (lo < hi) {
          if (ng > 0) {
            hq.flush(src, p);  // queued hits come first in visiting order
            const int t0 = __ldg(a.grp_off + slot);
            const bool own = p.i >= s0 && p.i < e0;  // i is one of the cell's particles
            int t = t0 + (lo - v0);
            const int tend = t0 + (hi - v0);
            constexpr int U = P::kGroupUnroll;  // groups' loads in flight (unused parts are not loaded)
            for (; t + U - 1 < tend; t += U) {
              float4 gp[U], gs[U], ga[U];
              int gc[U];
#pragma unroll
              for (int u = 0; u < U; ++u) {
                gp[u] = __ldg(a.grp_pos + t + u);
                gc[u] = __ldg(a.grp_cnt + t + u);
                gs[u] = __ldg(a.grp_sum + t + u);
                ga[u] = __ldg(a.grp_aux + t + u);
              }
#pragma unroll
              for (int u = 0; u < U; ++u) p.visit_group(gp[u], gc[u], gs[u], ga[u], own);
            }
            for (; t < tend; ++t)
              p.visit_group(__ldg(a.grp_pos + t), __ldg(a.grp_cnt + t), __ldg(a.grp_sum + t),
                            __ldg(a.grp_aux + t), own);
          } else {
            visit_run(src, s0 + (lo - v0), s0 + (hi - v0), r, p, p.skip_misses(), hq);
          }
        }
        v0 += len;
      }
    }
  }
  hq.flush(src, p);
}

// ---- the passes: per-candidate visit, partial-sum fields, finish ----------------------

struct LambdaPass {
  static constexpr int kFields = 5;
  static constexpr int kGroupUnroll = 2;
  const StepConsts& c;
  const SceneGeom& g;
  float4 xi;
  int i;
  float pho = 0.f, gx = 0.f, gy = 0.f, gz = 0.f, gl2 = 0.f;

  __device__ LambdaPass(const PassArgs& a, const SceneGeom& g_, float4 xi_, int i_, bool)
      : c(a.c), g(g_), xi(xi_), i(i_) {}
  // candidates outside the cutoff add nothing (no exact rule in this pass)
  __device__ __forceinline__ bool skip_misses() const { return true; }
  __device__ __forceinline__ bool hit(float4 xj, int) const {
    return !(dist2(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z) >= c.h2);
  }
  __device__ __forceinline__ void visit(float4 xj, int j) {
    const float ex = xi.x - xj.x, ey = xi.y - xj.y, ez = xi.z - xj.z;
    const float r2 = dist2(ex, ey, ez);
    if (!(r2 >= c.h2)) {  // NaN-inclusive, as getPoly6
      pho += poly6_inside(c, r2);
      if (!(r2 < c.keps2)) {  // as getSpikyGrad's |r| < KERNAL_EPS test
        const float ir = rsqrtf(r2);
        const float t = c.h - r2 * ir;
        const float sc = c.spiky_coef_rho0 * t * t * ir;
        const float ax = sc * ex, ay = sc * ey, az = sc * ez;
        gx += ax;
        gy += ay;
        gz += az;
        if (j != i) gl2 += dist2(ax, ay, az);
      }
    }
  }
  // `cnt` particles at xg.  The group holding i itself lies at r2 = 0 <
  // keps2 (grouping needs keps2 > 0): no gradient, as the reference's j != i.
  __device__ __forceinline__ void visit_group(float4 xg, int cnt, float4, float4, bool) {
    const float ex = xi.x - xg.x, ey = xi.y - xg.y, ez = xi.z - xg.z;
    const float r2 = dist2(ex, ey, ez);
    if (!(r2 >= c.h2)) {
      const float fc = (float)cnt;
      pho += fc * poly6_inside(c, r2);
      if (!(r2 < c.keps2)) {
        const float ir = rsqrtf(r2);
        const float t = c.h - r2 * ir;
        const float sc = c.spiky_coef_rho0 * t * t * ir;
        const float ax = sc * ex, ay = sc * ey, az = sc * ez;
        gx += fc * ax;
        gy += fc * ay;
        gz += fc * az;
        gl2 += fc * dist2(ax, ay, az);
      }
    }
  }
  __device__ void store(float* f, int stride) const {
    f[0] = pho, f[stride] = gx, f[2 * stride] = gy, f[3 * stride] = gz, f[4 * stride] = gl2;
  }
  __device__ void add(const float* f, int stride) {
    pho += f[0], gx += f[stride], gy += f[2 * stride], gz += f[3 * stride], gl2 += f[4 * stride];
  }
  __device__ void finish(const PassArgs& a) const {
    float rho = pho;
    if (c.k_b != 0.f) rho += c.k_b * boundary_density(c, g, xi);
    const float grad_l2 = gl2 + dist2(gx, gy, gz);
    const float lam = -(rho / c.pho0 - 1.f) / (grad_l2 + c.lambda_eps);
    a.lambda[i] = lam;
    a.rho[i] = rho;
    const uint32_t bits = (isfinite(lam) ? 0u : (uint32_t)kCellLambdaNonFinite) |
                          (rho > 0.f && isfinite(rho) ? 0u : (uint32_t)kCellRhoNotPositive);
    if (bits) {
      atomicOr(&a.cell_flags[a.skeys[i]], bits);
      if (bits & kCellLambdaNonFinite) atomicOr(&a.flags[kFlagLambdaNonFinite], 1u);
      if (bits & kCellRhoNotPositive) atomicOr(&a.flags[kFlagXsphExact], 1u);
    }
  }
};

// sum over neighbours j != i of (lambda_i + lambda_j + s_corr) grad W.  exact
// adds the reference's poisoning of the sum by a non-finite lambda through a
// zero gradient (candidates j != i outside the cutoff).
template <bool kFinal>
struct DeltaPPass {
  static constexpr int kFields = 4;
  static constexpr int kGroupUnroll = 2;
  const StepConsts& c;
  const SceneGeom& g;
  const float* __restrict__ lambda;
  float4 xi;
  int i;
  float li;
  bool exact;
  float ax = 0.f, ay = 0.f, az = 0.f;
  bool poison = false;

  __device__ DeltaPPass(const PassArgs& a, const SceneGeom& g_, float4 xi_, int i_, bool exact_)
      : c(a.c), g(g_), lambda(a.lambda), xi(xi_), i(i_), li(a.lambda[i_]), exact(exact_) {}
  __device__ __forceinline__ bool skip_misses() const { return !exact; }
  __device__ __forceinline__ bool hit(float4 xj, int j) const {
    const float r2 = dist2(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
    return !(r2 >= c.h2) && !(r2 < c.keps2) && j != i;
  }
  __device__ __forceinline__ void visit(float4 xj, int j) {
    // lambda_j first: its load overlaps the distance test (a visited candidate
    // is almost always a neighbour, so the load is rarely wasted)
    const float lj = __ldg(lambda + j);
    const float ex = xi.x - xj.x, ey = xi.y - xj.y, ez = xi.z - xj.z;
    const float r2 = dist2(ex, ey, ez);
    if (!(r2 >= c.h2) && !(r2 < c.keps2) && j != i) {  // NaN-inclusive, as the reference
      const float wgt = poly6_inside(c, r2);
      const float corr = c.coef_corr * pow_corr(c, wgt);
      const float ir = rsqrtf(r2);
      const float t = c.h - r2 * ir;
      const float f = (li + lj + corr) * (c.spiky_coef * t * t * ir);
      ax = fmaf(f, ex, ax);
      ay = fmaf(f, ey, ay);
      az = fmaf(f, ez, az);
    } else if (exact && j != i) {
      // zero gradient: (lambda_i + lambda_j + s_corr) * 0 is NaN iff a lambda is not finite
      poison |= !isfinite(li) || !isfinite(lj);
    }
  }
  // `cnt` particles at xg with lambda_j summing to cnt sum.x + sum.y (each
  // lambda_j - sum.x finite, or lambda_j the same bits as sum.x).  exact: the
  // poisoning rule for the group's members j != i (i is a member when it
  // belongs to the cell and sits at xg).
  __device__ __forceinline__ void visit_group(float4 xg, int cnt, float4 sum, float4, bool own) {
    const float ex = xi.x - xg.x, ey = xi.y - xg.y, ez = xi.z - xg.z;
    const float r2 = dist2(ex, ey, ez);
    if (!(r2 >= c.h2) && !(r2 < c.keps2)) {
      const float wgt = poly6_inside(c, r2);
      const float corr = c.coef_corr * pow_corr(c, wgt);
      const float ir = rsqrtf(r2);
      const float t = c.h - r2 * ir;
      const float f = ((float)cnt * (li + sum.x + corr) + sum.y) * (c.spiky_coef * t * t * ir);
      ax = fmaf(f, ex, ax);
      ay = fmaf(f, ey, ay);
      az = fmaf(f, ez, az);
    } else if (exact) {
      const bool member = own && __float_as_uint(xi.x) == __float_as_uint(xg.x) &&
                          __float_as_uint(xi.y) == __float_as_uint(xg.y) &&
                          __float_as_uint(xi.z) == __float_as_uint(xg.z);
      if (cnt > (member ? 1 : 0)) poison |= !isfinite(li) || !isfinite(sum.x);
    }
  }
  __device__ void store(float* f, int stride) const {
    f[0] = ax, f[stride] = ay, f[2 * stride] = az, f[3 * stride] = poison ? 1.f : 0.f;
  }
  __device__ void add(const float* f, int stride) {
    ax += f[0], ay += f[stride], az += f[2 * stride];
    poison |= f[3 * stride] != 0.f;
  }
  // d / pho0, per-component clamp to +-max_dp, wall clamp
  // (fluids/Simulator_kernel.cuh:184-193); fminf/fmaxf map a NaN to the bound.
  __device__ void finish(const PassArgs& a) const {
    float sx = ax, sy = ay, sz = az;
    if (poison) sx = sy = sz = __int_as_float(0x7fffffff);
    const float dx = fmaxf(fminf(sx / c.pho0, c.max_dp), -c.max_dp);
    const float dy = fmaxf(fminf(sy / c.pho0, c.max_dp), -c.max_dp);
    const float dz = fmaxf(fminf(sz / c.pho0, c.max_dp), -c.max_dp);
    const float4 xf = make_float4(fmaxf(fminf(xi.x + dx, g.hi[0]), g.lo[0]),
                                  fmaxf(fminf(xi.y + dy, g.hi[1]), g.lo[1]),
                                  fmaxf(fminf(xi.z + dz, g.hi[2]), g.lo[2]), xi.w);
    if (!kFinal) {
      a.T[i] = xf;
      return;
    }
    // last iteration: x_final -> npos, v = (x_final - x) * (1/dt) -> vel, and the
    // caller's pos / iid receive the permuted inputs (the reference's in-place sort)
    const float4 x0 = a.xs[i];
    a.npos[i] = make_float4(xf.x, xf.y, xf.z, x0.w);
    const float4 v = make_float4((xf.x - x0.x) * c.inv_dt, (xf.y - x0.y) * c.inv_dt,
                                 (xf.z - x0.z) * c.inv_dt, 0.f);
    a.vel[i] = v;
    if (!isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z)) {
      atomicOr(&a.cell_flags[a.skeys[i]], (uint32_t)kCellVelNonFinite);
      atomicOr(&a.flags[kFlagXsphExact], 1u);
    }
    a.pos[i] = x0;
    a.iid[i] = a.iid_s[i];
  }
};

// sum over the window of 2 (v_j - v_i) W / (rho_i + rho_j).  exact adds the
// reference's NaN from 0 * v / (rho_i + rho_j) outside the cutoff.
struct XsphPass {
  static constexpr int kFields = 6;
  static constexpr int kGroupUnroll = 2;
  const StepConsts& c;
  const float4* __restrict__ V;
  const float* __restrict__ rho;
  float4 xi, vi;
  float ri;
  int i;
  bool exact;
  float ax = 0.f, ay = 0.f, az = 0.f;
  bool px = false, py = false, pz = false;

  __device__ XsphPass(const PassArgs& a, const SceneGeom&, float4 xi_, int i_, bool exact_)
      : c(a.c), V(a.V), rho(a.rho), xi(xi_), vi(a.V[i_]), ri(a.rho[i_]), i(i_), exact(exact_) {}
  __device__ __forceinline__ bool skip_misses() const { return !exact; }
  __device__ __forceinline__ bool hit(float4 xj, int) const {
    return !(dist2(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z) >= c.h2);
  }
  __device__ __forceinline__ void visit(float4 xj, int j) {
    // v_j and rho_j first: their loads overlap the distance test (a visited
    // candidate is almost always a neighbour)
    const float4 vj = __ldg(V + j);
    const float rj = __ldg(rho + j);
    const float r2 = dist2(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
    if (!(r2 >= c.h2)) {  // NaN-inclusive, as getPoly6
      const float w2 = 2.f * poly6_inside(c, r2) / (ri + rj);
      ax = fmaf(vj.x - vi.x, w2, ax);
      ay = fmaf(vj.y - vi.y, w2, ay);
      az = fmaf(vj.z - vi.z, w2, az);
    } else if (exact) {
      // W = 0: 2 (v_j - v_i) * 0 / (rho_i + rho_j) is NaN iff the velocity
      // difference is not finite or the denominator is 0 or NaN
      const float den = ri + rj;
      const bool bad_den = !(den != 0.f) || isnan(den);
      px |= bad_den || !isfinite(vj.x - vi.x);
      py |= bad_den || !isfinite(vj.y - vi.y);
      pz |= bad_den || !isfinite(vj.z - vi.z);
    }
  }
  // `cnt` particles at xg sharing the density sum.w and the velocity aux.xyz
  // (sum.xyz: the sum over the group of v_j - aux.xyz, zero for the groups
  // built here).
  // exact: the rule for 0 * (v_j - v_i) / (rho_i + rho_j) outside the cutoff;
  // the group build guarantees that every member's v_j - aux is finite or
  // that v_j is aux itself, so the first member's velocity decides.
  __device__ __forceinline__ void visit_group(float4 xg, int cnt, float4 sum, float4 aux, bool) {
    const float r2 = dist2(xi.x - xg.x, xi.y - xg.y, xi.z - xg.z);
    if (!(r2 >= c.h2)) {
      const float fc = (float)cnt;
      const float w2 = 2.f * poly6_inside(c, r2) / (ri + sum.w);
      ax = fmaf(fmaf(fc, aux.x - vi.x, sum.x), w2, ax);
      ay = fmaf(fmaf(fc, aux.y - vi.y, sum.y), w2, ay);
      az = fmaf(fmaf(fc, aux.z - vi.z, sum.z), w2, az);
    } else if (exact) {
      const float den = ri + sum.w;
      const bool bad_den = !(den != 0.f) || isnan(den);
      px |= bad_den || !isfinite(aux.x - vi.x);
      py |= bad_den || !isfinite(aux.y - vi.y);
      pz |= bad_den || !isfinite(aux.z - vi.z);
    }
  }
  __device__ void store(float* f, int stride) const {
    f[0] = ax, f[stride] = ay, f[2 * stride] = az;
    f[3 * stride] = px ? 1.f : 0.f, f[4 * stride] = py ? 1.f : 0.f, f[5 * stride] = pz ? 1.f : 0.f;
  }
  __device__ void add(const float* f, int stride) {
    ax += f[0], ay += f[stride], az += f[2 * stride];
    px |= f[3 * stride] != 0.f, py |= f[4 * stride] != 0.f, pz |= f[5 * stride] != 0.f;
  }
  __device__ void finish(const PassArgs& a) const {
    const float qnan = __int_as_float(0x7fffffff);
    a.NV[i] = make_float4(fmaf(c.c_xsph, px ? qnan : ax, vi.x), fmaf(c.c_xsph, py ? qnan : ay, vi.y),
                          fmaf(c.c_xsph, pz ? qnan : az, vi.z), 0.f);
  }
};

template <int kKind> struct PassOf;
template <> struct PassOf<kLambda> { using type = LambdaPass; };
template <> struct PassOf<kDeltaP> { using type = DeltaPPass<false>; };
template <> struct PassOf<kDeltaPFinal> { using type = DeltaPPass<true>; };
template <> struct PassOf<kXsph> { using type = XsphPass; };

// Whether particle i must visit every candidate of its window to reproduce the
// reference's IEEE poisoning (a strict superset of the particles whose sums
// can be poisoned): only when the step raised the pass's flag and i's own
// values or a flagged cell of its window could poison its sum.
__device__ __forceinline__ bool exact_path(int kind, const PassArgs& a, const SceneGeom& g,
                                           int3 q, int i) {
  if (kind == kDeltaP || kind == kDeltaPFinal) {
    if (a.flags[kFlagLambdaNonFinite] == 0u) return false;
    return !isfinite(a.lambda[i]) || window_flagged(g, a.cell_flags, q, kCellLambdaNonFinite);
  }
  if (kind == kXsph) {
    if (a.flags[kFlagXsphExact] == 0u) return false;
    const float ri = a.rho[i];
    const float4 vi = a.V[i];
    return !(ri > 0.f && isfinite(ri)) || !isfinite(vi.x) || !isfinite(vi.y) || !isfinite(vi.z) ||
           window_flagged(g, a.cell_flags, q, kCellRhoNotPositive | kCellVelNonFinite);
  }
  return false;
}

// ---- window staging: bulk async copies into shared memory ------------------------------
//
// With the passes taking particles in current-cell order, the particles of a
// block usually sit in cells of one column (scene, x, y), z-consecutive: their
// windows are then made of the same 9 column runs, each particle's run r a
// z-sub-range of the block's run r, which covers cells [zmin - 1, zmax + 1] of
// column (x + dx, y + dy) -- one contiguous range of sorted slots.  Such a
// block copies its runs' positions (16 bytes a slot, 16-byte aligned) into
// shared memory with one cp.async.bulk per run, all completing on one
// mbarrier, and its threads then walk their windows there (FromStage) instead
// of through L1 (FromGlobal).  Blocks whose particles span several columns,
// whose runs exceed the stage, or whose runs hold a grouped cell read global
// memory as before.  The wait is bounded: past kStageSpins polls the block
// records kErrStageTimeout, stops staging and reads global memory (same
// results), and waits once more (bounded) for the copy before it exits.
// On GB300 the staged variants measured slower than the L1 path on every
// workload tried (the candidates are L1-resident already, and the stage costs
// resident blocks and a wait per block), so the default stages are 0 and
// pbf_autotune turns them on only where its trial steps find them faster.

constexpr int kStageSpins = 1 << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0u;
}
// Bounded wait for the phase of the given parity to complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (int k = 0; k < kStageSpins; ++k)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// bytes (a multiple of 16) from global src to shared dst (both 16-byte
// aligned), completing as transaction bytes on bar.  A CTA's own shared
// memory address is a valid shared::cluster address (no cluster launch, no
// multicast).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Orders this thread's earlier generic-proxy accesses of shared memory (the
// previous item's reads of the stage) before its following async-proxy writes.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// A block's staging state in shared memory.
struct StageState {
  uint64_t bar;
  int D[9];           // per run: staged index - first slot
  int ok;             // this item's runs are staged
  int failed;         // a wait gave up: the block stages no more
  int wx[kDenseThreads / 32], wy[kDenseThreads / 32], wcb[kDenseThreads / 32];
  int wzmin[kDenseThreads / 32], wzmax[kDenseThreads / 32], wi[kDenseThreads / 32];
  int wsame[kDenseThreads / 32];
};

// Votes of one warp: whether its participating lanes share (scene, x, y), the
// z-range they cover and one participating particle (lane 0 of the warp writes
// st.w*[w]).  Every lane of the warp calls it.
__device__ __forceinline__ void stage_vote(StageState& st, int w, bool part, const SceneGeom& g, int3 q,
                                           int i) {
  const unsigned pm = __ballot_sync(kFull, part);
  const int lead = pm ? __ffs(pm) - 1 : 0;
  const int lx = __shfl_sync(kFull, q.x, lead), ly = __shfl_sync(kFull, q.y, lead);
  const int lcb = __shfl_sync(kFull, g.cell_base, lead), li = __shfl_sync(kFull, i, lead);
  const bool same = __all_sync(kFull, !part || (q.x == lx && q.y == ly && g.cell_base == lcb));
  const int zmin = __reduce_min_sync(kFull, part ? q.z : INT_MAX);
  const int zmax = __reduce_max_sync(kFull, part ? q.z : INT_MIN);
  if ((threadIdx.x & 31) == 0) {
    st.wsame[w] = pm == 0u ? -1 : (same ? 1 : 0);  // -1: no participating lane
    st.wx[w] = lx, st.wy[w] = ly, st.wcb[w] = lcb, st.wi[w] = li;
    st.wzmin[w] = zmin, st.wzmax[w] = zmax;
  }
}

// Thread 0, after the votes of warps [0, nw): when every participating lane
// shares one column and its runs fit in `cap` slots and hold no grouped cell,
// sets st.D, arms st.bar for the runs' bytes and issues one bulk copy per
// non-empty run into S; st.ok says whether it did.
__device__ __forceinline__ void stage_issue(StageState& st, int nw, const PassArgs& a, float4* S, int cap) {
  st.ok = 0;
  if (st.failed || cap <= 0) return;
  int w0 = -1, zmin = INT_MAX, zmax = INT_MIN;
  for (int w = 0; w < nw; ++w) {
    if (st.wsame[w] < 0) continue;
    if (st.wsame[w] == 0) return;
    if (w0 < 0) {
      w0 = w;
    } else if (st.wx[w] != st.wx[w0] || st.wy[w] != st.wy[w0] || st.wcb[w] != st.wcb[w0]) {
      return;
    }
    zmin = min(zmin, st.wzmin[w]);
    zmax = max(zmax, st.wzmax[w]);
  }
  if (w0 < 0) return;
  const SceneGeom g = geom_of(a.c, a.G, st.wi[w0]);
  const int x0 = st.wx[w0], y0 = st.wy[w0];
  const int zlo = max(zmin - 1, 0), zhi = min(zmax + 1, g.dims[2] - 1);
  const bool groups = a.flags[kGroupCount] != 0u;
  int s[9], e[9], total = 0;
  for (int r = 0; r < 9; ++r) {
    const int x = x0 + r / 3 - 1, y = y0 + r % 3 - 1;
    s[r] = e[r] = 0;
    if (x < 0 || x >= g.dims[0] || y < 0 || y >= g.dims[1]) continue;
    const int base = g.cell_base + (x * g.dims[1] + y) * g.dims[2];
    s[r] = (int)__ldg(a.cs + base + zlo);
    e[r] = max(min((int)__ldg(a.cs + base + zhi + 1), a.n), s[r]);
    total += e[r] - s[r];
    if (groups)
      for (int z = zlo; z <= zhi; ++z)
        if (__ldg(a.cell_flags + base + z) >> kCellSlotShift) return;  // a grouped cell
  }
  if (total > cap) return;
  fence_proxy_async_smem();
  mbar_arrive_expect_tx(&st.bar, (uint32_t)total * (uint32_t)sizeof(float4));
  int v = 0;
  for (int r = 0; r < 9; ++r) {
    st.D[r] = v - s[r];
    const int len = e[r] - s[r];
    if (len > 0) bulk_g2s(S + v, a.X + s[r], (uint32_t)len * (uint32_t)sizeof(float4), &st.bar);
    v += len;
  }
  st.ok = 1;
}

// Every thread, after stage_issue and a barrier: waits (bounded) for the
// staged runs.  Returns whether the item reads them; a wait that gave up
// (block-uniform through the barrier) records the error and stops staging.
__device__ __forceinline__ bool stage_wait(StageState& st, const PassArgs& a, uint32_t& phase) {
  if (!st.ok) return false;  // uniform: written before the barrier
  const bool done = mbar_wait_bounded(&st.bar, phase);
  const bool any_failed = __syncthreads_or(!done);
  if (any_failed) {
    if (threadIdx.x == 0) {
      st.failed = 1;
      atomicOr(&a.flags[kErrorWord], (uint32_t)kErrStageTimeout);
    }
    return false;  // st.failed is read only after the next barrier
  }
  phase ^= 1u;
  return true;
}

// Before a block that staged exits: a wait that gave up leaves its copy in
// flight, so wait once more (bounded) for it.
__device__ __forceinline__ void stage_drain(StageState& st, uint32_t phase) {
  if (threadIdx.x == 0 && st.failed) mbar_wait_bounded(&st.bar, phase);
}

// ---- kernels ------------------------------------------------------------------------

// The plain (not grouped) walk of a sparse-kernel particle's window.
// t: the particle's thread slot in the pass's list, which indexes its saved
// masks (the lambda and delta_p passes of an iteration take the same list, so
// a particle keeps its slot; consecutive threads then store and load
// consecutive words).
template <int kKind, class P, class Src>
__device__ __forceinline__ void sparse_visit(const PassArgs& a, const SceneGeom& g, int3 q, const Src& src,
                                             P& p, bool exact, int t, int chunks, HitQueue& hq) {
  if (exact) {
    visit_window(g, a.cs, a.n, q, src, p);  // non-neighbours matter: visit every candidate
  } else if (kKind == kLambda) {
    visit_window_masked(g, a.cs, a.n, q, src, p, a.masks, a.mask_stride, t, hq);  // saves its masks
  } else if ((kKind == kDeltaP || kKind == kDeltaPFinal) && chunks <= kMaskWords) {
    visit_window_saved(g, a.cs, a.n, q, src, p, a.masks, a.mask_stride, t, chunks, hq);  // lambda's masks
  } else {
    visit_window_masked(g, a.cs, a.n, q, src, p, nullptr, 0, t, hq);
  }
}

// The stage's barrier, before first use (thread 0).
__device__ __forceinline__ void stage_init(StageState& st) {
  st.failed = 0;
  st.ok = 0;
  mbar_init(&st.bar, 1u);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One thread slot of the work list (or of all particles) per thread; the
// grid covers every particle, blocks past the list's end return at once.
// PBF_SPARSE_MIN_BLOCKS (a build-time tuning macro): resident blocks per SM the
// compiler must allow for, which caps the sparse kernels' registers.
#ifdef PBF_SPARSE_MIN_BLOCKS
#define PBF_SPARSE_BOUNDS __launch_bounds__(kSparseThreads, PBF_SPARSE_MIN_BLOCKS)
#else
#define PBF_SPARSE_BOUNDS __launch_bounds__(kSparseThreads)
#endif

// kStage: the variant that stages its block's column runs (launched when
// stage_sparse > 0); the other carries no staging code.
template <int kKind, bool kStage>
__global__ void PBF_SPARSE_BOUNDS k_sparse(PassArgs a) {
  using P = typename PassOf<kKind>::type;
  __shared__ StageState st;
  // dynamic shared memory: the hit queue (a.c.queue_sparse chunks per thread),
  // then the stage (a.c.stage_sparse slots, kStage only); the queue is sized
  // per launch so that a small queue leaves the SM's L1 its capacity
  extern __shared__ __align__(16) float4 dyn_smem[];
  uint32_t* q_mask = reinterpret_cast<uint32_t*>(dyn_smem);
  int* q_base = reinterpret_cast<int*>(q_mask + a.c.queue_sparse * kSparseThreads);
  float4* stage = dyn_smem + a.c.queue_sparse * kSparseThreads / 2;
  if (a.dense_all) return;
  const int count = work_count(a);
  if ((int)(blockIdx.x * kSparseThreads) >= count) return;  // uniform over the block
  // the queue is flushed once, at the window's end: a window of more chunks
  // than it holds runs each chunk's hits right away (a flush in mid-window
  // would run for some lanes while the others wait)
  HitQueue hq(q_mask + threadIdx.x, q_base + threadIdx.x, kSparseThreads, 1);
  const int t = blockIdx.x * kSparseThreads + threadIdx.x;
  const bool valid = t < count;
  const int i = valid ? work_particle(a, t) : 0;
  const float4 xi = valid ? a.X[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const SceneGeom g = geom_of(a.c, a.G, valid ? i : 0);
  const int3 q = cell_of(a.c, g, xi);
  int chunks = 0;
  const int total = valid ? window_total_chunks(g, a.cs, a.n, q, chunks) : 0;
  // a window over dense_window candidates that its grouped cells bring back
  // under it is walked here, group by group (no masks)
  const bool grouped = valid && total > a.c.dense_window && a.c.keps2 > 0.f;
  const int entries = grouped ? window_total_grouped(g, a, q) : total;
  // a window over dense_window entries goes to the dense kernel, particle by
  // particle (one list slot each, warp-aggregated): which kernel sums a
  // particle's window depends on its own window only, so results do not
  // depend on the list's order or on the particle's warp-mates
  const bool go_dense = valid && entries > a.c.dense_window;
  const unsigned dmask = __ballot_sync(kFull, go_dense);
  if (dmask) {
    const int lane = threadIdx.x & 31, leader = __ffs(dmask) - 1;
    uint32_t base = 0u;
    if (lane == leader) base = atomicAdd(&a.flags[a.counter], (uint32_t)__popc(dmask));
    base = __shfl_sync(kFull, base, leader);
    if (go_dense) a.dense[base + __popc(dmask & ((1u << lane) - 1u))] = (uint32_t)t;
  }
  const bool active = valid && !go_dense;
  const bool exact = active && exact_path(kKind, a, g, q, i);
  // the block's plain windows staged in shared memory (block-uniform branch)
  const int cap = kStage ? a.c.stage_sparse : 0;
  bool staged = false;
  uint32_t phase = 0u;
  if (kStage && cap > 0) {
    if (threadIdx.x == 0) stage_init(st);
    stage_vote(st, threadIdx.x >> 5, active && !grouped, g, q, i);
    __syncthreads();
    if (threadIdx.x == 0) stage_issue(st, kSparseThreads / 32, a, stage, cap);
    __syncthreads();
    staged = stage_wait(st, a, phase);
  }
  if (active) {
    P p(a, g, xi, i, exact);
    if (!grouped && !exact && chunks <= a.c.queue_sparse) hq.cap = a.c.queue_sparse;
    if (grouped)
      visit_window_grouped(g, a, q, FromGlobal{a.X}, p, 0, entries, hq);
    else if (kStage && staged)
      sparse_visit<kKind>(a, g, q, FromStage{stage, st.D}, p, exact, t, chunks, hq);
    else
      sparse_visit<kKind>(a, g, q, FromGlobal{a.X}, p, exact, t, chunks, hq);
    p.finish(a);
  }
  if (kStage && cap > 0) stage_drain(st, phase);
}

// PBF_DENSE_BLOCKS_PER_SM (a build-time tuning macro, pbf_internal.cuh): the
// dense kernel's resident blocks per SM, which its grid is sized for and its
// registers are capped to.
#define PBF_DENSE_BOUNDS __launch_bounds__(kDenseThreads, PBF_DENSE_BLOCKS_PER_SM)

// kStage: the variant that stages each item's column runs (launched when
// stage_dense > 0); the other carries no staging code.
template <int kKind, bool kStage>
__global__ void PBF_DENSE_BOUNDS k_dense(PassArgs a) {
  using P = typename PassOf<kKind>::type;
  __shared__ float part[kDenseWarps][kMaxFields][32];
  __shared__ StageState st;
  // dynamic shared memory: the hit queue (a.c.queue_dense chunks per thread),
  // then the stage (a.c.stage_dense slots, kStage only)
  extern __shared__ __align__(16) float4 dyn_smem[];
  uint32_t* q_mask = reinterpret_cast<uint32_t*>(dyn_smem);
  int* q_base = reinterpret_cast<int*>(q_mask + a.c.queue_dense * kDenseThreads);
  float4* stage = dyn_smem + a.c.queue_dense * kDenseThreads / 2;
  static_assert(P::kFields <= kMaxFields, "partial-sum fields");
  HitQueue hq(q_mask + threadIdx.x, q_base + threadIdx.x, kDenseThreads, a.c.queue_dense);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cap = kStage ? a.c.stage_dense : 0;
  if (kStage && threadIdx.x == 0 && cap > 0) stage_init(st);
  if (blockIdx.x == 0 && threadIdx.x == 0) {  // their pass has finished
    a.flags[a.next_counter] = 0u;
    a.flags[a.next_item_counter] = 0u;
  }
  // the slots the sparse kernel listed, or all of them, 32 per item
  const int work = work_count(a);
  const uint32_t listed = a.dense_all ? (uint32_t)work : a.flags[a.counter];
  const uint32_t count = (listed + 31) / 32;
  // kSplit warps share an item (each walks one contiguous part of every
  // lane's window); the block runs kDenseWarps / kSplit items at a time.  The
  // staged variant gives each item the whole block.
  const int split = kStage ? kDenseWarps : a.c.dense_split;  // 1, 2, 4 or 8
  const int split_log2 = 31 - __clz(split);
  const int slots = kDenseWarps >> split_log2;
  const int slot = warp >> split_log2, sub = warp & (split - 1);
  // no grouped cell this step: windows are walked as 9 column runs (the same
  // candidates in the same order as cell by cell, with fewer table reads)
  const bool groups = a.c.keps2 > 0.f && a.flags[kGroupCount] != 0u;
  // batches are handed out one block-load at a time by a counter, so a block
  // that drew light batches takes more (batches cost from a few hundred to
  // many thousand candidates); which block computes a batch changes nothing
  __shared__ uint32_t s_first;
  uint32_t phase = 0u;
  for (;;) {
    if (threadIdx.x == 0) s_first = atomicAdd(&a.flags[a.item_counter], (uint32_t)slots);
    __syncthreads();  // also: every thread has read the previous s_first
    const uint32_t first = s_first;
    if (first >= count) break;  // uniform over the block
    const uint32_t item = first + (uint32_t)slot;
    const uint32_t e = item * 32 + lane;
    const bool valid = item < count && e < listed;
    const int t = valid ? (int)(a.dense_all ? e : a.dense[e]) : 0;
    const int i = valid ? work_particle(a, t) : 0;
    const float4 xi = valid ? a.X[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const SceneGeom g = geom_of(a.c, a.G, valid ? i : 0);
    const int3 q = cell_of(a.c, g, xi);
    const bool exact = valid && exact_path(kKind, a, g, q, i);
    // the item's windows staged in shared memory: every warp holds the same
    // 32 particles, so warp 0's vote is the block's (block-uniform branch)
    bool staged = false;
    if (kStage && cap > 0) {
      if (warp == 0) stage_vote(st, 0, valid, g, q, i);
      __syncthreads();  // also: the previous item's reads of the stage are done
      if (threadIdx.x == 0) stage_issue(st, 1, a, stage, cap);
      __syncthreads();
      staged = stage_wait(st, a, phase);
    }
    if (valid) {
      const int total = groups ? window_total_grouped(g, a, q) : window_total(g, a.cs, a.n, q);
      const int lo = (int)(((long long)total * sub) >> split_log2);
      const int hi = (int)(((long long)total * (sub + 1)) >> split_log2);
      P p(a, g, xi, i, exact);
      // a staged window holds no grouped cell: its runs are walked as runs;
      // dense_interleave: the warps take every split-th chunk instead of
      // one contiguous part (windows without grouped cells)
      if (kStage && staged) {
        if (a.c.dense_interleave)
          visit_window_strided(g, a.cs, a.n, q, FromStage{stage, st.D}, p, sub, split, hq);
        else
          visit_window_chunk(g, a.cs, a.n, q, FromStage{stage, st.D}, p, lo, hi, hq);
      } else if (groups) {
        visit_window_grouped(g, a, q, FromGlobal{a.X}, p, lo, hi, hq);
      } else if (a.c.dense_interleave) {
        visit_window_strided(g, a.cs, a.n, q, FromGlobal{a.X}, p, sub, split, hq);
      } else {
        visit_window_chunk(g, a.cs, a.n, q, FromGlobal{a.X}, p, lo, hi, hq);
      }
      p.store(&part[warp][0][lane], 32);
    }
    __syncthreads();
    if (sub == 0 && valid) {
      P p(a, g, xi, i, exact);
      for (int k = 0; k < split; ++k) p.add(&part[slot * split + k][0][lane], 32);
      p.finish(a);
    }
    __syncthreads();
  }
  if (kStage && cap > 0) stage_drain(st, phase);
}

// Also registers every cell holding >= kGroupCell particles (its first
// particle takes a group slot).  flags and cell_flags start at zero.
__global__ void __launch_bounds__(256)
k_reorder(const uint32_t* __restrict__ perm, const float4* __restrict__ pos,
          const float4* __restrict__ vel, const uint32_t* __restrict__ iid, int n, StepConsts c,
          float4* __restrict__ xs, float4* __restrict__ xa, uint32_t* __restrict__ iid_s,
          uint32_t* __restrict__ flags, const uint32_t* __restrict__ skeys,
          const uint32_t* __restrict__ cs, uint32_t* __restrict__ cell_flags, int* __restrict__ grp_cell,
          int* __restrict__ grp_off, int* __restrict__ grp_item_off, int* __restrict__ grp_item_slot) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t key = skeys[k];
  const uint32_t pop = cs[key + 1] - cs[key];
  if ((uint32_t)k == cs[key] && pop >= (uint32_t)kGroupCell) {
    // one slot per such cell (< n / kGroupCell of them) and `pop` pool entries
    // (the pool holds n: the cells' populations sum to <= n)
    const uint32_t slot = atomicAdd(&flags[kGroupCount], 1u);
    grp_cell[slot] = (int)key;
    grp_off[slot] = (int)atomicAdd(&flags[kGroupPool], pop);
    // work items of kGroupChunk particles (< n / kGroupChunk + slots of them)
    const int items = (int)((pop + kGroupChunk - 1) / kGroupChunk);
    const int i0 = (int)atomicAdd(&flags[kGroupItems], (uint32_t)items);
    grp_item_off[slot] = i0;
    for (int t = 0; t < items; ++t) grp_item_slot[i0 + t] = (int)slot;
    atomicOr(&cell_flags[key], (slot + 1u) << kCellSlotShift);
  }
  const uint32_t p = min(perm[k], (uint32_t)(n - 1));  // a permutation of [0, n): the min never binds
  const float4 x = pos[p];
  const float4 v = vel[p];
  const float vx = fmaf(c.dt, c.g[0], v.x), vy = fmaf(c.dt, c.g[1], v.y),
              vz = fmaf(c.dt, c.g[2], v.z);
  xs[k] = x;
  xa[k] = make_float4(fmaf(c.dt, vx, x.x), fmaf(c.dt, vy, x.y), fmaf(c.dt, vz, x.z), x.w);
  iid_s[k] = iid[p];
}

// ---- group tables ----------------------------------------------------------------------

enum GroupsWhat { kGroupsPos = 0, kGroupsLambda = 1, kGroupsXsph = 2 };

constexpr int kGroupThreads = 1024;
constexpr int kGroupWarps = kGroupThreads / 32;
constexpr int kGroupList = 4096;  // groups ranked in shared memory; more: an ordered scan

struct GroupArgs {
  const float4* X;        // positions of the pass
  const float4* V;        // xsph: velocities
  const float* rho;       // xsph: densities
  const float* lambda;    // delta_p: lambda
  const uint32_t* cs;
  const uint32_t* flags;  // flags[kGroupCount]: slots, flags[kGroupItems]: work items
  int n;
  int np;                 // pool entries
  const int* cell;
  const int* off;
  const int* item_off;    // first work item of each slot
  const int* item_slot;   // slot of each work item
  int* done;              // per slot: work items finished (last-block-done; back to 0 after use)
  int* ng;
  int* rep;
  int* cnt;
  float4* pos;
  float4* sum;
  float4* aux;
  int* id;                // hash entry of each particle of a grouped cell
  int* hash;              // owner (k + 1), count, first (0x7fffffff - k), rank: 2 np each; 0 = empty
  int* list;              // pool: entries claimed per slot
  int* list_n;            // per slot: entries claimed
  unsigned* gmax;
  unsigned long long* acc;
  int* zero;              // per slot: every deviation is zero
};

// The key of particle j: the values that enter a pair term non-linearly.
template <int kWhat>
struct GroupKey {
  static constexpr int kWords = kWhat == kGroupsXsph ? 4 : 3;
  uint32_t w[kWords];
  GroupKey() = default;
  __device__ __forceinline__ GroupKey(const GroupArgs& a, int j) {
    const float4 x = a.X[j];
    w[0] = __float_as_uint(x.x), w[1] = __float_as_uint(x.y), w[2] = __float_as_uint(x.z);
    if constexpr (kWhat == kGroupsXsph) w[3] = __float_as_uint(a.rho[j]);
  }
  __device__ __forceinline__ bool operator==(const GroupKey& o) const {
    bool eq = true;
    for (int k = 0; k < kWords; ++k) eq &= w[k] == o.w[k];
    return eq;
  }
  __device__ __forceinline__ uint32_t hash() const {
    uint32_t h = 0x9e3779b9u;
    for (int k = 0; k < kWords; ++k) {
      h ^= w[k] + 0x7f4a7c15u + (h << 6) + (h >> 2);
      h *= 0x85ebca6bu;
    }
    return h ^ (h >> 15);
  }
};

// x - x_rep, and 0 where the two are the same bits (so a group whose members
// share one non-finite value keeps it).
__device__ __forceinline__ float dev_from(float x, float xr) {
  return __float_as_uint(x) == __float_as_uint(xr) ? 0.f : x - xr;
}

// Exclusive prefix of `flag` over the block in thread order; `total` gets the sum.
__device__ __forceinline__ int block_scan(int flag, int* sh, int& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned ball = __ballot_sync(0xffffffffu, flag);
  const int in_warp = __popc(ball & ((1u << lane) - 1u));
  __syncthreads();
  if (lane == 0) sh[warp] = __popc(ball);
  __syncthreads();
  if (warp == 0) {
    const int v = lane < kGroupWarps ? sh[lane] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane < kGroupWarps) sh[32 + lane] = x - v;  // exclusive
    if (lane == kGroupWarps - 1) sh[64] = x;
  }
  __syncthreads();
  total = sh[64];
  return sh[32 + warp] + in_warp;
}

// Exclusive prefix of `v` over the block in thread order; `total` gets the sum.
__device__ __forceinline__ int block_scan_value(int v, int* sh, int& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int w = lane < kGroupWarps ? sh[lane] : 0;
    int y = w;
    for (int o = 1; o < 32; o <<= 1) {
      const int z = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += z;
    }
    if (lane < kGroupWarps) sh[32 + lane] = y - w;  // exclusive
    if (lane == kGroupWarps - 1) sh[64] = y;
  }
  __syncthreads();
  total = sh[64];
  return sh[32 + warp] + x - v;
}

// A grouped cell's particles in work items of kGroupChunk; a kernel takes
// items grid-stride and the block that finishes a slot's last item (counted
// in done[slot], made visible by a fence) runs the slot's finishing step and
// sets the counter back to 0.
struct Item {
  int slot, b, m, k0, k1, t0;
};

__device__ __forceinline__ Item item_of(const GroupArgs& a, int item) {
  Item it;
  it.slot = a.item_slot[item];
  const int cell = a.cell[it.slot];
  it.b = (int)a.cs[cell];
  it.m = max(min((int)a.cs[cell + 1], a.n) - it.b, 0);
  it.k0 = (item - a.item_off[it.slot]) * kGroupChunk;
  it.k1 = min(it.k0 + kGroupChunk, it.m);
  it.t0 = a.off[it.slot];
  return it;
}

// After a block's share of an item: whether it finished the slot's last item.
__device__ __forceinline__ bool last_item(const GroupArgs& a, const Item& it, int* s_last) {
  __threadfence();  // this block's writes, before the count that may let another block read them
  __syncthreads();
  if (threadIdx.x == 0) {
    const int items = (it.m + kGroupChunk - 1) / kGroupChunk;
    *s_last = atomicAdd(&a.done[it.slot], 1) == items - 1;
  }
  __syncthreads();
  if (*s_last) __threadfence();
  return *s_last;
}

// Inserts the item's particles into the slot's hash table (2 entries per
// particle of the cell, so every key finds an entry; integer atomics only),
// kUnroll probe chains per thread in flight.  The block that finishes the
// slot numbers the groups in order of their first particle (by counting in
// shared memory, or for over kGroupList groups by an ordered block scan),
// writes rep, cnt, pos (and for xsph aux = the first particle's velocity and
// sum.w = its density), h_rank, ng, and clears the claimed entries.
template <int kWhat>
__global__ void __launch_bounds__(kGroupThreads) k_group_insert(GroupArgs a) {
  __shared__ int sh[80];
  __shared__ int s_last;
  __shared__ int s_buf[2 * kGroupList];
  const int items = (int)a.flags[kGroupItems];
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const Item it = item_of(a, item);
    const int H = 2 * it.m;
    int* h_owner = a.hash + 2 * it.t0;
    int* h_cnt = h_owner + 2 * a.np;
    int* h_first = h_owner + 4 * a.np;
    int* h_rank = h_owner + 6 * a.np;
    int* list = a.list + it.t0;
    constexpr int kUnroll = 4;
    for (int k0 = it.k0 + threadIdx.x; k0 < it.k1; k0 += kUnroll * kGroupThreads) {
      int found[kUnroll];
      GroupKey<kWhat> key[kUnroll];
      int h[kUnroll], o[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        const int k = min(k0 + u * kGroupThreads, it.k1 - 1);
        key[u] = GroupKey<kWhat>(a, it.b + k);
        h[u] = (int)(key[u].hash() % (uint32_t)H);
      }
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) o[u] = *(volatile int*)&h_owner[h[u]] - 1;
#pragma unroll
      for (int u = 0; u < kUnroll; ++u)  // the common case: the first entry holds the key
        found[u] = o[u] >= 0 && GroupKey<kWhat>(a, it.b + o[u]) == key[u] ? h[u] : -1;
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        const int k = k0 + u * kGroupThreads;
        if (k < it.k1 && found[u] < 0) {
          int hh = h[u];
          for (int probe = 0; probe < H; ++probe, hh = hh + 1 == H ? 0 : hh + 1) {
            int ow = *(volatile int*)&h_owner[hh] - 1;
            if (ow < 0) {
              ow = atomicCAS(&h_owner[hh], 0, k + 1) - 1;
              if (ow < 0) {
                found[u] = hh;  // claimed: a new group
                list[atomicAdd(&a.list_n[it.slot], 1)] = hh;
                break;
              }
            }
            if (GroupKey<kWhat>(a, it.b + ow) == key[u]) {
              found[u] = hh;
              break;
            }
          }
          // H = 2m entries for at most m keys: a probe always ends
        }
        if (k < it.k1) {
          const unsigned act = __activemask(), same = __match_any_sync(act, found[u]);
          if ((threadIdx.x & 31) == __ffs(same) - 1) {
            atomicAdd(&h_cnt[found[u]], __popc(same));
            atomicMax(&h_first[found[u]], 0x7fffffff - k);  // the lowest lane holds the lowest k
          }
          a.id[it.b + k] = found[u];
        }
      }
    }
    if (!last_item(a, it, &s_last)) continue;
    // ---- the slot's last item is in: number the groups ----
    // read through L2: other blocks wrote these
    int ng = __ldcg(&a.list_n[it.slot]);
    int* s_list = s_buf;
    int* s_first = s_buf + kGroupList;
    if (ng <= kGroupList) {
      for (int e = threadIdx.x; e < ng; e += kGroupThreads) {
        const int hh = __ldcg(&list[e]);
        s_list[e] = hh;
        s_first[e] = 0x7fffffff - __ldcg(&h_first[hh]);
      }
      __syncthreads();
      for (int e = threadIdx.x; e < ng; e += kGroupThreads) {
        const int f = s_first[e], hh = s_list[e];
        int r = 0;
        for (int u = 0; u < ng; ++u) r += s_first[u] < f;
        h_rank[hh] = r;
        a.rep[it.t0 + r] = it.b + f;
        a.cnt[it.t0 + r] = __ldcg(&h_cnt[hh]);
        a.pos[it.t0 + r] = a.X[it.b + f];
        if constexpr (kWhat == kGroupsXsph) {
          a.aux[it.t0 + r] = a.V[it.b + f];
          a.sum[it.t0 + r].w = a.rho[it.b + f];
        }
      }
    } else {
      ng = 0;
      for (int k0 = 0; k0 < it.m; k0 += kGroupThreads) {
        const int k = k0 + threadIdx.x;
        const int hh = k < it.m ? __ldcg(&a.id[it.b + k]) : 0;
        const bool first = k < it.m && 0x7fffffff - __ldcg(&h_first[hh]) == k;
        int total;
        const int r = ng + block_scan(first, sh, total);
        if (first) {
          h_rank[hh] = r;
          a.rep[it.t0 + r] = it.b + k;
          a.cnt[it.t0 + r] = __ldcg(&h_cnt[hh]);
          a.pos[it.t0 + r] = a.X[it.b + k];
          if constexpr (kWhat == kGroupsXsph) {
            a.aux[it.t0 + r] = a.V[it.b + k];
            a.sum[it.t0 + r].w = a.rho[it.b + k];
          }
        }
        ng += total;
      }
    }
    __syncthreads();
    // clear the claimed entries for the next pass (h_rank stays: the sums read it)
    const int claimed = __ldcg(&a.list_n[it.slot]);
    for (int e = threadIdx.x; e < claimed; e += kGroupThreads) {
      const int hh = __ldcg(&list[e]);
      h_owner[hh] = 0;
      h_cnt[hh] = 0;
      h_first[hh] = 0;
    }
    if (threadIdx.x == 0) {
      a.ng[it.slot] = ng;
      a.list_n[it.slot] = 0;
      a.done[it.slot] = 0;
    }
    __syncthreads();
  }
}

// Deviation of particle j (cell-relative k) from its group's first particle,
// component c: lambda (kGroupsLambda) or velocity (kGroupsXsph).
template <int kWhat>
__device__ __forceinline__ float group_dev(const GroupArgs& a, const Item& it, int k, int g, int c) {
  if constexpr (kWhat == kGroupsLambda) {
    return dev_from(a.lambda[it.b + k], a.lambda[a.rep[it.t0 + g]]);
  } else {
    const float4 v = a.V[it.b + k], r = a.aux[it.t0 + g];
    return c == 0 ? dev_from(v.x, r.x) : (c == 1 ? dev_from(v.y, r.y) : dev_from(v.z, r.z));
  }
}

// Fixed-point sums over each group of (value - the group's first particle's
// value), two kernels.  k_group_devmax: the largest |deviation| per group
// (atomicMax on the float bits; +inf marks a non-finite deviation); the last
// block of a slot sets ng = -1 on a non-finite one and zero[slot] when every
// deviation is 0.  k_group_devsum: each deviation scaled by 2^sh, sh from the
// group's bound max|dev| * count < 2^62, added as a 64-bit integer (order-
// free, exact to 2^-62 of the bound); the last block writes the sums
// (lambda: sum = (lambda_rep, sum dev); xsph: sum.xyz) and clears gmax / acc.
template <int kWhat>
__global__ void __launch_bounds__(kGroupThreads) k_group_devmax(GroupArgs a) {
  constexpr int C = kWhat == kGroupsLambda ? 1 : 3;
  __shared__ int s_last, s_flag;
  const int items = (int)a.flags[kGroupItems];
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const Item it = item_of(a, item);
    const int* h_rank = a.hash + 2 * it.t0 + 6 * a.np;
    const bool grouped = a.ng[it.slot] > 0;
    for (int k = it.k0 + threadIdx.x; grouped && k < it.k1; k += kGroupThreads) {
      const int g = h_rank[a.id[it.b + k]];
      float d = 0.f;
      bool fin = true;
      for (int c = 0; c < C; ++c) {
        const float e = group_dev<kWhat>(a, it, k, g, c);
        fin &= isfinite(e);
        d = fmaxf(d, fabsf(e));
      }
      const unsigned bits = fin ? __float_as_uint(d) : 0x7f800000u;
      const unsigned act = __activemask(), same = __match_any_sync(act, g);
      const unsigned mx = __reduce_max_sync(same, bits);
      if ((threadIdx.x & 31) == __ffs(same) - 1 && mx) atomicMax(&a.gmax[it.t0 + g], mx);
    }
    if (!last_item(a, it, &s_last)) continue;
    const int ng = a.ng[it.slot];
    if (threadIdx.x == 0) s_flag = 0;
    __syncthreads();
    for (int g = threadIdx.x; g < ng; g += kGroupThreads) {
      const unsigned mx = __ldcg(&a.gmax[it.t0 + g]);
      if (!isfinite(__uint_as_float(mx))) atomicOr(&s_flag, 1);
      if (mx) atomicOr(&s_flag, 2);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      if (s_flag & 1) a.ng[it.slot] = -1;
      a.zero[it.slot] = !(s_flag & 2);
      a.done[it.slot] = 0;
    }
    if (s_flag & 1)  // ungrouped: clear the bounds now (devsum skips the slot)
      for (int g = threadIdx.x; g < ng; g += kGroupThreads) a.gmax[it.t0 + g] = 0u;
    __syncthreads();
  }
}

template <int kWhat>
__global__ void __launch_bounds__(kGroupThreads) k_group_devsum(GroupArgs a) {
  constexpr int C = kWhat == kGroupsLambda ? 1 : 3;
  __shared__ int s_last;
  const int items = (int)a.flags[kGroupItems];
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const Item it = item_of(a, item);
    const int* h_rank = a.hash + 2 * it.t0 + 6 * a.np;
    const bool add = a.ng[it.slot] > 0 && !a.zero[it.slot];
    for (int k = it.k0 + threadIdx.x; add && k < it.k1; k += kGroupThreads) {
      const int g = h_rank[a.id[it.b + k]];
      const float mx = __uint_as_float(a.gmax[it.t0 + g]);
      int e = 0;
      if (mx > 0.f) frexpf(mx, &e);                            // mx < 2^e
      const int sh = 62 - e - (32 - __clz(a.cnt[it.t0 + g]));  // |sum| 2^sh < 2^62
      const unsigned act = __activemask(), same = __match_any_sync(act, g);
      for (int c = 0; c < C; ++c) {
        // |dev| 2^sh < 2^62 is a float without overflow; the scaling is exact
        long long q = __float2ll_rn(ldexpf(group_dev<kWhat>(a, it, k, g, c), sh));
        if (same == 0xffffffffu) {  // a full warp of one group; integer sums: any order, same result
          for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
          if ((threadIdx.x & 31) == 0 && q) atomicAdd(&a.acc[3 * (it.t0 + g) + c], (unsigned long long)q);
        } else if (q) {
          atomicAdd(&a.acc[3 * (it.t0 + g) + c], (unsigned long long)q);
        }
      }
    }
    if (!last_item(a, it, &s_last)) continue;
    const int ng = a.ng[it.slot];
    for (int g = threadIdx.x; g < ng; g += kGroupThreads) {
      const float mx = __uint_as_float(a.gmax[it.t0 + g]);  // from the previous kernel
      int e = 0;
      if (mx > 0.f) frexpf(mx, &e);
      const int sh = 62 - e - (32 - __clz(a.cnt[it.t0 + g]));
      float s3[3];
      for (int c = 0; c < C; ++c) {
        s3[c] = (float)ldexp((double)(long long)__ldcg(&a.acc[3 * (it.t0 + g) + c]), -sh);
        a.acc[3 * (it.t0 + g) + c] = 0ull;
      }
      a.gmax[it.t0 + g] = 0u;
      if constexpr (kWhat == kGroupsLambda) {
        a.sum[it.t0 + g] = make_float4(a.lambda[a.rep[it.t0 + g]], s3[0], 0.f, 0.f);
      } else {
        float4& s4 = a.sum[it.t0 + g];
        s4.x = s3[0], s4.y = s3[1], s4.z = s3[2];
      }
    }
    if (threadIdx.x == 0) a.done[it.slot] = 0;
    __syncthreads();
  }
}

// ---- work lists: one computing particle per position group -----------------------------

static_assert(kWorkThreads == kGroupThreads, "the work-list kernels use the group kernels' block scan");

// Marks the followers of the current position groups (the group tables the
// lambda pass of this iteration just built): follow[i] = the group's first
// particle when particle i of a grouped cell is not that particle, else -1;
// blocks[b] = the computing particles of block b.  The block that finishes
// last turns blocks[] into exclusive offsets (so the list is in cell order).
__global__ void __launch_bounds__(kWorkThreads)
k_work_mark(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ cell_flags,
            const int* __restrict__ grp_n, const int* __restrict__ grp_off, const int* __restrict__ grp_id,
            const int* __restrict__ grp_hash, const int* __restrict__ grp_rep, int np, int n,
            int* __restrict__ follow, int* __restrict__ blocks, uint32_t* __restrict__ flags) {
  __shared__ int sh[80];
  __shared__ int s_last;
  if (flags[kGroupCount] == 0u) {  // no grouped cell this step: every particle computes, in order
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      flags[kWorkCount] = (uint32_t)n;
      flags[kWorkIdentity] = 1u;
    }
    return;
  }
  const int i = blockIdx.x * kWorkThreads + threadIdx.x;
  int r = -1;
  if (i < n) {
    const uint32_t sl = cell_flags[skeys[i]] >> kCellSlotShift;
    if (sl) {
      const int slot = (int)sl - 1;
      if (grp_n[slot] > 0) {
        // the particle's hash entry -> its group's rank -> the group's first particle
        const int t0 = grp_off[slot];
        const int rank = grp_hash[2 * t0 + 6 * np + grp_id[i]];
        const int rep = grp_rep[t0 + rank];
        if (rep != i) r = rep;
      }
    }
    follow[i] = r;
  }
  const int cnt = __syncthreads_count(i < n && r < 0);
  if (threadIdx.x == 0) blocks[blockIdx.x] = cnt;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&flags[kWorkDone], 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // the last block: exclusive offsets of every block, in chunks of kWorkThreads
  int carry = 0;
  for (int b0 = 0; b0 < (int)gridDim.x; b0 += kWorkThreads) {
    const int b = b0 + threadIdx.x;
    const int v = b < (int)gridDim.x ? __ldcg(&blocks[b]) : 0;
    int total;
    const int ex = block_scan_value(v, sh, total);
    if (b < (int)gridDim.x) blocks[b] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) {
    flags[kWorkCount] = (uint32_t)carry;
    flags[kWorkDone] = 0u;
  }
}

// list[blocks[b] + rank] = i for the computing particles of block b, in order.
__global__ void __launch_bounds__(kWorkThreads)
k_work_list(const int* __restrict__ follow, const int* __restrict__ blocks, int n, int* __restrict__ list,
            const uint32_t* __restrict__ flags) {
  __shared__ int sh[80];
  if (flags[kWorkIdentity]) return;
  const int i = blockIdx.x * kWorkThreads + threadIdx.x;
  const bool keep = i < n && follow[i] < 0;
  int total;
  const int rank = block_scan(keep, sh, total);
  if (keep) list[blocks[blockIdx.x] + rank] = i;
}

// The followers take their group's results.
template <int kKind>
__global__ void __launch_bounds__(256)
k_follow(const int* __restrict__ follow, int n, StepConsts c, const float4* __restrict__ X, float* __restrict__ lambda,
         float* __restrict__ rho, float4* __restrict__ T, const float4* __restrict__ xs,
         const uint32_t* __restrict__ iid_s, float4* __restrict__ npos, float4* __restrict__ vel,
         float4* __restrict__ pos, uint32_t* __restrict__ iid, const uint32_t* __restrict__ skeys,
         uint32_t* __restrict__ cell_flags, uint32_t* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || flags[kWorkIdentity]) return;
  const int r = follow[i];
  if (r < 0) return;
  if constexpr (kKind == kLambda) {
    lambda[i] = lambda[r];
    rho[i] = rho[r];
  } else if constexpr (kKind == kDeltaP) {
    const float4 t = T[r];
    T[i] = make_float4(t.x, t.y, t.z, X[i].w);
  } else {
    // DeltaPPass<true>::finish with the group's final position
    const float4 xf = npos[r];
    const float4 x0 = xs[i];
    npos[i] = make_float4(xf.x, xf.y, xf.z, x0.w);
    const float4 v = make_float4((xf.x - x0.x) * c.inv_dt, (xf.y - x0.y) * c.inv_dt, (xf.z - x0.z) * c.inv_dt, 0.f);
    vel[i] = v;
    if (!isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z)) {
      atomicOr(&cell_flags[skeys[i]], (uint32_t)kCellVelNonFinite);
      atomicOr(&flags[kFlagXsphExact], 1u);
    }
    pos[i] = x0;
    iid[i] = iid_s[i];
  }
}

// ---- current-cell order ---------------------------------------------------------------

// The pass's computing particles (its list, or every particle) by the cell
// they are in now: count (integer atomics: the counts are exact, the rank
// inside a cell is arbitrary), exclusive scan over cells, scatter.  Consecutive
// particles of the resulting list mostly share a window, so a warp's lanes
// load the same candidates and run similar loops.  A particle's result does
// not depend on its place in the list (sparse / dense routing is per
// particle), so the arbitrary ranks leave results bitwise reproducible.
__global__ void __launch_bounds__(256) k_bucket_count(PassArgs a, uint32_t* __restrict__ bcnt,
                                                      uint2* __restrict__ bent) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int count = work_count(a);
  if (t == 0) a.flags[kBucketCount] = (uint32_t)count;
  if (t >= count) return;
  const int i = work_particle(a, t);
  const SceneGeom g = geom_of(a.c, a.G, i);
  const int3 q = cell_of(a.c, g, a.X[i]);
  const uint32_t cell = (uint32_t)cell_index(g, q.x, q.y, q.z);
  // one atomic per cell and warp (particles piled into a cell share it)
  const unsigned act = __activemask();
  const unsigned same = __match_any_sync(act, cell);
  const int lane = threadIdx.x & 31, leader = __ffs(same) - 1;
  uint32_t base = 0u;
  if (lane == leader) base = atomicAdd(&bcnt[cell], (uint32_t)__popc(same));
  base = __shfl_sync(same, base, leader);
  bent[t] = make_uint2(cell, base + (uint32_t)__popc(same & ((1u << lane) - 1u)));
}

__global__ void __launch_bounds__(256) k_bucket_scatter(PassArgs a, const uint32_t* __restrict__ bstart,
                                                        const uint2* __restrict__ bent, int* __restrict__ bucket) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= work_count(a)) return;
  const uint2 e = bent[t];
  bucket[bstart[e.x] + e.y] = work_particle(a, t);
}

GroupArgs group_args(const SolverScratch& s, const float4* X, const float4* V, int n) {
  GroupArgs a;
  a.X = X;
  a.V = V;
  a.rho = s.rho;
  a.lambda = s.lambda;
  a.cs = s.cell_start;
  a.flags = s.flags;
  a.n = n;
  a.np = s.grp_pool;
  a.cell = s.grp_cell;
  a.off = s.grp_off;
  a.item_off = s.grp_item_off;
  a.item_slot = s.grp_item_slot;
  a.done = s.grp_done;
  a.ng = s.grp_n;
  a.rep = s.grp_rep;
  a.cnt = s.grp_cnt;
  a.pos = s.grp_pos;
  a.sum = s.grp_sum;
  a.aux = s.grp_aux;
  a.id = s.grp_id;
  a.hash = s.grp_hash;
  a.list = s.grp_list;
  a.list_n = s.grp_list_n;
  a.gmax = s.grp_max;
  a.acc = s.grp_acc;
  a.zero = s.grp_zero;
  return a;
}

// kGroupsPos: the lambda pass's groups.  kGroupsLambda: their lambda sums for
// delta_p.  kGroupsXsph: the (position, density) groups and velocity sums.
template <int kWhat>
cudaError_t launch_groups(const StepConsts& c, const SolverScratch& s, const float4* X, const float4* V, int n,
                          cudaStream_t stream) {
  if (n < kGroupCell) return cudaSuccess;  // no cell can hold kGroupCell particles
  const GroupArgs a = group_args(s, X, V, n);
  const int grid = c.dense_grid;
  if constexpr (kWhat != kGroupsLambda) k_group_insert<kWhat><<<grid, kGroupThreads, 0, stream>>>(a);
  if constexpr (kWhat != kGroupsPos) {
    k_group_devmax<kWhat><<<grid, kGroupThreads, 0, stream>>>(a);
    k_group_devsum<kWhat><<<grid, kGroupThreads, 0, stream>>>(a);
  }
  return cudaGetLastError();
}

PassArgs base_args(const StepConsts& c, const Geometry& G, const float4* X, const uint32_t* cs,
                   int n, const SolverScratch& s, int pass) {
  PassArgs a = {};
  a.c = c;
  a.G = G;
  a.X = X;
  a.cs = cs;
  a.n = n;
  a.dense_all = c.dense_all >= 0 ? c.dense_all : n < kDenseAllBelow;
  a.counter = kDenseCount0 + (pass & 1);
  a.next_counter = kDenseCount0 + ((pass + 1) & 1);
  a.item_counter = kItemCount0 + (pass & 1);
  a.next_item_counter = kItemCount0 + ((pass + 1) & 1);
  a.flags = s.flags;
  a.dense = s.dense;
  a.masks = s.masks;
  a.mask_stride = s.mask_stride;
  a.cell_flags = s.cell_flags;
  a.skeys = s.keys_sorted;
  a.lambda = s.lambda;
  a.rho = s.rho;
  a.grp_off = s.grp_off;
  a.grp_n = s.grp_n;
  a.grp_cnt = s.grp_cnt;
  a.grp_pos = s.grp_pos;
  a.grp_sum = s.grp_sum;
  a.grp_aux = s.grp_aux;
  a.count_word = kWorkCount;
  a.identity_word = kWorkIdentity;
  return a;
}

// Makes the pass take its computing particles in current-cell order: buckets
// them (kBucketLaunches launches) and points the pass at the buckets.
cudaError_t bucket_by_cell(PassArgs& a, const SolverScratch& s, int n, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(s.bcnt, 0, sizeof(uint32_t) * (a.c.cells + 1), stream);
  if (e != cudaSuccess) return e;
  const int blocks = (n + 255) / 256;
  k_bucket_count<<<blocks, 256, 0, stream>>>(a, s.bcnt, s.bent);
  if ((e = exclusive_scan(s.bcnt, s.bstart, a.c.cells + 1, s.bpart, stream)) != cudaSuccess) return e;
  k_bucket_scatter<<<blocks, 256, 0, stream>>>(a, s.bstart, s.bent, s.bucket);
  a.list = s.bucket;
  a.count_word = kBucketCount;
  a.identity_word = -1;
  return cudaGetLastError();
}

// The delta_p passes of an iteration take the lambda pass's buckets (same positions).
void use_buckets(PassArgs& a, const SolverScratch& s) {
  a.list = s.bucket;
  a.count_word = kBucketCount;
  a.identity_word = -1;
}

template <int kKind>
cudaError_t run_pass(const PassArgs& a, cudaStream_t stream) {
  // dynamic shared memory: the hit queue (8 bytes per chunk and thread), then the stage
  const size_t sparse_queue = (size_t)8 * a.c.queue_sparse * kSparseThreads;
  const size_t dense_queue = (size_t)8 * a.c.queue_dense * kDenseThreads;
  const size_t sparse_smem = sizeof(float4) * (size_t)max(a.c.stage_sparse, 0);
  const size_t dense_smem = sizeof(float4) * (size_t)max(a.c.stage_dense, 0);
  const int sparse_blocks = (a.n + kSparseThreads - 1) / kSparseThreads;
  if (a.dense_all) {
    // else the sparse kernel has nothing to do
  } else if (sparse_smem) {
    k_sparse<kKind, true><<<sparse_blocks, kSparseThreads, sparse_queue + sparse_smem, stream>>>(a);
  } else {
    k_sparse<kKind, false><<<sparse_blocks, kSparseThreads, sparse_queue, stream>>>(a);
  }
  if (dense_smem)
    k_dense<kKind, true><<<a.c.dense_grid, kDenseThreads, dense_queue + dense_smem, stream>>>(a);
  else
    k_dense<kKind, false><<<a.c.dense_grid, kDenseThreads, dense_queue, stream>>>(a);
  return cudaGetLastError();
}

template <int kKind>
cudaError_t allow_stage(int bytes) {
  cudaError_t e = cudaFuncSetAttribute(k_sparse<kKind, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_dense<kKind, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}

}  // namespace

// Lets the staged pass kernels take their largest hit queue and up to
// kStageMax staged slots of dynamic shared memory (the current device; call
// before any capture).
cudaError_t set_pass_kernel_attributes() {
  const int queue = 8 * max(kMaxQueueSparse * kSparseThreads, kMaxQueueDense * kDenseThreads);
  const int bytes = (int)sizeof(float4) * kStageMax + queue;
  cudaError_t e = allow_stage<kLambda>(bytes);
  if (e == cudaSuccess) e = allow_stage<kDeltaP>(bytes);
  if (e == cudaSuccess) e = allow_stage<kDeltaPFinal>(bytes);
  if (e == cudaSuccess) e = allow_stage<kXsph>(bytes);
  return e;
}

cudaError_t reorder(const StepConsts& c, const uint32_t* perm, const float4* pos, const float4* vel,
                    const uint32_t* iid, int n, SolverScratch& s, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(s.cell_flags, 0, sizeof(uint32_t) * (c.cells + 1), stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(s.flags, 0, sizeof(uint32_t) * kNumFlags, stream);
  if (e != cudaSuccess) return e;
  k_reorder<<<(n + 255) / 256, 256, 0, stream>>>(perm, pos, vel, iid, n, c, s.xs, s.xa, s.iid_s,
                                                  s.flags, s.keys_sorted, s.cell_start, s.cell_flags,
                                                  s.grp_cell, s.grp_off, s.grp_item_off, s.grp_item_slot);
  return cudaGetLastError();
}

namespace {

// Whether the lambda / delta_p passes run on work lists (groups exist only
// from kGroupCell particles on, and the zero gradient of co-located particles
// needs kernel_eps > 0).
bool use_work_list(const StepConsts& c, int n) { return n >= kGroupCell && c.keps2 > 0.f; }

cudaError_t launch_work_list(const SolverScratch& s, int n, cudaStream_t stream) {
  const int blocks = (n + kWorkThreads - 1) / kWorkThreads;
  k_work_mark<<<blocks, kWorkThreads, 0, stream>>>(s.keys_sorted, s.cell_flags, s.grp_n, s.grp_off, s.grp_id,
                                                   s.grp_hash, s.grp_rep, s.grp_pool, n, s.work_follow,
                                                   s.work_blocks, s.flags);
  k_work_list<<<blocks, kWorkThreads, 0, stream>>>(s.work_follow, s.work_blocks, n, s.work_list, s.flags);
  return cudaGetLastError();
}

template <int kKind>
cudaError_t launch_follow(const StepConsts& c, const SolverScratch& s, const float4* X, int n, float4* T,
                          float4* pos, float4* npos, float4* vel, uint32_t* iid, cudaStream_t stream) {
  k_follow<kKind><<<(n + 255) / 256, 256, 0, stream>>>(s.work_follow, n, c, X, s.lambda, s.rho, T, s.xs, s.iid_s,
                                                       npos, vel, pos, iid, s.keys_sorted, s.cell_flags, s.flags);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_lambda(const StepConsts& c, const Geometry& G, const float4* X, const uint32_t* cs, int n,
                          const SolverScratch& s, int pass, cudaStream_t stream) {
  cudaError_t e = launch_groups<kGroupsPos>(c, s, X, nullptr, n, stream);
  if (e != cudaSuccess) return e;
  const bool wl = use_work_list(c, n);
  if (wl && (e = launch_work_list(s, n, stream)) != cudaSuccess) return e;
  PassArgs a = base_args(c, G, X, cs, n, s, pass);
  if (wl) a.list = s.work_list;
  if (c.order && (e = bucket_by_cell(a, s, n, stream)) != cudaSuccess) return e;
  if ((e = run_pass<kLambda>(a, stream)) != cudaSuccess) return e;
  return wl ? launch_follow<kLambda>(c, s, X, n, nullptr, nullptr, nullptr, nullptr, nullptr, stream) : cudaSuccess;
}

cudaError_t launch_delta_p(const StepConsts& c, const Geometry& G, const float4* X, const uint32_t* cs, int n,
                           const SolverScratch& s, int pass, float4* T, cudaStream_t stream) {
  cudaError_t e = launch_groups<kGroupsLambda>(c, s, X, nullptr, n, stream);
  if (e != cudaSuccess) return e;
  const bool wl = use_work_list(c, n);
  PassArgs a = base_args(c, G, X, cs, n, s, pass);
  a.T = T;
  if (wl) a.list = s.work_list;
  if (c.order) use_buckets(a, s);
  if ((e = run_pass<kDeltaP>(a, stream)) != cudaSuccess) return e;
  return wl ? launch_follow<kDeltaP>(c, s, X, n, T, nullptr, nullptr, nullptr, nullptr, stream) : cudaSuccess;
}

cudaError_t launch_delta_p_final(const StepConsts& c, const Geometry& G, const float4* X, const uint32_t* cs, int n,
                                 const SolverScratch& s, int pass, float4* pos, float4* npos,
                                 float4* vel, uint32_t* iid, cudaStream_t stream) {
  cudaError_t e = launch_groups<kGroupsLambda>(c, s, X, nullptr, n, stream);
  if (e != cudaSuccess) return e;
  const bool wl = use_work_list(c, n);
  PassArgs a = base_args(c, G, X, cs, n, s, pass);
  a.xs = s.xs;
  a.iid_s = s.iid_s;
  a.npos = npos;
  a.vel = vel;
  a.pos = pos;
  a.iid = iid;
  if (wl) a.list = s.work_list;
  if (c.order) use_buckets(a, s);
  if ((e = run_pass<kDeltaPFinal>(a, stream)) != cudaSuccess) return e;
  return wl ? launch_follow<kDeltaPFinal>(c, s, X, n, nullptr, pos, npos, vel, iid, stream) : cudaSuccess;
}

// ---- vorticity confinement ---------------------------------------------------------------

namespace {

// Spiky gradient grad W(r) for kernel_eps <= |r| < h (else zero), r = x_i - x_j.
__device__ __forceinline__ bool spiky_grad(const StepConsts& c, float ex, float ey, float ez, float& gx,
                                           float& gy, float& gz) {
  const float r2 = dist2(ex, ey, ez);
  if (!(r2 < c.h2) || r2 < c.keps2) return false;
  const float ir = rsqrtf(r2);
  const float t = c.h - r2 * ir;
  const float sc = c.spiky_coef * t * t * ir;
  gx = sc * ex, gy = sc * ey, gz = sc * ez;
  return true;
}

struct VortOmega {
  const StepConsts& c;
  const float4* __restrict__ U;
  float4 xi, ui;
  int i;
  float wx = 0.f, wy = 0.f, wz = 0.f;
  __device__ __forceinline__ void visit(float4 xj, int j) {
    float gx, gy, gz;
    if (j == i || !spiky_grad(c, xi.x - xj.x, xi.y - xj.y, xi.z - xj.z, gx, gy, gz)) return;
    const float4 uj = __ldg(U + j);
    const float dx = uj.x - ui.x, dy = uj.y - ui.y, dz = uj.z - ui.z;
    wx += dy * gz - dz * gy;
    wy += dz * gx - dx * gz;
    wz += dx * gy - dy * gx;
  }
};

struct VortEta {
  const StepConsts& c;
  const float4* __restrict__ W;
  float4 xi;
  int i;
  float ex = 0.f, ey = 0.f, ez = 0.f;
  __device__ __forceinline__ void visit(float4 xj, int j) {
    float gx, gy, gz;
    if (j == i || !spiky_grad(c, xi.x - xj.x, xi.y - xj.y, xi.z - xj.z, gx, gy, gz)) return;
    const float m = __ldg(W + j).w;
    ex += m * gx;
    ey += m * gy;
    ez += m * gz;
  }
};

__global__ void __launch_bounds__(128)
k_vort_omega(StepConsts c, Geometry G, const float4* __restrict__ X, const float4* __restrict__ U,
             const uint32_t* __restrict__ cs, int n, float4* __restrict__ W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = X[i];
  const SceneGeom g = geom_of(c, G, i);
  VortOmega p{c, U, xi, U[i], i};
  visit_window(g, cs, n, cell_of(c, g, xi), FromGlobal{X}, p);
  W[i] = make_float4(p.wx, p.wy, p.wz, sqrtf(dist2(p.wx, p.wy, p.wz)));
}

__global__ void __launch_bounds__(128)
k_vort_force(StepConsts c, Geometry G, const float4* __restrict__ X, const float4* __restrict__ W,
             const uint32_t* __restrict__ cs, int n, float4* __restrict__ U) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = X[i];
  const SceneGeom g = geom_of(c, G, i);
  VortEta p{c, W, xi, i};
  visit_window(g, cs, n, cell_of(c, g, xi), FromGlobal{X}, p);
  const float len = sqrtf(dist2(p.ex, p.ey, p.ez));
  if (!(len > 0.f) || !isfinite(len)) return;
  const float nx = p.ex / len, ny = p.ey / len, nz = p.ez / len;
  const float4 w = W[i];
  const float s = c.dt * c.vort_eps;
  float4 u = U[i];
  u.x += s * (ny * w.z - nz * w.y);
  u.y += s * (nz * w.x - nx * w.z);
  u.z += s * (nx * w.y - ny * w.x);
  U[i] = u;
}

}  // namespace

cudaError_t launch_vorticity(const StepConsts& c, const Geometry& G, const float4* X, const uint32_t* cs, int n,
                             const SolverScratch& s, float4* NV, cudaStream_t stream) {
  const int blocks = (n + 127) / 128;
  k_vort_omega<<<blocks, 128, 0, stream>>>(c, G, X, NV, cs, n, s.xb);
  k_vort_force<<<blocks, 128, 0, stream>>>(c, G, X, s.xb, cs, n, NV);
  return cudaGetLastError();
}

cudaError_t launch_xsph(const StepConsts& c, const Geometry& G, const float4* X, const float4* V, const uint32_t* cs,
                        int n, const SolverScratch& s, int pass, float4* NV, cudaStream_t stream) {
  cudaError_t e = launch_groups<kGroupsXsph>(c, s, X, V, n, stream);
  if (e != cudaSuccess) return e;
  PassArgs a = base_args(c, G, X, cs, n, s, pass);
  a.V = V;
  a.NV = NV;
  if (c.order && (e = bucket_by_cell(a, s, n, stream)) != cudaSuccess) return e;
  return run_pass<kXsph>(a, stream);
}

}  // namespace pbf

namespace pbf {

int pass_launches(const StepConsts& c, int n) {
  const bool all = c.dense_all >= 0 ? c.dense_all != 0 : n < kDenseAllBelow;
  return all ? 1 : 2;
}

// launch_groups: 1 launch before each lambda pass, 2 before each delta_p pass, 3 before xsph;
// with work lists 2 more before each lambda pass and one follower launch after
// each lambda and delta_p pass.
int group_launches(const StepConsts& c, int n, int niter) {
  if (n < kGroupCell) return 0;
  return 3 * niter + 3 + (use_work_list(c, n) ? 4 * niter : 0);
}

}  // namespace pbf
