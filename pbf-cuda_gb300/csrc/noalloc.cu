// noalloc.cu — pbf_step_noalloc: one PBF step that allocates nothing.
//
// Who needs it: callers that cannot call cudaMalloc.  Typical cases are a host
// application whose device memory is owned by its own memory manager (a fixed
// arena or budget that a plug-in must not grow, e.g. a renderer's frame loop
// that lends the solver only its particle buffers), and real-time loops that
// cannot afford the implicit device-wide synchronisation a cudaMalloc or
// cudaFree may cause.  Such callers cannot create a pbf_solver, because
// pbf_create allocates the solver's scratch.
//
// How: the scratch lives in one file-scope __device__ array of fixed size,
// kNoAllocScratchBytes (about 10.5 MB), which is part of this library's device
// image: every GPU that loads the library holds it until the process exits.
// It bounds the problem to kNoAllocMaxParticles particles and
// kNoAllocMaxCells grid cells; larger calls are rejected with
// PBF_ERR_CAPACITY.  The caller still passes every input and output buffer.
//
// Host code cannot use the array's name as a device address (on the host it
// names a stand-in object).  The device address is looked up with
// cudaGetSymbolAddress on the first call made while a device is current, and
// cached together with that device's CUDA context; a call that finds another
// context current on the device (after cudaDeviceReset, say, the module is
// loaded again and the array may sit elsewhere) looks it up again.  A first
// call therefore does set-up work and should be made before any stream
// capture.
//
// The array is shared by every call and keeps the last call's contents; the
// step clears what must start at zero (the per-cell counters and the group
// tables' hash entries, sums and counters) itself.  Calls
// whose work overlaps on the GPU (different streams, different host threads)
// race on the array: serialise them.
//
// The kernels and their sequence are exactly those of pbf_step; only where the
// scratch comes from differs.
#include <cuda.h>  // CUcontext / CUresult: the driver call below is resolved at run time

#include <mutex>

#include "pbf_internal.cuh"

namespace pbf {
pbf_status set_error(pbf_status s, const char* msg);
pbf_status set_cuda_error(cudaError_t e, const char* what);
pbf_status validate_step_setup(const pbf_params* params, const float ulim[3], const float llim[3],
                               long long max_cells, StepConsts* out);
pbf_status validate_step_buffers(const void* pos, const void* npos, const void* vel, const void* nvel,
                                 const void* iid);
}  // namespace pbf

namespace {

constexpr int kNoAllocMaxParticles = 32768;
constexpr int kNoAllocMaxCells = 131072;
constexpr size_t kAlign = 256;

constexpr size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// Byte offsets of every scratch buffer inside the static array.
constexpr size_t kNp = (size_t)kNoAllocMaxParticles;
constexpr size_t kNc = (size_t)kNoAllocMaxCells + 1;
constexpr size_t kSortTiles = (kNp + pbf::kSortTile - 1) / pbf::kSortTile;
constexpr size_t kOffKeysA = 0;
constexpr size_t kOffKeysB = kOffKeysA + align_up(4 * kNp);
constexpr size_t kOffValsA = kOffKeysB + align_up(4 * kNp);
constexpr size_t kOffValsB = kOffValsA + align_up(4 * kNp);
constexpr size_t kOffCount = kOffValsB + align_up(4 * kNp);
constexpr size_t kOffStart = kOffCount + align_up(4 * kNc);
constexpr size_t kOffRadix = kOffStart + align_up(4 * kNc);
constexpr size_t kOffPartials = kOffRadix + align_up(4 * 256 * kSortTiles);
constexpr size_t kOffXs = kOffPartials + align_up(4 * (size_t)pbf::kMaxScanPartials);
constexpr size_t kOffXa = kOffXs + align_up(16 * kNp);
constexpr size_t kOffXb = kOffXa + align_up(16 * kNp);
constexpr size_t kOffIid = kOffXb + align_up(16 * kNp);
constexpr size_t kOffLambda = kOffIid + align_up(4 * kNp);
constexpr size_t kOffRho = kOffLambda + align_up(4 * kNp);
constexpr size_t kOffFlags = kOffRho + align_up(4 * kNp);
constexpr size_t kOffDense = kOffFlags + align_up(4 * (size_t)pbf::kFlagWords);
constexpr size_t kOffMasks = kOffDense + align_up(4 * pbf::dense_list_len(kNoAllocMaxParticles));
constexpr size_t kOffCellFlags = kOffMasks + align_up(4 * (size_t)pbf::kMaskWords * kNp);
constexpr size_t kSlots = (size_t)kNoAllocMaxParticles / pbf::kGroupCell + 1;
constexpr size_t kEntries = kNp;
constexpr size_t kOffGrpCell = kOffCellFlags + align_up(4 * kNc);
constexpr size_t kOffGrpOff = kOffGrpCell + align_up(4 * kSlots);
constexpr size_t kOffGrpN = kOffGrpOff + align_up(4 * kSlots);
constexpr size_t kOffGrpRep = kOffGrpN + align_up(4 * kSlots);
constexpr size_t kOffGrpCnt = kOffGrpRep + align_up(4 * kEntries);
constexpr size_t kOffGrpPos = kOffGrpCnt + align_up(4 * kEntries);
constexpr size_t kOffGrpSum = kOffGrpPos + align_up(16 * kEntries);
constexpr size_t kOffGrpAux = kOffGrpSum + align_up(16 * kEntries);
constexpr size_t kOffGrpId = kOffGrpAux + align_up(16 * kEntries);
constexpr size_t kOffGrpHash = kOffGrpId + align_up(4 * kNp);
constexpr size_t kOffGrpMax = kOffGrpHash + align_up(4 * 8 * kNp);
constexpr size_t kOffGrpAcc = kOffGrpMax + align_up(4 * kNp);
constexpr size_t kItems = kNp / pbf::kGroupChunk + kSlots + 1;
constexpr size_t kOffGrpList = kOffGrpAcc + align_up(8 * 3 * kNp);
constexpr size_t kOffGrpListN = kOffGrpList + align_up(4 * kNp);
constexpr size_t kOffGrpDone = kOffGrpListN + align_up(4 * kSlots);
constexpr size_t kOffGrpZero = kOffGrpDone + align_up(4 * kSlots);
constexpr size_t kOffGrpItemOff = kOffGrpZero + align_up(4 * kSlots);
constexpr size_t kOffGrpItemSlot = kOffGrpItemOff + align_up(4 * kSlots);
constexpr size_t kOffWorkList = kOffGrpItemSlot + align_up(4 * kItems);
constexpr size_t kOffWorkFollow = kOffWorkList + align_up(4 * (kNp + 1));
constexpr size_t kOffWorkBlocks = kOffWorkFollow + align_up(4 * (kNp + 1));
constexpr size_t kOffBcnt = kOffWorkBlocks + align_up(4 * pbf::work_blocks_len(kNoAllocMaxParticles));
constexpr size_t kOffBstart = kOffBcnt + align_up(4 * kNc);
constexpr size_t kOffBent = kOffBstart + align_up(4 * kNc);
constexpr size_t kOffBucket = kOffBent + align_up(8 * kNp);
constexpr size_t kOffBpart = kOffBucket + align_up(4 * kNp);
constexpr size_t kNoAllocScratchBytes = kOffBpart + align_up(4 * (size_t)pbf::kMaxScanPartials);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_base[kMaxDevices] = {};
CUcontext g_ctx[kMaxDevices] = {};

// The driver's cuCtxGetCurrent, found through the runtime (no link against
// the driver library); null where it cannot be found.
using CtxGetCurrent = CUresult (*)(CUcontext*);
CtxGetCurrent ctx_get_current() {
  static const CtxGetCurrent fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      f = nullptr;
    }
    return (CtxGetCurrent)f;
  }();
  return fn;
}

CUcontext current_context() {
  CUcontext c = nullptr;
  const CtxGetCurrent fn = ctx_get_current();
  if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
  return c;
}

// Device address of g_noalloc_scratch on the current device: looked up on the
// first call with this device's context current, again when another context
// is current, and on every call when the context cannot be identified.
pbf_status scratch_base(unsigned char** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return pbf::set_cuda_error(e, "pbf_step_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return pbf::set_error(PBF_ERR_INVALID_ARG, "pbf_step_noalloc: device index out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  CUcontext ctx = current_context();
  if (!g_base[dev] || !ctx || ctx != g_ctx[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return pbf::set_cuda_error(e, "pbf_step_noalloc: cudaGetSymbolAddress");
    g_base[dev] = p;
    g_ctx[dev] = current_context();  // the lookup makes the device's context current if none was
  }
  *out = (unsigned char*)g_base[dev];
  return PBF_OK;
}

}  // namespace

extern "C" pbf_status pbf_step_noalloc(const pbf_params* params, const float ulim[3],
                                       const float llim[3], void* pos, void* npos, void* vel,
                                       void* nvel, uint32_t* iid, int n, void* stream) {
  const pbf::NvtxRange range("pbf_step_noalloc");
  if (n < 0) return pbf::set_error(PBF_ERR_INVALID_ARG, "pbf_step_noalloc: n < 0");
  if (n > kNoAllocMaxParticles)
    return pbf::set_error(PBF_ERR_CAPACITY,
                          "pbf_step_noalloc: n exceeds the fixed scratch limit of 32768 particles");
  pbf::StepConsts c;
  pbf_status st = pbf::validate_step_setup(params, ulim, llim, kNoAllocMaxCells, &c);
  if (st != PBF_OK) return st;
  if (n == 0) return PBF_OK;
  if ((st = pbf::validate_step_buffers(pos, npos, vel, nvel, iid)) != PBF_OK) return st;
  unsigned char* base = nullptr;
  if ((st = scratch_base(&base)) != PBF_OK) return st;

  pbf::GridScratch g;
  g.keys_a = (uint32_t*)(base + kOffKeysA);
  g.keys_b = (uint32_t*)(base + kOffKeysB);
  g.vals_a = (uint32_t*)(base + kOffValsA);
  g.vals_b = (uint32_t*)(base + kOffValsB);
  g.cell_count = (uint32_t*)(base + kOffCount);
  g.cell_start = (uint32_t*)(base + kOffStart);
  g.radix_counts = (uint32_t*)(base + kOffRadix);
  g.scan_partials = (uint32_t*)(base + kOffPartials);
  pbf::SolverScratch s = {};  // fields this step does not use stay null
  s.xs = (float4*)(base + kOffXs);
  s.xa = (float4*)(base + kOffXa);
  s.xb = (float4*)(base + kOffXb);
  s.iid_s = (uint32_t*)(base + kOffIid);
  s.lambda = (float*)(base + kOffLambda);
  s.rho = (float*)(base + kOffRho);
  s.flags = (uint32_t*)(base + kOffFlags);
  s.dense = (uint32_t*)(base + kOffDense);
  s.masks = (uint32_t*)(base + kOffMasks);
  s.mask_stride = kNoAllocMaxParticles;
  s.cell_flags = (uint32_t*)(base + kOffCellFlags);
  s.grp_pool = kNoAllocMaxParticles;
  s.grp_cell = (int*)(base + kOffGrpCell);
  s.grp_off = (int*)(base + kOffGrpOff);
  s.grp_n = (int*)(base + kOffGrpN);
  s.grp_rep = (int*)(base + kOffGrpRep);
  s.grp_cnt = (int*)(base + kOffGrpCnt);
  s.grp_pos = (float4*)(base + kOffGrpPos);
  s.grp_sum = (float4*)(base + kOffGrpSum);
  s.grp_aux = (float4*)(base + kOffGrpAux);
  s.grp_id = (int*)(base + kOffGrpId);
  s.grp_hash = (int*)(base + kOffGrpHash);
  s.grp_max = (unsigned*)(base + kOffGrpMax);
  s.grp_acc = (unsigned long long*)(base + kOffGrpAcc);
  s.grp_list = (int*)(base + kOffGrpList);
  s.grp_list_n = (int*)(base + kOffGrpListN);
  s.grp_done = (int*)(base + kOffGrpDone);
  s.grp_zero = (int*)(base + kOffGrpZero);
  s.grp_item_off = (int*)(base + kOffGrpItemOff);
  s.grp_item_slot = (int*)(base + kOffGrpItemSlot);
  s.work_list = (int*)(base + kOffWorkList);
  s.work_follow = (int*)(base + kOffWorkFollow);
  s.work_blocks = (int*)(base + kOffWorkBlocks);
  s.bcnt = (uint32_t*)(base + kOffBcnt);
  s.bstart = (uint32_t*)(base + kOffBstart);
  s.bent = (uint2*)(base + kOffBent);
  s.bucket = (int*)(base + kOffBucket);
  s.bpart = (uint32_t*)(base + kOffBpart);

  cudaStream_t strm = (cudaStream_t)stream;
  cudaError_t e;
  // the group tables' hash entries, bounds, fixed-point sums and per-slot
  // counters must be zero when a step starts (every pass leaves them so);
  // cleared here so that no call depends on what an earlier one left
  if ((e = cudaMemsetAsync(base + kOffGrpHash, 0, kOffGrpList - kOffGrpHash, strm)) != cudaSuccess ||
      (e = cudaMemsetAsync(base + kOffGrpListN, 0, kOffGrpZero - kOffGrpListN, strm)) != cudaSuccess)
    return pbf::set_cuda_error(e, "pbf_step_noalloc: clear");
  const uint32_t* perm = nullptr;
  // build_grid clears the per-cell counters itself (cudaMemsetAsync, no allocation)
  const pbf::Geometry G{nullptr, nullptr};
  if ((e = pbf::build_grid(c, G, (const float4*)pos, (const float4*)vel, nullptr, n, g, &perm, nullptr,
                           strm)) != cudaSuccess)
    return pbf::set_cuda_error(e, "pbf_step_noalloc: grid");
  s.keys_sorted = g.keys_sorted;
  s.cell_start = g.cell_start;
  if ((e = pbf::reorder(c, perm, (const float4*)pos, (const float4*)vel, iid, n, s, strm)) != cudaSuccess)
    return pbf::set_cuda_error(e, "pbf_step_noalloc: reorder");
  const int niter = params->niter;
  float4* X = s.xa;
  float4* T = s.xb;
  for (int it = 0; it < niter; ++it) {
    if ((e = pbf::launch_lambda(c, G, X, g.cell_start, n, s, 2 * it, strm)) != cudaSuccess)
      return pbf::set_cuda_error(e, "pbf_step_noalloc: lambda");
    if (it + 1 < niter) {
      if ((e = pbf::launch_delta_p(c, G, X, g.cell_start, n, s, 2 * it + 1, T, strm)) != cudaSuccess)
        return pbf::set_cuda_error(e, "pbf_step_noalloc: delta_p");
      float4* t = X;
      X = T;
      T = t;
    } else if ((e = pbf::launch_delta_p_final(c, G, X, g.cell_start, n, s, 2 * it + 1, (float4*)pos,
                                              (float4*)npos, (float4*)vel, iid, strm)) != cudaSuccess) {
      return pbf::set_cuda_error(e, "pbf_step_noalloc: delta_p");
    }
  }
  if ((e = pbf::launch_xsph(c, G, (const float4*)npos, (const float4*)vel, g.cell_start, n, s, 2 * niter,
                            (float4*)nvel, strm)) != cudaSuccess)
    return pbf::set_cuda_error(e, "pbf_step_noalloc: xsph");
  if (c.vort_eps > 0.f &&
      (e = pbf::launch_vorticity(c, G, (const float4*)npos, g.cell_start, n, s, (float4*)nvel, strm)) != cudaSuccess)
    return pbf::set_cuda_error(e, "pbf_step_noalloc: vorticity");
  return PBF_OK;
}
