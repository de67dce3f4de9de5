// ref_kernels.cu — device-only build of the reference's kernels (test
// infrastructure, part of the oracle).
//
// Compiled with nvcc -cubin against the reference's own, unmodified sources
// (fluids/Simulator.cu and the fluids/Simulator_kernel.cuh it includes), found
// through -I; only device code is emitted.  Besides the reference's kernels the
// cubin holds two wrapper kernels that apply the reference's own functors
// where the reference applies them through thrust::transform:
//   getGridId        (fluids/Simulator.cu:56-73, used at :190-193)
//   h_updateVelocity (fluids/Simulator.cu:127-137, used at :267-273)
#include "Simulator.cu"

extern "C" __global__ void pbfref_grid_id(const float3* npos, unsigned* ids, int n, getGridId f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ids[i] = (unsigned)f(npos[i]);
}

extern "C" __global__ void pbfref_update_velocity(const float3* pos, const float3* npos, float3* vel,
                                                  int n, h_updateVelocity f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) vel[i] = f(thrust::make_tuple(pos[i], npos[i]));
}

// The instantiations Simulator::correctDensity / correctVelocity launch
// (fluids/Simulator.cu:222-230, :237-245, :257-264).
template __global__ void computeLambda<getGridxyz, xyzToId, DensityBoundary, getPoly6, getSpikyGrad>(
    uint*, float*, float*, uint*, uint*, uint*, int3, float3*, int, float, float, float, float, getGridxyz,
    xyzToId, DensityBoundary, getPoly6, getSpikyGrad);
template __global__ void computetpos<getGridxyz, xyzToId, getPoly6, getSpikyGrad>(
    float*, uint*, uint*, uint*, uint*, int3, float3*, float3*, int, float, float, float, float, getGridxyz,
    xyzToId, float3, float3, getPoly6, getSpikyGrad);
template __global__ void computeXSPH<getGridxyz, xyzToId, getPoly6>(float*, uint*, uint*, uint*, int3, float3*,
                                                                     float3*, float3*, int, float, float,
                                                                     getGridxyz, xyzToId, getPoly6);
