/* Stand-in for the CUDA-samples helper_cuda.h the reference includes
 * (fluids/Simulator.h:5): only checkCudaErrors is used by the translation
 * unit compiled here, and only in host code, which a device-only build drops. */
#pragma once
#include <cuda_runtime.h>
#define checkCudaErrors(x) (x)
