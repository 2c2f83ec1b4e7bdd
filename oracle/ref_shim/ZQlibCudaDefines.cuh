// Stand-in for ZQlibCuda's ZQlibCudaDefines.cuh (ZQlibCuda is not part of the
// reference tree).  TEST INFRASTRUCTURE ONLY: used by oracle/build_ref.py to
// compile the reference's own kernel files (ZQ_CUDA_MACtoRegular.cu,
// ZQ_CUDA_Attenuation3D.cu, ZQ_CUDA_AddForce3D.cu, ZQ_CUDA_Advection3D.cu)
// into device-only modules.  The reference uses BLOCK_SIZE for its 2D thread
// blocks (e.g. ZQ_CUDA_MACtoRegular.cu:104) and checkCudaErrors around host
// CUDA calls; the host code is never compiled for the modules, so the macro
// only has to parse.
#pragma once
#include <cuda_runtime.h>

#define BLOCK_SIZE 16
#define checkCudaErrors(x) (x)
