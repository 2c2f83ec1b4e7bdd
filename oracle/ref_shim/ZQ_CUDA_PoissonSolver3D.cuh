// Stand-in declaration for ZQlibCuda's ZQ_CUDA_PoissonSolver3D.cuh (not in the
// reference tree).  TEST INFRASTRUCTURE ONLY.  ZQ_CUDA_AddForce3D.cu:523 calls
// cu_MAC_to_Regular_vel from its host wrapper; the device-only modules built by
// oracle/build_ref.py never compile that host code, so only the declaration
// (argument list as at the call site) is needed to parse the file.
#pragma once

namespace ZQ_CUDA_PoissonSolver3D {
void cu_MAC_to_Regular_vel(float* u, float* v, float* w, const float* mac_u, const float* mac_v,
                           const float* mac_w, int width, int height, int depth);
}
