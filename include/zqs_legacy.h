/*
 * zqs_legacy.h -- the reference's own entry points for the smoke step, with
 * the reference's names, signatures, enum values and host-pointer semantics,
 * implemented by libzqs_gb300.so so existing callers relink without edits.
 *
 * Behaviour shared by every host-pointer shim below (as in the reference):
 * synchronous; arrays are the caller's unpadded host arrays, updated in place;
 * the return value is the elapsed milliseconds of the whole call measured with
 * CUDA events, transfers included.  Differences, all deliberate:
 *   - no per-call cudaMalloc: device buffers are cached per grid size;
 *   - CUDA errors do not exit the process: the shim returns a negative value
 *     (-zqs_status) and zqs_last_error() has the message;
 *   - Advect_Scalar with a BFECC type runs the three BFECC passes of the
 *     reference's cu_Advect_Scalar_*_BFECC (Adv3D:1507-1554, 1586-1648); the
 *     reference's entry point never calls them and returns zeros for those
 *     types (Adv3D:1786-1794).  Advect_Velocity runs all six types as the
 *     reference does; an unknown type returns -ZQS_EINVAL, arrays untouched.
 * Not re-entrant: ZQ_Cuda_Prepare_Advection sets process-wide state exactly
 * like the reference (ZQ_CUDA_Advection3D.cu:1652-1668).
 */
#ifndef ZQS_LEGACY_H
#define ZQS_LEGACY_H

#include <stdint.h>
#include <vector_types.h> /* float4 */

#include "zqs_capi.h"

#ifdef __cplusplus

namespace ZQ_CUDA_Advection3D {
/* ZQ_SmokeSimulation3D/ZQ_CUDA_Advection3D.h:7-21 */
enum AdvectVelocityType {
    ADV_VEL_INREG_OUTREG = 0,
    ADV_VEL_INREG_OUTREG_BFECC,
    ADV_VEL_INMAC_OUTMAC,
    ADV_VEL_INMAC_OUTMAC_BFECC,
    ADV_VEL_INREG_OUTMAC,
    ADV_VEL_INREG_OUTMAC_BFECC
};
enum AdvectScalarType { ADV_SCA_MAC, ADV_SCA_MAC_BFECC, ADV_SCA_REG, ADV_SCA_REG_BFECC };

/* replaces ZQ_CUDA_Advection3D.h:23 (impl. ZQ_CUDA_Advection3D.cu:1652-1684) */
extern "C" ZQS_API void ZQ_Cuda_Prepare_Advection(const unsigned int width, const unsigned int height,
                                                  const unsigned int depth, const float voxelSize,
                                                  const unsigned int steps, const float deltatt);
/* replaces ZQ_CUDA_Advection3D.h:31 (impl. ZQ_CUDA_Advection3D.cu:1686-1749) */
extern "C" ZQS_API float Advect_Velocity(float* u, float* v, float* w, const bool* occupy, bool is_open,
                                         enum AdvectVelocityType type);
/* replaces ZQ_CUDA_Advection3D.h:43-44 (impl. ZQ_CUDA_Advection3D.cu:1751-1821); in == out allowed */
extern "C" ZQS_API float Advect_Scalar(const float* u, const float* v, const float* w, const bool* occupy,
                                       const float* input_temperature, const float* input_density,
                                       float* output_temperature, float* output_density,
                                       enum AdvectScalarType type);
}  // namespace ZQ_CUDA_Advection3D

namespace ZQ_CUDA_AddForce3D {
/* ZQ_SmokeSimulation3D/ZQ_CUDA_AddForce3D.h:6-10 */
enum AddForceType { ADD_FORCE_ENTIRE, ADD_FORCE_SLICE };
/* replaces ZQ_CUDA_AddForce3D.h:12-14 (impl. ZQ_CUDA_AddForce3D.cu:606-659); both types run the
 * same fused kernels (the reference's SLICE also dispatches the ENTIRE path, :636-640) */
extern "C" ZQS_API float AddForce3D(float* mac_u, float* mac_v, float* mac_w, const bool* occupy,
                                    const float* temperature, const float deltah, const float deltat,
                                    const float buoyCoeff, const float confineCoeff, const float Tamb,
                                    const int width, const int height, const int depth, enum AddForceType type);
}  // namespace ZQ_CUDA_AddForce3D

namespace ZQ_CUDA_Attenuation3D {
/* replaces ZQ_CUDA_Attenuation3D.h:6-8 (impl. ZQ_CUDA_Attenuation3D.cu:138-194); factors, not coefficients */
extern "C" ZQS_API float Attenuation3D(float* mac_u, float* mac_v, float* mac_w, float* temperature,
                                       float* density, const bool* occupy, const float velAtten,
                                       const float tempAtten, const float densityAtten, const int width,
                                       const int height, const int depth);
}  // namespace ZQ_CUDA_Attenuation3D

namespace ZQ_CUDA_MACtoRegular {
/* replace ZQ_CUDA_MACtoRegular.cuh:21-23: DEVICE pointers, unpadded layouts, default stream */
ZQS_API void cu_MAC_to_Regular4(const float* mac_u, const float* mac_v, const float* mac_w, float4* vel4,
                                int width, int height, int depth);
ZQS_API void cu_Regular4_to_MAC(const float4* vel4, float* mac_u, float* mac_v, float* mac_w, int width,
                                int height, int depth);
}  // namespace ZQ_CUDA_MACtoRegular

namespace ZQ_CUDA_PoissonSolver3D {
/* The reference calls these from ZQlibCuda, which is not part of its tree
 * (call sites ZQ_SmokeSimulationUtils3D.cpp:2354-2363, 2424-2437; signature
 * inferred from them).  Host pointers, in place, omega = 1 (plain red-black
 * Gauss-Seidel as in every solver of the reference). */
ZQS_API void SolveOpenPoissonRedBlackwithOccupy3D_MAC(float* mac_u, float* mac_v, float* mac_w,
                                                      const bool* occupy, int width, int height, int depth,
                                                      int maxIter);
ZQS_API void SolveClosedPoissonRedBlackwithOccupy3D_MAC(float* mac_u, float* mac_v, float* mac_w,
                                                        const bool* occupy, float div_per_volume, int width,
                                                        int height, int depth, int maxIter);
/* called by cu_AddForce3D (ZQ_CUDA_AddForce3D.cu:523): DEVICE pointers, cell-centre velocity */
ZQS_API void cu_MAC_to_Regular_vel(float* u, float* v, float* w, const float* mac_u, const float* mac_v,
                                   const float* mac_w, int width, int height, int depth);
}  // namespace ZQ_CUDA_PoissonSolver3D

extern "C" {
#endif /* __cplusplus */

/* C-linkage form of the two solvers above with over-relaxation: solver is
 * zqs_solver; for ZQS_SOLVER_CLOSED the mean divergence over free cells is
 * computed in FP64 and removed.  Host pointers, in place.  Returns zqs_status. */
ZQS_API int zqs_project_sor(float* mac_u, float* mac_v, float* mac_w, const uint8_t* occupy, int width, int height,
                            int depth, int solver, int maxIter, float omega);

/* No counterpart in the reference.  The same projection for callers that
 * must not allocate GPU memory (a pre-reserved memory pool, code that runs
 * while a CUDA graph is being captured, runtimes without an allocator):
 * DEVICE pointers in the reference layouts, updated in place, asynchronous on
 * `stream` (NULL: the default stream).  It calls no cudaMalloc/cudaFree: its
 * working fields live in one fixed array compiled into the library (about
 * 7.6 MB, held by every GPU that loads the library until the process exits),
 * which limits the grid to ZQS_NOALLOC_MAX_ELEMS padded elements per field,
 * (W+1 rounded up to 4)*(H+1)*(D+3); 64x64x64 fits.  Larger grids return
 * ZQS_EINVAL.  The first call on each device does the one-time setup for that
 * device: the array's device address, the shared-memory attributes and
 * occupancy of the SOR kernels, and the loading of the kernels it runs (the
 * closed solver runs two more than the open one); make a first call with each
 * solver type you use before any stream capture.  Every device that calls it
 * has its own copy of the array; the devices of one process must be the same
 * GPU model (another model returns ZQS_EUNSUPPORTED).  All calls on a device
 * share its array, so calls that overlap on the GPU (different streams, or
 * concurrent host threads) race; serialise them.  Returns zqs_status. */
#define ZQS_NOALLOC_MAX_ELEMS 300000
ZQS_API int zqs_project_sor_noalloc(float* d_u, float* d_v, float* d_w, const uint8_t* d_occupy, int width,
                                    int height, int depth, int solver, int maxIter, float omega, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ZQS_LEGACY_H */
