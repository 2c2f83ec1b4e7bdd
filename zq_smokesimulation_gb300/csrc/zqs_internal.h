// Internal declarations of the GB300 smoke-step library (not installed).
//
// Device layout.  Every field of a grid (u, v, w, T, rho, p, div, flags) uses
// one shared padded index space so a single index addresses all of them:
//     idx(i,j,k) = (k*rows + j)*pitch + i,  pitch = roundup(W+1, 4), rows = H+1,
// with D+1 data planes plus one zero guard plane on each side (the field
// pointer points at plane 0, so k = -1 and i-1 at i = 0 stay in bounds).
// u uses i in [0,W], v uses j in [0,H], w uses k in [0,D]; cells use
// [0,W)x[0,H)x[0,D).  Rows are 16-byte aligned (float4 loads along x).
// Entries outside a field's extent stay zero, which the SOR relies on.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/zqs_capi.h"

namespace zqs {

// flags byte per cell index
enum : uint8_t {
    F_FREE = 1u << 0,     // in-domain cell, not occupied
    F_CNT_SHIFT = 1,      // bits 1-3: SOR stencil weight (0..6) of a free cell
    F_CNT_MASK = 7u << 1,
    F_UFACE = 1u << 4,    // u face (i,j,k) live under the open rule
    F_VFACE = 1u << 5,
    F_WFACE = 1u << 6,
};

struct Layout {
    int W, H, D;
    int px;            // pitch in elements
    int py;            // rows per plane
    int pz;            // data planes
    long long plane;   // px*py
    long long elems;   // per-field allocation incl. the two guard planes
};

__host__ __device__ inline int lidx(const Layout& L, int i, int j, int k) {
    return (k * L.py + j) * L.px + i;
}

// Kernel-side copy of the run parameters (everything a kernel reads).
struct KParams {
    float h;            // voxel size
    float dt;           // step time
    float dt_sub;       // step_time / substeps, float division as the reference
    float inv_h;        // 1/h when h is a power of two (exact), else 0
    int substeps;
    int full;           // backtrace_full
    float cc;           // confine * h
    float twoh;         // 2*h
    float beta, alpha, tamb;
    float vel_atten, temp_atten, dens_atten;
    float omega, om1;   // omega and 1-omega
    int solver;
    int mean_override;  // closed solver: subtract mean_value instead of the FP64 mean
    float mean_value;
    // External per-cell force added to the cell force after the buoyancy terms
    // (the control of the adjoint problem): component q of cell c at
    // fext[q*elems + c] in the padded layout; null when absent.
    const float* fext;
};

struct SourceList {
    int n;
    zqs_source s[ZQS_MAX_SOURCES];
};

// Pointers of one grid's device state.
struct CoarseState;  // zqs_coarse.h

struct DevGrid {
    Layout L;
    float *u, *v, *w;          // current velocity
    float *u2, *v2, *w2;       // next velocity (advection target)
    float *T, *rho;            // current scalars
    float *T2, *rho2;          // next scalars
    float *p, *p2;             // pressure ping-pong
    float *div;                // projection right-hand side
    uint8_t* flags;
    float4 *t4a, *t4b;         // float4 temporaries (vorticity/force or centre velocity)
    float4 *qu, *qv, *qw;      // quad copies of the velocity for the MAC sampler (tri0_quad)
    double* red;               // FP64 reduction scratch (the closed-solver mean sits in the last 2)
    long long red_len;
    CoarseState* coarse = nullptr;  // ZQS_SOLVER_COARSE_OPEN state (owned by the grid handle)
};

// ---- device allocation -----------------------------------------------------
// Every device allocation of the library goes through dev_alloc, so the test
// hook zqs_debug_fail_alloc can make a chosen one fail as out-of-memory.
cudaError_t dev_alloc_raw(void** p, size_t bytes);
template <class T>
inline cudaError_t dev_alloc(T** p, size_t bytes) {
    return dev_alloc_raw(reinterpret_cast<void**>(p), bytes);
}

// ---- error reporting -------------------------------------------------------
void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
#define ZQS_CUDA_TRY(expr)                                   \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) return ::zqs::cuda_fail(_e, #expr); \
    } while (0)
#define ZQS_LAUNCH_CHECK(what)                               \
    do {                                                     \
        cudaError_t _e = cudaGetLastError();                 \
        if (_e != cudaSuccess) return ::zqs::cuda_fail(_e, what); \
    } while (0)

// ---- launchers (each returns a zqs_status and counts its launches) ----------
struct LaunchCounter {
    long long n = 0;
};

int launch_build_flags(const DevGrid& g, const uint8_t* occ_dense, int solver, cudaStream_t s, LaunchCounter& lc);
int launch_mac_to_reg4(const DevGrid& g, const float* u, const float* v, const float* w, float4* out,
                       cudaStream_t s, LaunchCounter& lc);
int launch_reg4_dense(const DevGrid& g, const float4* src, float4* dense, cudaStream_t s, LaunchCounter& lc);

int launch_dense_mac_to_centre(int W, int H, int D, const float* u, const float* v, const float* w, float4* vel4,
                               float* uc, float* vc, float* wc, cudaStream_t s);
int launch_dense_reg4_to_mac(int W, int H, int D, const float4* vel4, float* u, float* v, float* w, cudaStream_t s);

int make_kparams(const zqs_params& p, KParams& kp);
int validate_params(const zqs_params& p);

int launch_force(const DevGrid& g, const KParams& kp, bool fuse_vel_atten, cudaStream_t s, LaunchCounter& lc);
int launch_attenuate(const DevGrid& g, const KParams& kp, cudaStream_t s, LaunchCounter& lc);

int launch_advect_velocity(DevGrid& g, const KParams& kp, int mode, bool open, cudaStream_t s,
                           LaunchCounter& lc);  // writes u2,v2,w2 (caller swaps)
int launch_advect_scalar(const DevGrid& g, const KParams& kp, int mode, bool fold_atten,
                         const SourceList* src, cudaStream_t s, LaunchCounter& lc);  // writes T2,rho2
int launch_reinject(const DevGrid& g, const SourceList& src, cudaStream_t s, LaunchCounter& lc);

struct SorConfig {
    int temporal_depth = 0;  // iterations per fused pass; 0: the tuned variant (launch_project
                             // itself falls back to the depth-2 default when nothing was tuned)
    int split = 0;           // 1: one launch per colour (plain kernel)
    int variant = -1;        // fused kernel variant (-1: default for the depth)
    int zchunk = 0;          // z planes per CTA (0: chosen from the grid)
};
int sor_variant_count();
int sor_variant_info(int i, zqs_sor_variant* out);
int sor_default_variant(int depth);  // the fixed variant launch_project uses for a depth (0: 2)

// Per grid shape and device: the fused SOR variant and z chunk with the
// shortest measured time per iteration.  Times every variant that fits, at a
// few z chunks each, on the grid's own pressure, divergence and flags
// buffers (the pressure is overwritten: call it where the next projection
// starts from p = 0 anyway); synchronises the stream, so never inside a
// stream capture.  Results are kept in memory and in an on-disk file.
struct SorChoice {
    int variant = -1;
    int zchunk = 0;
    float us_per_iter = 0.0f;
    int source = 0;  // 0 none, 1 measured now, 2 this process's cache, 3 the on-disk cache
};
int sor_autotune(const DevGrid& g, const KParams& kp, cudaStream_t s, SorChoice& out);
int launch_project(DevGrid& g, const KParams& kp, int K, const SorConfig& cfg, cudaStream_t s,
                   LaunchCounter& lc, float** p_final);
int sor_prepare();  // sets the SOR kernels' attributes once per device (outside any capture)
// ZQS_ETIMEOUT (and clears the count) when a bounded wait of the split-barrier
// SOR variants gave up on the current device since the last check.
int sor_sync_check();
int launch_stats(const DevGrid& g, const KParams& kp, const float* p, zqs_stats* out, cudaStream_t s);

}  // namespace zqs
