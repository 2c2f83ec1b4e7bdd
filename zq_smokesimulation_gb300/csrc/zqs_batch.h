// Batched execution of many independent grids: one launch per stage walks a
// tile work list that spans every instance (internal header).
//
// A launch for shape class C covers instance i's tiles [pre[i], pre[i+1]) of
// a flat tile index space; blocks loop over that space with a grid stride
// (a persistent launch sized to the device), look up their instance with a
// binary search in the prefix array and run the same tile function the
// single-grid kernel runs, on that instance's buffers and parameters.
#pragma once

#include <vector>

#include "zqs_internal.h"

namespace zqs {

// Everything a batched kernel needs about one instance.
struct InstDesc {
    Layout L;
    float* vel[2][3];   // velocity ping-pong: [buffer][u,v,w]
    float* sca[2][2];   // scalar ping-pong: [buffer][T,rho]
    float* p[2];        // pressure ping-pong
    float* div;
    uint8_t* flags;
    float4* t4a;
    float4* t4b;
    float4* q4[3];      // quad copies of the current velocity (MAC sampler)
    double* red;
    long long red_len;
    KParams kp;
    SourceList src;
    int zc[2];          // SOR z chunk of this instance for the main and the remainder pass
    int closed;         // closed solver (divergence partials go to red, the mean to red[red_len-2])
    int pad;
};

// Shape classes of tile index spaces (per instance):
//   CELL  ceil(W/32) x ceil(H/8) x D          32x8 blocks over cells
//   FACE  ceil((W+1)/32) x ceil((H+1)/8) x (D+1)  over faces
//   ADVF  as FACE with 3(D+1) z-blocks        one per face component
//   SORM  ceil(W/TX) x ceil(H/TY) x ceil(D/zc[0])  fused SOR tiles, main pass
//   SORR  as SORM for the remainder pass (tile and zc[1] of its variant)
enum TileClass { TC_CELL = 0, TC_FACE = 1, TC_ADVF = 2, TC_SORM = 3, TC_SORR = 4, TC_COUNT = 5 };

__device__ __forceinline__ int batch_find(const int* __restrict__ pre, int n, int t) {
    int lo = 0, hi = n - 1;  // largest i with pre[i] <= t
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(pre + mid) <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The fields the batched advection kernels read inside their backtrace loops,
// for a chunk of consecutive instances, passed by value in the kernels'
// parameter space: loop invariants (extents, pitches, step sizes, buffer
// pointers) are then constant-bank operands, as in the single-grid kernels,
// rather than registers loaded from the descriptor in global memory, which
// cost the batched kernels occupancy.
struct AdvHot {
    Layout L;
    KParams kp;
    const float4* q[3];   // quad copies of the current velocity
    const uint8_t* flags;
    float* vel[2][3];     // velocity ping-pong
    float* sca[2][2];     // scalar ping-pong
};
constexpr int kAdvHotMax = 96;  // instances per table (the parameter space holds 32 KB)
struct AdvHotTable {
    int base;  // first instance (table row) of the chunk
    int n;     // instances in the chunk
    AdvHot h[kAdvHotMax];
};

struct BatchLaunch {
    const InstDesc* desc;  // device array of n descriptors
    const int* pre;        // device prefix array (n+1) of the launch's tile class
    int n;
    int total;             // pre[n]
    const int* pre_host = nullptr;  // host copy of pre (launch ranges of table chunks)
};

// SOR plan of a batch: the main fused variant (depth S/2) and the variant that
// runs the K mod depth remaining iterations; both are register-column kernels.
struct SorBatchPlan {
    int vmain = -1, vrem = -1;
    int S[2] = {0, 0}, TX[2] = {0, 0}, TY[2] = {0, 0};
    int slots[2] = {0, 0};  // resident CTAs on the device (SMs x CTAs per SM)
};
// Blocks of a persistent batched launch: as many as are resident on the
// device at once for this kernel (its occupancy x SM count), at most cap.  A
// larger grid would leave blocks waiting for whole tile lists of others.
int persistent_blocks(const void* kernel, int threads, size_t dyn_smem, int cap);

int sor_batch_plan(int variant, SorBatchPlan& out);  // variant -1: the batch default
bool sor_variant_batchable(int variant);
// One fused SOR pass of kind `which` (0: main variant, 1: remainder) over the
// tile list B, pressure p[pcur] -> p[pcur ^ 1] of every instance (the tuner's probe).
cudaError_t launch_sor_batch_pass(const SorBatchPlan& plan, int which, const BatchLaunch& B, int pcur,
                                  cudaStream_t s);

int launch_force_batch(const BatchLaunch& cell, const BatchLaunch& face, int vcur, int scur, int blocks,
                       cudaStream_t s, LaunchCounter& lc);
int launch_mac_quads_batch(const BatchLaunch& face, int vcur, int blocks, cudaStream_t s, LaunchCounter& lc);
// One launch per table chunk, over the chunk's tiles [pre[base], pre[base + n]).
int launch_advect_velocity_batch(const BatchLaunch& advf, const std::vector<AdvHotTable>& hot, int vcur,
                                 cudaStream_t s, LaunchCounter& lc);
int launch_advect_scalar_batch(const BatchLaunch& cell, const std::vector<AdvHotTable>& hot, int vcur, int scur,
                               cudaStream_t s, LaunchCounter& lc);
// Divergence (+ closed-solver mean removal), K SOR iterations, gradient on the
// velocity buffer vcur; *pfin receives the pressure buffer holding the result.
int launch_project_batch(const BatchLaunch& cell, const BatchLaunch& face, const BatchLaunch& sorm,
                         const BatchLaunch& sorr, const SorBatchPlan& plan, int K, bool any_closed, int vcur,
                         int blocks, cudaStream_t s, LaunchCounter& lc, int* pfin);

}  // namespace zqs
