// Reverse mode of the smoke step on the padded device layout (internal header).
//
// The adjoint of one step runs, in order (every buffer in the grid's padded
// index space; "g" = adjoint):
//   quads    k_mac_quads x2    quad copies of the end-of-step velocity and of
//                              the advection input (the forward's sampler)
//   scalar   k_adj_scalar      per cell: sources zeroed, backtrace through the
//                              end-of-step velocity recorded, the final sample
//                              scattered to gTa/grhoa (attenuation folded) and
//                              the position chain scattered into the quad
//                              accumulators gq (16-byte atomics)
//            k_adj_fold        per face: gu += gq folded onto its texels
//   project  k_adj_gradT       per cell: q = (omega/cnt) * G^T gu
//            k_adj_sor_sweep   2K-1 red/black in-place sweeps of the reversed
//                              SOR (acc collects -gdiv), plus a tail
//            k_adj_divT        per face: gu3 = gu + div^T(gdiv); gu2 seeded
//                              with gu3 on faces the advection leaves alone
//   advect   k_adj_advect_vel  per live face: backtrace through u2 recorded,
//                              final sample and position chain scattered
//                              into gq (16-byte atomics)
//            k_adj_fold        per face: gu2 += gq folded onto its texels
//   force    k_adj_force_cell  per cell: face averaging transposed (with the
//                              velocity attenuation), gF, gT, grho, and the
//                              confinement cross product / normalisation
//            k_adj_vs          per cell: the |w|-gradient stencil transposed,
//                              d|w|/dw, the 1/(2h) of the curl
//            k_adj_centre      per cell: the curl stencil transposed
//            k_adj_faces       per face: gu = gu1 + centre average transposed
#pragma once

#include "zqs_internal.h"

namespace zqs {

constexpr int kAdjMaxSubsteps = 32;  // backtrace positions kept per thread

struct AdjBufs {
    float *gu, *gv, *gw;        // adjoint of the end-of-step velocity in, of the start velocity out
    float *gu3, *gv3, *gw3;     // adjoint of the velocity advection output
    float *gu2, *gv2, *gw2;     // adjoint of the velocity advection input
    float *gT, *grho;           // adjoint of the scalars (end in, start out)
    float *gTa, *grhoa;         // scatter accumulators of the scalar advection
    float *q, *acc, *wt;        // reversed SOR: scaled adjoint pressure, -gdiv, omega/cnt
    float* q2;                  // second q buffer of the fused passes
    float *gF;                  // adjoint of the control, 3 components at stride elems
    float4 *gom4, *gg4, *gw4;   // confinement temporaries
    // Quad accumulators of the transposed trilinear samples, one per face
    // component, in the layout of the forward's quad copies: gq[c][r] =
    // contributions to texels (r, r + plane, r + 1, r + plane + 1), so one
    // sample scatters with two 16-byte atomics (at r and r + px).  Each
    // pointer has one float4 of margin before its leading guard plane (the
    // fold reads r - plane - 1).
    float4* gq[3];
    double* red;                // FP64 partials (closed-solver mean)
    long long red_len;
};

// Forward state a step's adjoint reads (all padded, read-only).
struct AdjFwd {
    const float *u4, *v4, *w4;  // velocity at the end of the step (after projection)
    const float *u2, *v2, *w2;  // velocity after force + attenuation (advection input)
    const float *T0, *rho0;     // scalars at the start of the step
    const float4* vort;         // (wx, wy, wz, |w|) of the start velocity
    const float4* q4[3];        // quad copies of u4, v4, w4 (zqs_sample.cuh, tri0_quad)
    const float4* q2[3];        // quad copies of u2, v2, w2
    const uint8_t* flags;
};

int launch_adj_weights(const Layout& L, const uint8_t* flags, float omega, float* wt, cudaStream_t s,
                       LaunchCounter& lc);
// npairs black/red pairs of the reversed SOR in temporally blocked passes
// (register-column kernel, ADJ form); q and q2 ping-pong, *qcur = result.
int launch_sor_adjoint_pairs(const Layout& L, float* q, float* q2, const float* wt, float* acc, float om1,
                             int npairs, cudaStream_t s, LaunchCounter& lc, float** qcur);
// Once per (device, shape): time the ADJ forms of the depth-2 variants on
// these buffers (q, q2 and acc are overwritten) and keep the fastest for
// launch_sor_adjoint_pairs; synchronises s, never inside a capture.
// ZQS_AUTOTUNE=0 keeps the fixed order.
int sor_adj_autotune(const Layout& L, float* q, float* q2, const float* wt, float* acc, float om1, cudaStream_t s);
// Quad copies of the three face components of g (g.u/v/w into g.qu/qv/qw).
int launch_mac_quads(const DevGrid& g, cudaStream_t s, LaunchCounter& lc);
int launch_adj_step(const Layout& L, const AdjFwd& f, const AdjBufs& b, const KParams& kp, const SourceList& src,
                    int K, cudaStream_t s, LaunchCounter& lc);

// Dense (x fastest, no padding) <-> padded copies of an nx x ny x nz block.
int copy_dense_padded(float* padded, const float* dense, const Layout& L, int nx, int ny, int nz, bool src_on_device,
                      cudaStream_t s);
int copy_padded_dense(float* dense, const float* padded, const Layout& L, int nx, int ny, int nz, bool dst_on_device,
                      cudaStream_t s);

}  // namespace zqs
