// Coarse-grid projection (ZQS_SOLVER_COARSE_OPEN), internal header.
//
// ZQ_TotalProjection3D for the coarse SOR solvers (Utils3D:3688-3794): face
// un-occupancy ratios of the grid coarsened by s, the fine faces averaged onto
// the coarse faces, red-black SOR on the face-ratio Poisson system, the
// correction added back to the free fine faces, then (s > 1) an exact
// projection inside every s^3 block: a dense matrix for blocks without an
// occupied cell, a least-squares solve (CG in double) for the others.
#pragma once

#include <vector>

#include "zqs_internal.h"

namespace zqs {

struct CoarseState {
    int s = 0;                  // block edge (sub_size)
    Layout Lc{};                // coarse padded layout (cW = W / s, ...)
    void* base = nullptr;       // one allocation for the fields below
    float *ru, *rv, *rw;        // face un-occupancy ratios
    float *cu, *cv, *cw;        // coarse velocity
    float *du, *dv, *dw;        // coarse correction
    float *div, *diag, *p;      // coarse system
    uint8_t* occ;               // coarse occupancy (1 = occupied)
    uint8_t* bobs;              // per block (coarse cell, dense): 1 = has an occupied fine cell
    float* X;                   // gathered block faces, nblocks x nf
    int nf = 0, rows = 0, nblocks = 0;
    const float* MT = nullptr;  // sub-projection matrix transposed, nf x rows (shared per s)
};

// Allocate (or reuse) the coarse state of a grid with layout L for block edge
// s; s must divide W, H and D.  Not for use inside a stream capture.
int coarse_prepare(CoarseState*& cs, const Layout& L, int s);
void coarse_free(CoarseState*& cs);

// One coarse projection of g's velocity (in place); K coarse SOR iterations.
int launch_project_coarse(DevGrid& g, const KParams& kp, int K, cudaStream_t s, LaunchCounter& lc);

// The sub-projection matrix of ZQ_InitSubMatPoisson3D (Utils3D:1151-1391) for
// block edge s: rows = 3 s^2 (s-1) interior faces, cols = 3 s^2 (s+1) block
// faces, row-major floats (built in double on the host).
std::vector<float> coarse_submatrix(int s);

}  // namespace zqs
