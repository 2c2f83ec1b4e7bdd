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
    int tc = 1;                 // obstacle-free blocks: 1 tensor cores (3xTF32), 0 exact FP32 SIMT
    float* Xsplit = nullptr;    // tensor-core operands: xh then xl, blocks x kpad each (tc only)
    int* err = nullptr;         // device flag: a tensor-core wait timed out
};

// Block face q (u: k, j, i <= s; v: k, j <= s, i; w: k <= s, j, i) of block
// (bi, bj, bk) -> the fine face's padded index and component.
__host__ __device__ __forceinline__ int subproj_block_face(const Layout& L, int s, int q, int bi, int bj, int bk, int& comp) {
    const int nu = s * s * (s + 1);
    int i, j, k;
    if (q < nu) {
        comp = 0;
        i = q % (s + 1);
        j = (q / (s + 1)) % s;
        k = q / (s * (s + 1));
    } else if (q < 2 * nu) {
        comp = 1;
        const int x = q - nu;
        i = x % s;
        j = (x / s) % (s + 1);
        k = x / (s * (s + 1));
    } else {
        comp = 2;
        const int x = q - 2 * nu;
        i = x % s;
        j = (x / s) % s;
        k = x / (s * s);
    }
    return lidx(L, bi * s + i, bj * s + j, bk * s + k);
}

// Interior row r (u: k, j, i = 1..s-1; v: k, j = 1..s-1, i; w: k = 1..s-1, j, i)
// -> block face index.
__device__ __forceinline__ int subproj_interior_face(int s, int r) {
    const int nu = s * s * (s + 1);
    const int ni = s * s * (s - 1);
    if (r < ni) {
        const int i = 1 + r % (s - 1), j = (r / (s - 1)) % s, k = r / ((s - 1) * s);
        return (k * s + j) * (s + 1) + i;
    }
    if (r < 2 * ni) {
        const int x = r - ni;
        const int i = x % s, j = 1 + (x / s) % (s - 1), k = x / (s * (s - 1));
        return nu + (k * (s + 1) + j) * s + i;
    }
    const int x = r - 2 * ni;
    const int i = x % s, j = (x / s) % s, k = 1 + x / (s * s);
    return 2 * nu + (k * s + j) * s + i;
}

// Allocate (or reuse) the coarse state of a grid with layout L for block edge
// s; s must divide W, H and D.  Not for use inside a stream capture.
int coarse_prepare(CoarseState*& cs, const Layout& L, int s, int tc);
void coarse_free(CoarseState*& cs);

// The split matrix of block edge s on the device (cached per s) and the
// kernel's shared-memory limit: before the first launch, outside any capture.
int subproj_tc_prepare(int s);
// Bytes of the tensor-core operand split (xh, xl) for nblocks blocks of nf faces.
size_t subproj_tc_split_bytes(int nblocks, int nf);
// Obstacle-free blocks on the tensor cores: the block faces gathered from
// u, v, w and split into Xsplit, then Y = X M^T written to the blocks' interior
// faces (blocks with bobs set skipped).
int launch_subproj_tc(const Layout& L, const Layout& Lc, int s, int nf, int rows, int nblocks, float* Xsplit,
                      const uint8_t* bobs, float* u, float* v, float* w, int* err, cudaStream_t st,
                      LaunchCounter& lc);
// A tensor-core wait of an earlier projection timed out (reads and clears the
// device flag; synchronises the stream).
int coarse_check(CoarseState* cs, cudaStream_t st);

// One coarse projection of g's velocity (in place); K coarse SOR iterations.
int launch_project_coarse(DevGrid& g, const KParams& kp, int K, cudaStream_t s, LaunchCounter& lc);

// The sub-projection matrix of ZQ_InitSubMatPoisson3D (Utils3D:1151-1391) for
// block edge s: rows = 3 s^2 (s-1) interior faces, cols = 3 s^2 (s+1) block
// faces, row-major floats (built in double on the host).
std::vector<float> coarse_submatrix(int s);

}  // namespace zqs
