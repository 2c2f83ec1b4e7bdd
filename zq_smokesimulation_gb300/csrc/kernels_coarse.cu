// Coarse-grid projection on the device (ZQS_SOLVER_COARSE_OPEN): the restated
// ZQ_TotalProjection3D for COARSE_{OPEN,CLOSED}_POISSON_SOR (Utils3D:3688-3794).
//
//   k_coarse_ratios    face un-occupancy ratios (ZQ_InitCoarseGrid3D, Utils3D:1666-1888)
//   k_coarse_cells     coarse occupancy (all six ratios 0) and per-block obstacle flags
//   k_coarse_diag      diagonal of the face-ratio system (ZQ_InitMatOpenPoisson3D,
//                      Utils3D:476-601: domain faces weight 1, free neighbours their ratio)
//   k_fine2coarse      coarse face = mean of its fine faces (Utils3D:2170-2258)
//   k_coarse_div / k_coarse_sor   red-black SOR of the coarse system
//   k_coarse_delta     (u - grad p) - u on faces with ratio > 0 (Utils3D:2611-2642, 2794-2866)
//   k_coarse2fine      the delta added to free fine faces (Utils3D:3172-3296)
//   k_subproj_gather / k_subproj_fast / k_subproj_obstacle
//                      exact projection inside every s^3 block (Utils3D:3298-3685):
//                      dense matrix for obstacle-free blocks, CG in double on the
//                      least-squares problem of ZQ_SolveSubGrid3D (Utils3D:1393-1521)
//                      for the others.
// Every expression follows the oracle's order (oracle/zqs_oracle.cpp,
// project_coarse); the least-squares CG reduces in a fixed tree order and so
// agrees with the oracle's sequential CG to rounding, not bit for bit.
#include <cooperative_groups.h>

#include <algorithm>
#include <climits>
#include <map>
#include <mutex>

#include "zqs_coarse.h"

namespace zqs {

namespace {

__device__ __forceinline__ bool fine_occ(const Layout& L, const uint8_t* __restrict__ flags, int x, int y, int z) {
    return (__ldg(flags + lidx(L, x, y, z)) & F_FREE) == 0;
}

// One thread per coarse face index (i <= cW, j <= cH, k <= cD), three components.
__global__ void k_coarse_ratios(Layout L, Layout Lc, int s, const uint8_t* __restrict__ flags,
                                float* __restrict__ ru, float* __restrict__ rv, float* __restrict__ rw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > Lc.W || j > Lc.H || k > Lc.D) return;
    const int c = lidx(Lc, i, j, k);
    const float area = (float)(s * s);
    if (j < Lc.H && k < Lc.D) {
        int n = 0;
        for (int sk = 0; sk < s; sk++)
            for (int sj = 0; sj < s; sj++) {
                const int y = j * s + sj, z = k * s + sk;
                bool o;
                if (i == 0) o = fine_occ(L, flags, 0, y, z);
                else if (i == Lc.W) o = fine_occ(L, flags, L.W - 1, y, z);
                else o = fine_occ(L, flags, i * s, y, z) || fine_occ(L, flags, i * s - 1, y, z);
                n += o ? 1 : 0;
            }
        ru[c] = 1.0f - (float)n / area;
    }
    if (i < Lc.W && k < Lc.D) {
        int n = 0;
        for (int sk = 0; sk < s; sk++)
            for (int si = 0; si < s; si++) {
                const int x = i * s + si, z = k * s + sk;
                bool o;
                if (j == 0) o = fine_occ(L, flags, x, 0, z);
                else if (j == Lc.H) o = fine_occ(L, flags, x, L.H - 1, z);
                else o = fine_occ(L, flags, x, j * s, z) || fine_occ(L, flags, x, j * s - 1, z);
                n += o ? 1 : 0;
            }
        rv[c] = 1.0f - (float)n / area;
    }
    if (i < Lc.W && j < Lc.H) {
        int n = 0;
        for (int sj = 0; sj < s; sj++)
            for (int si = 0; si < s; si++) {
                const int x = i * s + si, y = j * s + sj;
                bool o;
                if (k == 0) o = fine_occ(L, flags, x, y, 0);
                else if (k == Lc.D) o = fine_occ(L, flags, x, y, L.D - 1);
                else o = fine_occ(L, flags, x, y, k * s) || fine_occ(L, flags, x, y, k * s - 1);
                n += o ? 1 : 0;
            }
        rw[c] = 1.0f - (float)n / area;
    }
}

// Coarse occupancy and the per-block obstacle flag (dense block index).
__global__ void k_coarse_cells(Layout L, Layout Lc, int s, const uint8_t* __restrict__ flags,
                               const float* __restrict__ ru, const float* __restrict__ rv,
                               const float* __restrict__ rw, uint8_t* __restrict__ occ, uint8_t* __restrict__ bobs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= Lc.W || j >= Lc.H || k >= Lc.D) return;
    const int c = lidx(Lc, i, j, k);
    const int px = Lc.px, pl = (int)Lc.plane;
    occ[c] = (ru[c] == 0.0f && ru[c + 1] == 0.0f && rv[c] == 0.0f && rv[c + px] == 0.0f && rw[c] == 0.0f &&
              rw[c + pl] == 0.0f)
                 ? 1
                 : 0;
    bool any = false;
    for (int sk = 0; sk < s && !any; sk++)
        for (int sj = 0; sj < s && !any; sj++)
            for (int si = 0; si < s; si++)
                if (fine_occ(L, flags, i * s + si, j * s + sj, k * s + sk)) {
                    any = true;
                    break;
                }
    bobs[((size_t)k * Lc.H + j) * Lc.W + i] = any ? 1 : 0;
}

// Diagonal: the count of domain faces, then the ratios of the faces to free
// in-domain neighbours in the order z-, z+, y-, y+, x-, x+.
__global__ void k_coarse_diag(Layout Lc, const float* __restrict__ ru, const float* __restrict__ rv,
                              const float* __restrict__ rw, const uint8_t* __restrict__ occ,
                              float* __restrict__ diag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= Lc.W || j >= Lc.H || k >= Lc.D) return;
    const int c = lidx(Lc, i, j, k);
    const int px = Lc.px, pl = (int)Lc.plane;
    float cnt = 0.0f;
    if (!occ[c]) {
        const int nin = (k > 0) + (k < Lc.D - 1) + (j > 0) + (j < Lc.H - 1) + (i > 0) + (i < Lc.W - 1);
        cnt = (float)(6 - nin);
        if (k > 0 && !occ[c - pl]) cnt += rw[c];
        if (k < Lc.D - 1 && !occ[c + pl]) cnt += rw[c + pl];
        if (j > 0 && !occ[c - px]) cnt += rv[c];
        if (j < Lc.H - 1 && !occ[c + px]) cnt += rv[c + px];
        if (i > 0 && !occ[c - 1]) cnt += ru[c];
        if (i < Lc.W - 1 && !occ[c + 1]) cnt += ru[c + 1];
    }
    diag[c] = cnt;
}

// Coarse face = (sum of its s x s fine faces, outer loop first) / s^2.
__global__ void k_fine2coarse(Layout L, Layout Lc, int s, const float* __restrict__ u, const float* __restrict__ v,
                              const float* __restrict__ w, float* __restrict__ cu, float* __restrict__ cv,
                              float* __restrict__ cw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > Lc.W || j > Lc.H || k > Lc.D) return;
    const int c = lidx(Lc, i, j, k);
    const float area = (float)(s * s);
    if (j < Lc.H && k < Lc.D) {
        float sum = 0.0f;
        for (int sk = 0; sk < s; sk++)
            for (int sj = 0; sj < s; sj++) sum += __ldg(u + lidx(L, i * s, j * s + sj, k * s + sk));
        cu[c] = sum / area;
    }
    if (i < Lc.W && k < Lc.D) {
        float sum = 0.0f;
        for (int sk = 0; sk < s; sk++)
            for (int si = 0; si < s; si++) sum += __ldg(v + lidx(L, i * s + si, j * s, k * s + sk));
        cv[c] = sum / area;
    }
    if (i < Lc.W && j < Lc.H) {
        float sum = 0.0f;
        for (int sj = 0; sj < s; sj++)
            for (int si = 0; si < s; si++) sum += __ldg(w + lidx(L, i * s + si, j * s + sj, k * s));
        cw[c] = sum / area;
    }
}

__global__ void k_coarse_div(Layout Lc, const float* __restrict__ cu, const float* __restrict__ cv,
                             const float* __restrict__ cw, const uint8_t* __restrict__ occ, float* __restrict__ div,
                             float* __restrict__ p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= Lc.W || j >= Lc.H || k >= Lc.D) return;
    const int c = lidx(Lc, i, j, k);
    const int px = Lc.px, pl = (int)Lc.plane;
    div[c] = occ[c] ? 0.0f : ((((cu[c + 1] - cu[c]) + cv[c + px]) - cv[c]) + cw[c + pl]) - cw[c];
    p[c] = 0.0f;  // cold start every projection
}

// One colour of the face-ratio SOR: s = ((rx- px- + rx+ px+) + (ry- py- + ry+ py+))
// + (rz- pz- + rz+ pz+) over free in-domain neighbours (+0 otherwise), then
// p = fma(omega/diag, s - div, (1-omega) p).
__global__ void k_coarse_sor(Layout Lc, const float* __restrict__ ru, const float* __restrict__ rv,
                             const float* __restrict__ rw, const uint8_t* __restrict__ occ,
                             const float* __restrict__ diag, const float* __restrict__ div, float* __restrict__ p,
                             int colour, float omega, float om1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= Lc.W || j >= Lc.H || k >= Lc.D) return;
    if (((i + j + k) & 1) != colour) return;
    const int c = lidx(Lc, i, j, k);
    if (occ[c] || diag[c] == 0.0f) return;
    const int px = Lc.px, pl = (int)Lc.plane;
    const float xm = (i > 0 && !occ[c - 1]) ? ru[c] * p[c - 1] : 0.0f;
    const float xp = (i < Lc.W - 1 && !occ[c + 1]) ? ru[c + 1] * p[c + 1] : 0.0f;
    const float ym = (j > 0 && !occ[c - px]) ? rv[c] * p[c - px] : 0.0f;
    const float yp = (j < Lc.H - 1 && !occ[c + px]) ? rv[c + px] * p[c + px] : 0.0f;
    const float zm = (k > 0 && !occ[c - pl]) ? rw[c] * p[c - pl] : 0.0f;
    const float zp = (k < Lc.D - 1 && !occ[c + pl]) ? rw[c + pl] * p[c + pl] : 0.0f;
    const float sum = ((xm + xp) + (ym + yp)) + (zm + zp);
    const float wc = omega / diag[c];
    p[c] = __fmaf_rn(wc, sum - div[c], om1 * p[c]);
}

// All K iterations of the coarse SOR in one launch of one thread-block
// cluster of kClusterCtas CTAs (small coarse grids): CTA r of the cluster
// keeps planes [r P, (r+1) P) of p in its shared memory and reads the z
// neighbours across the slab boundary from the adjacent CTA's shared memory
// (distributed shared memory); a hardware cluster barrier separates the
// half-sweeps.  Each thread owns kClusterPairs pairs of x-adjacent cells, so
// that every half-sweep updates exactly one cell of each pair (the one of that
// colour) and no lane of a warp idles; the cells' six weights, neighbour mask,
// omega/diag weight and divergence stay in registers, ordered by colour.  Same
// arithmetic as k_coarse_sor (a colour reads only the other colour, so the
// order of updates inside a half-sweep does not matter): identical results.
constexpr int kClusterCtas = 8;
constexpr int kClusterThreads = 1024;
constexpr int kClusterPairs = 2;
constexpr int kClusterCpt = 2 * kClusterPairs;

__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kClusterThreads)
    k_coarse_sor_cluster(Layout Lc, int P, const float* __restrict__ ru, const float* __restrict__ rv,
                         const float* __restrict__ rw, const uint8_t* __restrict__ occ,
                         const float* __restrict__ diag, const float* __restrict__ div, float* __restrict__ pout,
                         int K, float omega, float om1) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ float ps[];  // [P][cH][cW] this CTA's planes
    const int rank = (int)cluster.block_rank();
    const int W = Lc.W, H = Lc.H, D = Lc.D;
    const int z0 = rank * P;
    const int nloc = max(0, min(P, D - z0)) * H * W;
    for (int e = threadIdx.x; e < P * H * W; e += blockDim.x) ps[e] = 0.0f;
    float* below = rank > 0 ? cluster.map_shared_rank(ps, rank - 1) : nullptr;   // planes z0-P .. z0-1
    float* above = rank < kClusterCtas - 1 ? cluster.map_shared_rank(ps, rank + 1) : nullptr;
    // cell m = 2 q + colour: the cell of that colour in this thread's pair q
    float w6[kClusterCpt][6], wc[kClusterCpt], dv[kClusterCpt];
    unsigned mk[kClusterCpt];  // bits 0-5 free neighbours, 6 z- in the CTA below, 7 z+ in the CTA above
    int le[kClusterCpt];
    bool act[kClusterCpt];
    const int Wp = (W + 1) / 2;
    const int npairs = max(0, min(P, D - z0)) * H * Wp;
#pragma unroll
    for (int m = 0; m < kClusterCpt; m++) {
        const int pr = threadIdx.x + (m >> 1) * kClusterThreads;
        const int colour = m & 1;
        le[m] = 0;
        mk[m] = 0;
        act[m] = false;
        wc[m] = 0.0f;
        dv[m] = 0.0f;
#pragma unroll
        for (int q = 0; q < 6; q++) w6[m][q] = 0.0f;
        if (pr >= npairs) continue;
        const int pi = pr % Wp, j = (pr / Wp) % H, zl = pr / (Wp * H), k = z0 + zl;
        const int i = 2 * pi + ((colour + j + k) & 1);
        if (i >= W) continue;
        const int e = (zl * H + j) * W + i;
        le[m] = e;
        const int c = lidx(Lc, i, j, k);
        if (occ[c] || diag[c] == 0.0f) continue;
        const int px = Lc.px, pl = (int)Lc.plane;
        act[m] = true;
        if (zl == 0) mk[m] |= 64u;
        if (zl == P - 1) mk[m] |= 128u;
        // neighbours x-, x+, y-, y+, z-, z+ (bit q) that are in the domain and free
        if (i > 0 && !occ[c - 1]) mk[m] |= 1u, w6[m][0] = ru[c];
        if (i < W - 1 && !occ[c + 1]) mk[m] |= 2u, w6[m][1] = ru[c + 1];
        if (j > 0 && !occ[c - px]) mk[m] |= 4u, w6[m][2] = rv[c];
        if (j < H - 1 && !occ[c + px]) mk[m] |= 8u, w6[m][3] = rv[c + px];
        if (k > 0 && !occ[c - pl]) mk[m] |= 16u, w6[m][4] = rw[c];
        if (k < D - 1 && !occ[c + pl]) mk[m] |= 32u, w6[m][5] = rw[c + pl];
        wc[m] = omega / diag[c];
        dv[m] = div[c];
    }
    cluster.sync();
    const int plane = H * W;
    for (int it = 0; it < K; it++) {
#pragma unroll
        for (int colour = 0; colour < 2; colour++) {
#pragma unroll
            for (int q = 0; q < kClusterPairs; q++) {
                const int m = 2 * q + colour;
                if (!act[m]) continue;
                const int e = le[m];
                const float* pe = ps + e;
                const float xm = (mk[m] & 1u) ? w6[m][0] * pe[-1] : 0.0f;
                const float xp = (mk[m] & 2u) ? w6[m][1] * pe[1] : 0.0f;
                const float ym = (mk[m] & 4u) ? w6[m][2] * pe[-W] : 0.0f;
                const float yp = (mk[m] & 8u) ? w6[m][3] * pe[W] : 0.0f;
                float zm = 0.0f, zp = 0.0f;
                if (mk[m] & 16u) {
                    const float pn = (mk[m] & 64u) ? below[e + (P - 1) * plane] : pe[-plane];
                    zm = w6[m][4] * pn;
                }
                if (mk[m] & 32u) {
                    const float pn = (mk[m] & 128u) ? above[e - (P - 1) * plane] : pe[plane];
                    zp = w6[m][5] * pn;
                }
                const float sum = ((xm + xp) + (ym + yp)) + (zm + zp);
                ps[e] = __fmaf_rn(wc[m], sum - dv[m], om1 * ps[e]);
            }
            cluster.sync();
        }
    }
    for (int e = threadIdx.x; e < nloc; e += blockDim.x) {
        const int i = e % W, j = (e / W) % H, k = z0 + e / (W * H);
        pout[lidx(Lc, i, j, k)] = ps[e];
    }
}

// delta = (u - g) - u with g = p_R - p_L (p = 0 outside the domain) on faces
// whose ratio is > 0, else 0.
__global__ void k_coarse_delta(Layout Lc, const float* __restrict__ ru, const float* __restrict__ rv,
                               const float* __restrict__ rw, const float* __restrict__ cu,
                               const float* __restrict__ cv, const float* __restrict__ cw,
                               const float* __restrict__ p, float* __restrict__ du, float* __restrict__ dv,
                               float* __restrict__ dw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > Lc.W || j > Lc.H || k > Lc.D) return;
    const int c = lidx(Lc, i, j, k);
    const int px = Lc.px, pl = (int)Lc.plane;
    const float zero = 0.0f;
    if (j < Lc.H && k < Lc.D) {
        float d = 0.0f;
        if (ru[c] > 0.0f) {
            const float g = i == 0 ? p[c] - zero : (i == Lc.W ? zero - p[c - 1] : p[c] - p[c - 1]);
            d = (cu[c] - g) - cu[c];
        }
        du[c] = d;
    }
    if (i < Lc.W && k < Lc.D) {
        float d = 0.0f;
        if (rv[c] > 0.0f) {
            const float g = j == 0 ? p[c] - zero : (j == Lc.H ? zero - p[c - px] : p[c] - p[c - px]);
            d = (cv[c] - g) - cv[c];
        }
        dv[c] = d;
    }
    if (i < Lc.W && j < Lc.H) {
        float d = 0.0f;
        if (rw[c] > 0.0f) {
            const float g = k == 0 ? p[c] - zero : (k == Lc.D ? zero - p[c - pl] : p[c] - p[c - pl]);
            d = (cw[c] - g) - cw[c];
        }
        dw[c] = d;
    }
}

// One thread per fine face index; faces on coarse face planes whose fine
// cells are free take the delta of their coarse face (the x = W face tests the
// inside cell x = W-1).
__global__ void k_coarse2fine(Layout L, Layout Lc, int s, const uint8_t* __restrict__ flags,
                              const float* __restrict__ du, const float* __restrict__ dv,
                              const float* __restrict__ dw, float* __restrict__ u, float* __restrict__ v,
                              float* __restrict__ w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > L.W || j > L.H || k > L.D) return;
    const int c = lidx(L, i, j, k);
    if (j < L.H && k < L.D && i % s == 0) {
        bool ok;
        if (i == 0) ok = !fine_occ(L, flags, 0, j, k);
        else if (i == L.W) ok = !fine_occ(L, flags, L.W - 1, j, k);
        else ok = !fine_occ(L, flags, i, j, k) && !fine_occ(L, flags, i - 1, j, k);
        if (ok) u[c] = u[c] + __ldg(du + lidx(Lc, i / s, j / s, k / s));
    }
    if (i < L.W && k < L.D && j % s == 0) {
        bool ok;
        if (j == 0) ok = !fine_occ(L, flags, i, 0, k);
        else if (j == L.H) ok = !fine_occ(L, flags, i, L.H - 1, k);
        else ok = !fine_occ(L, flags, i, j, k) && !fine_occ(L, flags, i, j - 1, k);
        if (ok) v[c] = v[c] + __ldg(dv + lidx(Lc, i / s, j / s, k / s));
    }
    if (i < L.W && j < L.H && k % s == 0) {
        bool ok;
        if (k == 0) ok = !fine_occ(L, flags, i, j, 0);
        else if (k == L.D) ok = !fine_occ(L, flags, i, j, L.D - 1);
        else ok = !fine_occ(L, flags, i, j, k) && !fine_occ(L, flags, i, j, k - 1);
        if (ok) w[c] = w[c] + __ldg(dw + lidx(Lc, i / s, j / s, k / s));
    }
}

__device__ __forceinline__ int block_face(const Layout& L, int s, int q, int bi, int bj, int bk, int& comp) {
    return subproj_block_face(L, s, q, bi, bj, bk, comp);
}

__device__ __forceinline__ int interior_face(int s, int r) { return subproj_interior_face(s, r); }

__device__ __forceinline__ float* comp_ptr(int comp, float* u, float* v, float* w) {
    return comp == 0 ? u : (comp == 1 ? v : w);
}

// X[b * nf + q] = block face q of block b.
__global__ void k_subproj_gather(Layout L, Layout Lc, int s, int nf, long long total, const float* __restrict__ u,
                                 const float* __restrict__ v, const float* __restrict__ w, float* __restrict__ X) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    const int b = (int)(e / nf), q = (int)(e - (long long)b * nf);
    const int bi = b % Lc.W, bj = (b / Lc.W) % Lc.H, bk = b / (Lc.W * Lc.H);
    int comp;
    const int c = block_face(L, s, q, bi, bj, bk, comp);
    X[e] = __ldg((comp == 0 ? u : (comp == 1 ? v : w)) + c);
}

// Obstacle-free blocks as one matrix product Y = M X (rows x nblocks, inner
// dimension nf), written to the blocks' interior fine faces.  Tiled SGEMM:
// a CTA owns a 128-row x 128-block tile; 16-deep slices of M (from its
// transpose MT[q][r]) and X (X[b][q]) are staged through shared memory, double
// buffered; thread (tx, ty) accumulates rows 8 ty + i and blocks 8 tx + j
// (i, j < 8; two 16-byte shared loads each per step) with fused multiply-adds
// in q order from 0, so every output is the sequential sum of the oracle
// (padding beyond nf adds exact zeros).
constexpr int kGemmTile = 128;
constexpr int kGemmK = 16;
constexpr int kGemmThreads = 256;

__global__ void __launch_bounds__(kGemmThreads, 2) k_subproj_fast(Layout L, Layout Lc, int s, int nf, int rows,
                                                               int nblocks, const float* __restrict__ MT,
                                                               const float* __restrict__ X,
                                                               const uint8_t* __restrict__ bobs,
                                                               float* __restrict__ u, float* __restrict__ v,
                                                               float* __restrict__ w) {
    __shared__ __align__(16) float As[2][kGemmK][kGemmTile];
    // B rows padded by 4 floats: the transposing stores (16 q of one block per
    // 16 threads) then spread over 8 banks instead of one
    __shared__ __align__(16) float Bs[2][kGemmK][kGemmTile + 4];
    const int t = threadIdx.x;
    const int tx = t & 15, ty = t >> 4;
    const int r0 = blockIdx.x * kGemmTile, b0 = blockIdx.y * kGemmTile;
    // one slice: 2048 elements of each of A (q-major, 128 rows per q) and B
    // (block-major, 16 q per block); eight of each per thread
    float ra[8], rb[8];
    auto load = [&](int q0) {
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int idx = t + e * kGemmThreads;  // 0 .. 2047
            const int kk = idx >> 7, c = idx & 127;
            const int q = q0 + kk, r = r0 + c;
            ra[e] = (q < nf && r < rows) ? __ldg(MT + (size_t)q * rows + r) : 0.0f;
            // B: 128 blocks x 16 q, q fastest within a block
            const int bb = idx >> 4, k2 = idx & 15;
            const int qb = q0 + k2, b = b0 + bb;
            rb[e] = (qb < nf && b < nblocks) ? __ldg(X + (size_t)b * nf + qb) : 0.0f;
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int idx = t + e * kGemmThreads;
            As[buf][idx >> 7][idx & 127] = ra[e];
            Bs[buf][idx & 15][idx >> 4] = rb[e];
        }
    };
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = 0.0f;
    const int nk = (nf + kGemmK - 1) / kGemmK;
    load(0);
    store(0);
    __syncthreads();
    for (int kt = 0; kt < nk; kt++) {
        const int buf = kt & 1;
        if (kt + 1 < nk) load((kt + 1) * kGemmK);
#pragma unroll
        for (int kk = 0; kk < kGemmK; kk++) {
            float a[8], bv[8];
            const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][8 * ty]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][8 * ty + 4]);
            const float4 c0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][8 * tx]);
            const float4 c1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][8 * tx + 4]);
            a[0] = a0.x, a[1] = a0.y, a[2] = a0.z, a[3] = a0.w, a[4] = a1.x, a[5] = a1.y, a[6] = a1.z, a[7] = a1.w;
            bv[0] = c0.x, bv[1] = c0.y, bv[2] = c0.z, bv[3] = c0.w, bv[4] = c1.x, bv[5] = c1.y, bv[6] = c1.z,
            bv[7] = c1.w;
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = __fmaf_rn(a[i], bv[j], acc[i][j]);
        }
        if (kt + 1 < nk) store(buf ^ 1);
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int r = r0 + 8 * ty + i;
        if (r >= rows) continue;
        const int f = interior_face(s, r);
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int gb = b0 + 8 * tx + j;
            if (gb >= nblocks || bobs[gb]) continue;
            const int bi = gb % Lc.W, bj = (gb / Lc.W) % Lc.H, bk = gb / (Lc.W * Lc.H);
            int comp;
            const int c = block_face(L, s, f, bi, bj, bk, comp);
            comp_ptr(comp, u, v, w)[c] = acc[i][j];
        }
    }
}

// Blocks with obstacles: one thread per block cell, at most this many.
constexpr int kMaxBlockCells = 1024;

// Sum over the CTA in a fixed order (warp trees, then the warp sums in warp
// order by the first warp); blockDim.x is a multiple of 32, at most 1024.
__device__ double block_sum(double x, double* red) {
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[wid] = x;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        double y = lane < nw ? red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) y += __shfl_down_sync(0xffffffffu, y, o);
        if (lane == 0) red[32] = y;
    }
    __syncthreads();
    const double r = red[32];
    __syncthreads();
    return r;
}

__device__ int block_min(int x, int* redi) {
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = min(x, __shfl_down_sync(0xffffffffu, x, o));
    if (lane == 0) redi[wid] = x;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        int y = lane < nw ? redi[lane] : INT_MAX;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) y = min(y, __shfl_down_sync(0xffffffffu, y, o));
        if (lane == 0) redi[32] = y;
    }
    __syncthreads();
    const int r = redi[32];
    __syncthreads();
    return r;
}

// Blocks with an occupied fine cell (ZQ_SolveSubGrid3D, Utils3D:1393-1521):
// the least-squares pressure of the block's closed Poisson problem.  The
// least-squares solutions of A p = b (A the Laplacian of the free cells, weight
// 1 between free neighbours) are the solutions of A p = b' with b' = b minus
// its mean over each connected free region, unique up to a constant per
// region, which the face corrections do not see.  So: label the regions (min
// cell index, propagated), remove each region's mean (regions in increasing
// root order, fixed-order sums), then CG on -A p = -b' in double from 0 to a
// relative residual of 1e-12 (the reference's PCG tolerance), one thread per
// cell.  Pressures rounded to float; interior faces between free cells get
// -(p_b - p_a).
//
// The block's faces are read from u, v, w directly: the divergence reads
// happen before any write, and each interior face is written only by the
// thread that read its value (the +x/+y/+z faces of other cells are boundary
// faces of the block, never written here).
__global__ void k_subproj_obstacle(Layout L, Layout Lc, int s, int nf, const uint8_t* __restrict__ flags,
                                   const uint8_t* __restrict__ bobs, float* u, float* v, float* w) {
    const int b = blockIdx.x;
    if (!bobs[b]) return;
    extern __shared__ double sm[];
    const int nthr = blockDim.x;
    double* pd = sm;                                      // [nthr] direction
    double* tv = pd + nthr;                               // [nthr] scratch; pressures as float at the end
    int* lab = reinterpret_cast<int*>(tv + nthr);         // [nthr] region labels
    __shared__ double red[33];
    __shared__ int redi[33];
    const int n = s * s * s;
    const int c = threadIdx.x;
    const int bi = b % Lc.W, bj = (b / Lc.W) % Lc.H, bk = b / (Lc.W * Lc.H);
    const int ci = c % s, cj = (c / s) % s, ck = c / (s * s);
    const bool in = c < n;
    const bool occ = in ? fine_occ(L, flags, bi * s + ci, bj * s + cj, bk * s + ck) : true;
    const bool fr = in && !occ;
    // free in-block neighbours in the order z-, z+, y-, y+, x-, x+ (bit q), their count
    const int dk[6] = {-1, 1, 0, 0, 0, 0}, dj[6] = {0, 0, -1, 1, 0, 0}, di[6] = {0, 0, 0, 0, -1, 1};
    const int off[6] = {-s * s, s * s, -s, s, -1, 1};
    unsigned nbm = 0;
    int cnt = 0;
    if (fr) {
#pragma unroll
        for (int q = 0; q < 6; q++) {
            const int a = ci + di[q], bb = cj + dj[q], e = ck + dk[q];
            if (a < 0 || a >= s || bb < 0 || bb >= s || e < 0 || e >= s) continue;
            if (fine_occ(L, flags, bi * s + a, bj * s + bb, bk * s + e)) continue;
            nbm |= 1u << q;
            cnt++;
        }
    }
    // regions: every free cell takes the smallest index reachable (at most n rounds)
    lab[c] = fr ? c : INT_MAX;
    __syncthreads();
    for (int round = 0; round < n; round++) {
        int m = lab[c];
        if (fr)
#pragma unroll
            for (int q = 0; q < 6; q++)
                if (nbm & (1u << q)) m = min(m, lab[c + off[q]]);
        __syncthreads();
        const bool ch = fr && m < lab[c];
        if (ch) lab[c] = m;
        if (!__syncthreads_or(ch)) break;
    }
    // this cell's padded index: its -x/-y/-z faces sit there in u/v/w
    const int fc = lidx(L, bi * s + ci, bj * s + cj, bk * s + ck);
    // right-hand side: the float divergence of the free cell, minus its region's mean
    double bval = 0.0;
    if (fr) {
        const float dvg = ((((u[fc + 1] - u[fc]) + v[fc + L.px]) - v[fc]) + w[fc + (int)L.plane]) - w[fc];
        bval = (double)dvg;
    }
    double bp = bval;
    bool done = !fr;
    for (;;) {
        const int root = block_min(done ? INT_MAX : lab[c], redi);
        if (root == INT_MAX) break;
        const bool mine = fr && lab[c] == root;
        const double sum = block_sum(mine ? bval : 0.0, red);
        const double num = block_sum(mine ? 1.0 : 0.0, red);
        if (mine) {
            bp = bval - sum / num;
            done = true;
        }
    }
    // CG on -A x = -b'
    auto applyM = [&](const double* x, double xc) -> double {
        if (!fr) return 0.0;
        double acc = 0.0;
#pragma unroll
        for (int q = 0; q < 6; q++)
            if (nbm & (1u << q)) acc += x[c + off[q]];
        return (double)cnt * xc - acc;
    };
    double xv = 0.0;
    double rv = -bp;
    pd[c] = rv;
    __syncthreads();
    double rr = block_sum(rv * rv, red);
    const double rr0 = rr;
    const int maxit = 2 * (n + nf + 1);
    for (int it = 0; it < maxit && rr > 1e-24 * rr0 && rr > 0.0; it++) {
        const double pc = pd[c];
        const double t = applyM(pd, pc);
        const double pt = block_sum(pc * t, red);
        if (!(pt > 0.0)) break;
        const double alpha = rr / pt;
        xv += alpha * pc;
        rv = rv - alpha * t;
        const double rn = block_sum(rv * rv, red);
        const double beta = rn / rr;
        rr = rn;
        pd[c] = rv + beta * pc;
        __syncthreads();
    }
    // pressures to float, then the interior faces between free cells
    float* pf = reinterpret_cast<float*>(tv);
    pf[c] = (float)xv;
    __syncthreads();
    if (!fr) return;
    auto put = [&](int comp, int lo) {
        const float d = -(pf[c] - pf[lo]);
        float* f = comp_ptr(comp, u, v, w) + fc;
        *f = *f + d;
    };
    if (nbm & (1u << 4)) put(0, c - 1);
    if (nbm & (1u << 2)) put(1, c - s);
    if (nbm & (1u << 0)) put(2, c - s * s);
}

// The sub-projection matrix per block edge, transposed on the device, shared by
// every grid of the process.
std::mutex g_mt_mu;
std::map<int, float*> g_mt;

int get_mt(int s, const float** out) {
    std::lock_guard<std::mutex> lk(g_mt_mu);
    auto it = g_mt.find(s);
    if (it != g_mt.end()) {
        *out = it->second;
        return ZQS_OK;
    }
    const std::vector<float> M = coarse_submatrix(s);
    const int nf = 3 * s * s * (s + 1), rows = 3 * s * s * (s - 1);
    std::vector<float> MT((size_t)nf * rows);
    for (int r = 0; r < rows; r++)
        for (int q = 0; q < nf; q++) MT[(size_t)q * rows + r] = M[(size_t)r * nf + q];
    float* d = nullptr;
    ZQS_CUDA_TRY(dev_alloc(&d, MT.size() * sizeof(float)));
    cudaError_t e = cudaMemcpy(d, MT.data(), MT.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(e, "coarse sub-projection matrix upload");
    }
    g_mt[s] = d;
    *out = d;
    return ZQS_OK;
}

Layout coarse_layout(int W, int H, int D) {
    Layout L;
    L.W = W;
    L.H = H;
    L.D = D;
    L.px = ((W + 1) + 3) / 4 * 4;
    L.py = H + 1;
    L.pz = D + 1;
    L.plane = (long long)L.px * L.py;
    L.elems = L.plane * (L.pz + 2);
    return L;
}

}  // namespace

namespace {

// The tensor-core operands and the timeout flag of a state with s > 1.
int coarse_alloc_tc(CoarseState* c) {
    if (c->s < 2 || c->Xsplit) return ZQS_OK;
    int rc = subproj_tc_prepare(c->s);
    if (rc) return rc;
    ZQS_CUDA_TRY(dev_alloc(&c->Xsplit, subproj_tc_split_bytes(c->nblocks, c->nf)));
    if (!c->err) {
        ZQS_CUDA_TRY(dev_alloc(&c->err, sizeof(int)));
        ZQS_CUDA_TRY(cudaMemset(c->err, 0, sizeof(int)));
    }
    return ZQS_OK;
}

}  // namespace

int coarse_check(CoarseState* cs, cudaStream_t st) {
    if (!cs || !cs->err) return ZQS_OK;
    ZQS_CUDA_TRY(cudaStreamSynchronize(st));
    int flag = 0;
    ZQS_CUDA_TRY(cudaMemcpy(&flag, cs->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (!flag) return ZQS_OK;
    ZQS_CUDA_TRY(cudaMemset(cs->err, 0, sizeof(int)));
    set_error("coarse projection: a tensor-core pipeline wait timed out; those blocks were not projected");
    return ZQS_ETIMEOUT;
}

int coarse_prepare(CoarseState*& cs, const Layout& L, int s, int tc) {
    if (s < 1 || L.W % s || L.H % s || L.D % s) {
        set_error("sub_size must be >= 1 and divide the grid's width, height and depth");
        return ZQS_EINVAL;
    }
    if (s * s * s > kMaxBlockCells) {
        set_error("sub_size must be at most 10 (one thread per block cell)");
        return ZQS_EINVAL;
    }
    if (cs && cs->s == s && cs->Lc.W == L.W / s && cs->Lc.H == L.H / s && cs->Lc.D == L.D / s) {
        cs->tc = tc ? 1 : 0;
        return cs->tc ? coarse_alloc_tc(cs) : ZQS_OK;
    }
    coarse_free(cs);
    CoarseState* c = new CoarseState();
    c->s = s;
    c->Lc = coarse_layout(L.W / s, L.H / s, L.D / s);
    const Layout& Lc = c->Lc;
    c->nblocks = Lc.W * Lc.H * Lc.D;
    c->nf = 3 * s * s * (s + 1);
    c->rows = 3 * s * s * (s - 1);
    const size_t fb = (size_t)Lc.elems * 4;
    const size_t ob = ((size_t)Lc.elems + 255) / 256 * 256;
    const size_t bb = ((size_t)c->nblocks + 255) / 256 * 256;
    const size_t xb = s > 1 ? (size_t)c->nblocks * c->nf * 4 : 0;
    const size_t total = 12 * fb + ob + bb + xb;
    cudaError_t e = dev_alloc(&c->base, total);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "coarse state allocation");
    }
    e = cudaMemset(c->base, 0, total);
    if (e != cudaSuccess) {
        cudaFree(c->base);
        delete c;
        return cuda_fail(e, "coarse state clear");
    }
    char* b = (char*)c->base;
    auto take = [&]() -> float* {
        float* p = (float*)b + Lc.plane;
        b += fb;
        return p;
    };
    c->ru = take();
    c->rv = take();
    c->rw = take();
    c->cu = take();
    c->cv = take();
    c->cw = take();
    c->du = take();
    c->dv = take();
    c->dw = take();
    c->div = take();
    c->diag = take();
    c->p = take();
    c->occ = (uint8_t*)b + Lc.plane;
    b += ob;
    c->bobs = (uint8_t*)b;
    b += bb;
    c->X = s > 1 ? (float*)b : nullptr;
    c->tc = tc ? 1 : 0;
    if (s > 1) {
        int rc = get_mt(s, &c->MT);
        if (!rc && c->tc) rc = coarse_alloc_tc(c);
        if (rc) {
            coarse_free(c);
            return rc;
        }
    }
    cs = c;
    return ZQS_OK;
}

void coarse_free(CoarseState*& cs) {
    if (!cs) return;
    cudaFree(cs->base);
    if (cs->Xsplit) cudaFree(cs->Xsplit);
    if (cs->err) cudaFree(cs->err);
    delete cs;
    cs = nullptr;
}

int launch_project_coarse(DevGrid& g, const KParams& kp, int K, cudaStream_t st, LaunchCounter& lc) {
    CoarseState* cs = g.coarse;
    if (!cs) {
        set_error("coarse projection: the grid has no coarse state (set the parameters first)");
        return ZQS_ENOTREADY;
    }
    const Layout& L = g.L;
    const Layout& Lc = cs->Lc;
    const int s = cs->s;
    dim3 b(32, 8, 1);
    const dim3 gcf((Lc.W + 1 + 31) / 32, (Lc.H + 1 + 7) / 8, Lc.D + 1);  // coarse face box
    const dim3 gcc((Lc.W + 31) / 32, (Lc.H + 7) / 8, Lc.D);               // coarse cells
    const dim3 gff((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, L.D + 1);      // fine face box
    k_coarse_ratios<<<gcf, b, 0, st>>>(L, Lc, s, g.flags, cs->ru, cs->rv, cs->rw);
    k_coarse_cells<<<gcc, b, 0, st>>>(L, Lc, s, g.flags, cs->ru, cs->rv, cs->rw, cs->occ, cs->bobs);
    k_coarse_diag<<<gcc, b, 0, st>>>(Lc, cs->ru, cs->rv, cs->rw, cs->occ, cs->diag);
    k_fine2coarse<<<gcf, b, 0, st>>>(L, Lc, s, g.u, g.v, g.w, cs->cu, cs->cv, cs->cw);
    k_coarse_div<<<gcc, b, 0, st>>>(Lc, cs->cu, cs->cv, cs->cw, cs->occ, cs->div, cs->p);
    lc.n += 5;
    // small coarse grids: every iteration in one cluster launch; else one launch per colour
    const int P = (Lc.D + kClusterCtas - 1) / kClusterCtas;
    if (K > 0 && P * Lc.H * ((Lc.W + 1) / 2) <= kClusterThreads * kClusterPairs) {
        const size_t smc = (size_t)P * Lc.H * Lc.W * sizeof(float);
        k_coarse_sor_cluster<<<kClusterCtas, kClusterThreads, smc, st>>>(Lc, P, cs->ru, cs->rv, cs->rw, cs->occ,
                                                                       cs->diag, cs->div, cs->p, K, kp.omega,
                                                                       kp.om1);
        lc.n++;
    } else {
        for (int it = 0; it < K; it++)
            for (int colour = 0; colour < 2; colour++) {
                k_coarse_sor<<<gcc, b, 0, st>>>(Lc, cs->ru, cs->rv, cs->rw, cs->occ, cs->diag, cs->div, cs->p,
                                                colour, kp.omega, kp.om1);
                lc.n++;
            }
    }
    k_coarse_delta<<<gcf, b, 0, st>>>(Lc, cs->ru, cs->rv, cs->rw, cs->cu, cs->cv, cs->cw, cs->p, cs->du, cs->dv,
                                      cs->dw);
    k_coarse2fine<<<gff, b, 0, st>>>(L, Lc, s, g.flags, cs->du, cs->dv, cs->dw, g.u, g.v, g.w);
    lc.n += 2;
    ZQS_LAUNCH_CHECK("coarse correction");
    if (s > 1) {
        if (cs->tc && cs->Xsplit) {
            // gathers the block faces itself, into the tensor-core operand images
            int rc = launch_subproj_tc(L, Lc, s, cs->nf, cs->rows, cs->nblocks, cs->Xsplit, cs->bobs, g.u, g.v, g.w,
                                       cs->err, st, lc);
            if (rc) return rc;
        } else {
            const long long total = (long long)cs->nblocks * cs->nf;
            k_subproj_gather<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(L, Lc, s, cs->nf, total, g.u, g.v,
                                                                                g.w, cs->X);
            const dim3 gf((cs->rows + kGemmTile - 1) / kGemmTile, (cs->nblocks + kGemmTile - 1) / kGemmTile, 1);
            k_subproj_fast<<<gf, kGemmThreads, 0, st>>>(L, Lc, s, cs->nf, cs->rows, cs->nblocks, cs->MT, cs->X,
                                                        cs->bobs, g.u, g.v, g.w);
            lc.n += 2;
        }
        int nthr = 32;
        while (nthr < s * s * s) nthr <<= 1;
        const size_t smo = (size_t)2 * nthr * sizeof(double) + (size_t)nthr * sizeof(int);
        k_subproj_obstacle<<<cs->nblocks, nthr, smo, st>>>(L, Lc, s, cs->nf, g.flags, cs->bobs, g.u, g.v, g.w);
        lc.n += 1;
        ZQS_LAUNCH_CHECK("block sub-projection");
    }
    return ZQS_OK;
}

}  // namespace zqs
