// Pressure projection: divergence, fixed-K red-black SOR, gradient subtraction.
//
// Restates ZQ_CUDA_PoissonSolver3D::Solve{Open,Closed}PoissonRedBlackwithOccupy3D_MAC,
// whose source is not part of the reference tree (call sites
// ZQ_SmokeSimulationUtils3D.cpp:2354-2363, 2424-2437).  The rule is the one the
// oracle states (oracle/zqs_oracle.cpp, project()):
//   div  = ((((u[i+1]-u[i]) + v[j+1]) - v[j]) + w[k+1]) - w[k]   (closed: minus the FP64 mean)
//   red cells ((i+j+k)&1)==0 then black, each free cell:
//     s  = ((p[x-] + p[x+]) + (p[y-] + p[y+])) + (p[z-] + p[z+])
//     p  = fma(omega/cnt, s - div, (1-omega)*p)   (omega/cnt rounded once)
//   u -= p_R - p_L on live faces (open domain faces use p = 0 outside).
// Non-free cells and everything outside the domain hold p = +0 permanently,
// so summing all six neighbours equals the oracle's sum, which substitutes +0
// for the neighbours it excludes.
//
// Two SOR kernels:
//   k_sor_colour  one launch per colour, in place: the plain form, and the
//                 colour-race self-check of the fused kernel.
//   k_sor_rb<S>   S half-sweeps (S/2 iterations) per HBM pass.  A CTA owns a
//                 TX x TY tile plus an S-cell halo and streams a z chunk through
//                 a ring of 2S+2 shared-memory planes.  One thread per (red,
//                 black) cell pair along x; each plane is stored colour-
//                 compressed (red cells and black cells in separate arrays), so
//                 every neighbour read of a warp is contiguous.  Half-sweep s
//                 runs on plane t-2s at step t over the tile grown by S-s cells:
//                 the two-plane lag lets all S half-sweeps of a step run at once
//                 with one barrier per step, and every value each reads is at the
//                 right sweep.  Results equal S/2 iterations of k_sor_colour.
#include "zqs_adjoint.h"
#include "zqs_batch.h"
#include "zqs_coarse.h"

#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <set>
#include <sstream>
#include <string>
#include <vector>

namespace zqs {

namespace {

// Divergence of one 32x8 block at plane bz; with want_partials the block's FP64
// sum and free-cell count go to part[2*blk], part[2*blk+1].
__device__ __forceinline__ void divergence_tile(const Layout& L, const float* __restrict__ u,
                                                const float* __restrict__ v, const float* __restrict__ w,
                                                const uint8_t* __restrict__ flags, float* __restrict__ div,
                                                float* __restrict__ p, double* __restrict__ part, int want_partials,
                                                int bx, int by, int bz, long long blk) {
    const int i = bx * 32 + threadIdx.x;
    const int j = by * 8 + threadIdx.y;
    const int k = bz;
    double sum = 0.0, cnt = 0.0;
    if (i < L.W && j < L.H && k < L.D) {
        const int c = lidx(L, i, j, k);
        if (__ldg(flags + c) & F_FREE) {
            float d = ((((__ldg(u + c + 1) - __ldg(u + c)) + __ldg(v + c + L.px)) - __ldg(v + c)) +
                       __ldg(w + c + (int)L.plane)) -
                      __ldg(w + c);
            div[c] = d;
            p[c] = 0.0f;
            sum = (double)d;
            cnt = 1.0;
        }
    }
    if (want_partials) {
        // fixed-shape block reduction (deterministic)
        __shared__ double ss[256], sc[256];
        const int t = threadIdx.y * blockDim.x + threadIdx.x;
        ss[t] = sum;
        sc[t] = cnt;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (t < o) {
                ss[t] += ss[t + o];
                sc[t] += sc[t + o];
            }
            __syncthreads();
        }
        if (t == 0) {
            part[2 * blk] = ss[0];
            part[2 * blk + 1] = sc[0];
        }
        __syncthreads();  // the shared partials are reused by the next tile of a persistent block
    }
}

__global__ void k_divergence(Layout L, const float* __restrict__ u, const float* __restrict__ v,
                             const float* __restrict__ w, const uint8_t* __restrict__ flags, float* __restrict__ div,
                             float* __restrict__ p, double* __restrict__ part, int want_partials) {
    const long long blk = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    divergence_tile(L, u, v, w, flags, div, p, part, want_partials, blockIdx.x, blockIdx.y, blockIdx.z, blk);
}

// Single block: sums the partials in a fixed order, stores the mean in out[0].
__global__ void k_reduce_mean(const double* __restrict__ part, long long nblocks, double* __restrict__ out) {
    __shared__ double ss[256], sc[256];
    double s = 0.0, c = 0.0;
    for (long long b = threadIdx.x; b < nblocks; b += 256) {
        s += part[2 * b];
        c += part[2 * b + 1];
    }
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = c;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            ss[threadIdx.x] += ss[threadIdx.x + o];
            sc[threadIdx.x] += sc[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sc[0] > 0.0 ? ss[0] / sc[0] : 0.0;
        out[1] = sc[0];
    }
}

__global__ void k_div_subtract_mean(Layout L, const uint8_t* __restrict__ flags, float* __restrict__ div,
                                    const double* __restrict__ mean) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    if (__ldg(flags + c) & F_FREE) {
        const float m = (float)mean[0];
        div[c] = div[c] - m;
    }
}

__global__ void k_div_subtract_const(Layout L, const uint8_t* __restrict__ flags, float* __restrict__ div, float m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    if (__ldg(flags + c) & F_FREE) div[c] = div[c] - m;
}

// p = (1-omega) p + (omega/cnt)(s - d), evaluated as one fused multiply-add
// with the per-cell weight wc = omega/cnt (one rounding), as the oracle does.
__device__ __forceinline__ float sor_update(float pc, float s, float d, float wc, float om1) {
    return __fmaf_rn(wc, s - d, om1 * pc);
}

// One colour, in place; one thread per cell.
__global__ void k_sor_colour(Layout L, float* __restrict__ p, const float* __restrict__ div,
                             const uint8_t* __restrict__ flags, int colour, float omega, float om1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    if (((i + j + k) & 1) != colour) return;
    const int c = lidx(L, i, j, k);
    const uint8_t f = __ldg(flags + c);
    const int cnt = (f & F_CNT_MASK) >> F_CNT_SHIFT;
    if (!(f & F_FREE) || cnt == 0) return;
    const int px = L.px, pl = (int)L.plane;
    const float s = ((p[c - 1] + p[c + 1]) + (p[c - px] + p[c + px])) + (p[c - pl] + p[c + pl]);
    p[c] = sor_update(p[c], s, __ldg(div + c), omega / (float)cnt, om1);
}

template <int S, int TX, int TY, int PPT>
struct RbShape {
    static_assert(S % 2 == 0 && TX % 2 == 0, "S and TX must be even");
    static constexpr int RW = TX + 2 * S;  // region width in cells
    static constexpr int RH = TY + 2 * S;  // region height
    static_assert(RH % PPT == 0, "region rows must split evenly over a thread's pairs");
    static constexpr int PW = RW / 2;      // cell pairs per row
    static constexpr int CA = PW * RH;     // pairs (= cells of one colour) per plane
    static constexpr int NT = CA / PPT;    // threads per CTA; pair q of thread t is t + q*NT
    static constexpr int NP = 2 * S + 2;   // ring planes
    static constexpr size_t smem = (size_t)NP * 2 * CA * (4 + 4 + 1);
};

// The t loop is unrolled by the ring size NP, so every shared-memory slot of a
// step is a compile-time constant and each access is base + immediate.
template <int S, int TX, int TY, int PPT>
__global__ void __launch_bounds__(RbShape<S, TX, TY, PPT>::NT)
    k_sor_rb(Layout L, const float* __restrict__ pin, float* __restrict__ pout, const float* __restrict__ div,
             const uint8_t* __restrict__ flags, float omega, float om1, int zc) {
    using Sh = RbShape<S, TX, TY, PPT>;
    constexpr int PW = Sh::PW, NP = Sh::NP, CA = Sh::CA, NT = Sh::NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sp = reinterpret_cast<float*>(smem_raw);              // [NP][2][CA] pressure, colour-compressed
    float* sd = sp + NP * 2 * CA;                                  // [NP][2][CA] divergence
    uint8_t* sf = reinterpret_cast<uint8_t*>(sd + NP * 2 * CA);    // [NP][2][CA] flags

    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, L.D);
    const int plane = (int)L.plane;

    int me[PPT], jrow[PPT], gaddr[PPT];
    unsigned amask[PPT];
    bool pin_ok[PPT], out_ok[PPT];
#pragma unroll
    for (int q = 0; q < PPT; q++) {
        const int e = threadIdx.x + q * NT;
        const int row = e / PW, m = e - row * PW;
        me[q] = e;
        const int xl = x0 - S + 2 * m;  // left cell of the pair (even)
        const int j = y0 - S + row;
        jrow[q] = j;
        const int ly = row - S, lxl = 2 * m - S;
        unsigned mk = 0;
#pragma unroll
        for (int r = 0; r < S; r++)
#pragma unroll
            for (int o = 0; o < 2; o++) {
                const int lx = lxl + o;
                if (lx >= -r && lx < TX + r && ly >= -r && ly < TY + r) mk |= 1u << (2 * r + o);
            }
        amask[q] = mk;
        pin_ok[q] = xl >= 0 && xl < L.W && j >= 0 && j < L.H;
        out_ok[q] = pin_ok[q] && ly >= 0 && ly < TY && lxl >= 0 && lxl < TX;
        gaddr[q] = pin_ok[q] ? lidx(L, xl, j, z0 - S) : 0;  // dereferenced only for planes inside [0,D)
    }

    const int tbeg = z0 - S;
    const int nsteps = (z1 - z0) + 3 * S + 1;  // t = z0-S .. z1+2S
    const int flo = max(0, z0 - S), fhi = min(L.D, z1 + S);

    float2 np_[PPT], nd[PPT];
    unsigned nf[PPT];
#pragma unroll
    for (int q = 0; q < PPT; q++) {
        np_[q] = make_float2(0.0f, 0.0f);
        nd[q] = np_[q];
        nf[q] = 0;
        if (pin_ok[q] && tbeg >= flo && tbeg < fhi) {
            np_[q] = __ldg(reinterpret_cast<const float2*>(pin + gaddr[q]));
            nd[q] = __ldg(reinterpret_cast<const float2*>(div + gaddr[q]));
            nf[q] = __ldg(reinterpret_cast<const unsigned short*>(flags + gaddr[q]));
        }
    }

    for (int g = 0; g < nsteps; g += NP) {
#pragma unroll
        for (int qs = 0; qs < NP; qs++) {
            if (g + qs < nsteps) {
                const int t = tbeg + g + qs;  // plane t lives in slot qs
                // 1. the prefetched plane t into its slot
#pragma unroll
                for (int q = 0; q < PPT; q++) {
                    const int lc = (jrow[q] + t) & 1;  // colour of the left cell
                    const int a0 = lc ? CA : 0, a1 = CA - a0;
                    float* P = sp + qs * 2 * CA + me[q];
                    float* Dv = sd + qs * 2 * CA + me[q];
                    uint8_t* F = sf + qs * 2 * CA + me[q];
                    P[a0] = np_[q].x;
                    P[a1] = np_[q].y;
                    Dv[a0] = nd[q].x;
                    Dv[a1] = nd[q].y;
                    F[a0] = (uint8_t)(nf[q] & 0xffu);
                    F[a1] = (uint8_t)(nf[q] >> 8);
                }
                // 2. prefetch plane t+1 (in flight during the half-sweeps)
#pragma unroll
                for (int q = 0; q < PPT; q++) {
                    gaddr[q] += plane;
                    np_[q] = make_float2(0.0f, 0.0f);
                    nd[q] = np_[q];
                    nf[q] = 0;
                    if (pin_ok[q] && t + 1 >= flo && t + 1 < fhi) {
                        np_[q] = __ldg(reinterpret_cast<const float2*>(pin + gaddr[q]));
                        nd[q] = __ldg(reinterpret_cast<const float2*>(div + gaddr[q]));
                        nf[q] = __ldg(reinterpret_cast<const unsigned short*>(flags + gaddr[q]));
                    }
                }
                // 3. half-sweep s on plane t-2s (all S at once; they touch disjoint data)
#pragma unroll
                for (int s = 1; s <= S; s++) {
                    const int z = t - 2 * s;
                    const int r = S - s;
                    if (z >= max(z0 - r, 0) && z < min(z1 + r, L.D)) {
                        const int c = (s - 1) & 1;  // red first
                        const int sz = (qs - 2 * s + 2 * NP) % NP;
                        const int szm = (sz + NP - 1) % NP;
                        const int szp = (sz + 1) % NP;
#pragma unroll
                        for (int q = 0; q < PPT; q++) {
                            const int o = ((jrow[q] + t) & 1) ^ c;  // parity of z equals parity of t
                            if ((amask[q] >> (2 * r + o)) & 1u) {
                                const int cnt = (sf[(sz * 2 + c) * CA + me[q]] >> F_CNT_SHIFT) & 7;
                                if (cnt) {  // zero for cells that are not free
                                    const float* Po = sp + (sz * 2 + (c ^ 1)) * CA + me[q];
                                    const float sum = ((Po[o - 1] + Po[o]) + (Po[-PW] + Po[PW])) +
                                                      (sp[(szm * 2 + (c ^ 1)) * CA + me[q]] +
                                                       sp[(szp * 2 + (c ^ 1)) * CA + me[q]]);
                                    float* Pc = sp + (sz * 2 + c) * CA + me[q];
                                    *Pc = sor_update(*Pc, sum, sd[(sz * 2 + c) * CA + me[q]], omega / (float)cnt, om1);
                                }
                            }
                        }
                    }
                }
                // 4. plane t-2S-1 finished its last half-sweep in the previous step
                const int zo = t - 2 * S - 1;
                if (zo >= z0 && zo < z1) {
                    const int so = (qs - 2 * S - 1 + 2 * NP) % NP;
#pragma unroll
                    for (int q = 0; q < PPT; q++) {
                        if (out_ok[q]) {
                            const int lc = (jrow[q] + zo) & 1;
                            const float a = sp[(so * 2 + lc) * CA + me[q]];
                            const float b = sp[(so * 2 + (lc ^ 1)) * CA + me[q]];
                            *reinterpret_cast<float2*>(pout + gaddr[q] - (2 * S + 2) * plane) = make_float2(a, b);
                        }
                    }
                }
                __syncthreads();
            }
        }
    }
}

// Register-column form of k_sor_rb: each thread keeps its pair's pressure
// (both colours, every plane in flight) and flags in registers, so the self,
// same-pair x and both z neighbours never touch shared memory.  Shared memory
// holds the published pressure (for the x neighbour in the adjacent pair and
// the y neighbours) and the divergence.  Same schedule, same results.
template <int S, int TX, int TY, int PPT>
struct RegShape {
    static_assert(S % 2 == 0 && TX % 2 == 0, "S and TX must be even");
    static constexpr int RW = TX + 2 * S;
    static constexpr int RH = TY + 2 * S;
    static_assert(RH % PPT == 0, "region rows must split evenly over a thread's pairs");
    static constexpr int PW = RW / 2;
    static constexpr int CA = PW * RH;
    static constexpr int NT = CA / PPT;
    static constexpr int NP = 2 * S + 2;
    // floats ahead of the pressure ring: the branch-free half-sweep of the
    // WREG form reads its neighbours before it knows whether the pair updates,
    // and the row -1 / x -1 neighbours of the first slot fall here
    static constexpr int GUARD = (PW + 1 + 3) / 4 * 4;
    static constexpr size_t smem = (size_t)NP * 2 * CA * (4 + 4) + (size_t)GUARD * 4;
};

// One CTA tile (bx, by) of TX x TY columns over output planes [z0, z1); every
// thread of the block takes part (barriers inside), and the last step ends
// with a barrier, so a persistent block may run the next tile on the same
// shared memory.  The result of a plane does not depend on how the column's
// planes are split into ranges (each range recomputes its z halo).
//
// WREG (forward): each ring plane's update weights omega/cnt are kept in
// registers by colour (formed once when the plane arrives) and the x
// neighbour in the adjacent pair is read at one of two per-thread offsets;
// without it the flags stay in registers and each half-sweep extracts the
// stencil count and reads the weight table.  WREG takes ~10 more registers:
// it suits the one-CTA-per-SM tiles, the plain form the two-CTA ones.
//
// ADJ: the reversed SOR of the adjoint in its scaled variable q (see
// kernels_adjoint.cu): `div` carries wt = omega/cnt (0 where the forward never
// updates), flags are not read, the half-sweeps run black first, each update
// is q = (1-omega) q + wt * sum(q_n), and every cell's value before each
// update is added to acc (read and written in place by the owning thread).
// Bounded waits of the split-barrier form (SPLIT below): a wait that gives up
// counts itself here and lets the thread go on (the pass's result is then
// wrong, which the caller can detect; the kernel still ends).
__device__ unsigned int g_sor_sync_timeouts;

__device__ __forceinline__ void sor_bar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"((uint32_t)__cvta_generic_to_shared(bar)),
                 "r"(count)
                 : "memory");
}
__device__ __forceinline__ void sor_bar_inval(uint64_t* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"((uint32_t)__cvta_generic_to_shared(bar)) : "memory");
}
__device__ __forceinline__ void sor_bar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"((uint32_t)__cvta_generic_to_shared(bar))
                 : "memory");
}
__device__ __forceinline__ bool sor_bar_try(uint32_t a, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __noinline__ void sor_bar_wait_slow(uint32_t a, uint32_t parity) {
    for (int it = 0; it < (1 << 22); it++)
        if (sor_bar_try(a, parity)) return;
    atomicAdd(&g_sor_sync_timeouts, 1u);
}
// One try inline (the phase has usually completed: warps drift by less than
// a step), the bounded polling loop out of line.
__device__ __forceinline__ void sor_bar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
    if (!sor_bar_try(a, parity)) sor_bar_wait_slow(a, parity);
}

template <int S, int TX, int TY, int PPT, bool ADJ = false, bool WREG = false, bool SPLIT = false>
__device__ __forceinline__ void sor_reg_tile(const Layout& L, const float* __restrict__ pin,
                                             float* __restrict__ pout, const float* __restrict__ div,
                                             const uint8_t* __restrict__ flags, float omega, float om1, int bx,
                                             int by, int z0, int z1, float* __restrict__ acc = nullptr) {
    using Sh = RegShape<S, TX, TY, PPT>;
    constexpr int PW = Sh::PW, NP = Sh::NP, CA = Sh::CA, NT = Sh::NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sp = reinterpret_cast<float*>(smem_raw) + Sh::GUARD;  // [NP][2][CA] published pressure
    float* sd = sp + NP * 2 * CA;                                  // [NP][2][CA] divergence

    const int x0 = bx * TX, y0 = by * TY;
    const int plane = (int)L.plane;
    // forward: the update weight omega/cnt by stencil weight (entry 0 unused)
    __shared__ float wtab[8];
    if (!ADJ) {
        if (threadIdx.x < 8) wtab[threadIdx.x] = threadIdx.x ? omega / (float)threadIdx.x : 0.0f;
        __syncthreads();
    }

    constexpr bool WR = WREG && !ADJ;
    int me[PPT], jrow[PPT], gaddr[PPT], bpar[PPT], xoff[PPT][WR ? 2 : 1];
    unsigned amask[PPT], act[PPT][2];
    bool pin_ok[PPT], out_ok[PPT];
#pragma unroll
    for (int q = 0; q < PPT; q++) {
        const int e = threadIdx.x + q * NT;
        const int row = e / PW, m = e - row * PW;
        me[q] = e;
        const int xl = x0 - S + 2 * m;
        const int j = y0 - S + row;
        jrow[q] = j;
        const int ly = row - S, lxl = 2 * m - S;
        unsigned mk = 0;
#pragma unroll
        for (int r = 0; r < S; r++)
#pragma unroll
            for (int o = 0; o < 2; o++) {
                const int lx = lxl + o;
                if (lx >= -r && lx < TX + r && ly >= -r && ly < TY + r) mk |= 1u << (2 * r + o);
            }
        amask[q] = mk;
        pin_ok[q] = xl >= 0 && xl < L.W && j >= 0 && j < L.H;
        out_ok[q] = pin_ok[q] && ly >= 0 && ly < TY && lxl >= 0 && lxl < TX;
        gaddr[q] = pin_ok[q] ? lidx(L, xl, j, z0 - S) : 0;
        // plane t has parity z0 + (ring slot) since t = z0 - S + (multiple of
        // NP) + slot with S and NP even: the left cell is black at slot qs when
        // bpar ^ (qs & 1); act[q][qs & 1] bit s-1: half-sweep s updates this pair
        bpar[q] = (j + z0) & 1;
        // x neighbour in the adjacent pair: right pair (+1) when the updated
        // cell is the right one of its pair (o = bpar ^ x = 1), else left (-1)
        if (WR) {
            xoff[q][0] = e + (bpar[q] ? 1 : -1);
            xoff[q][WR ? 1 : 0] = e + (bpar[q] ? -1 : 1);
        }
#pragma unroll
        for (int par = 0; par < 2; par++) {
            unsigned a = 0;
#pragma unroll
            for (int sw = 1; sw <= S; sw++) {
                const int cs = ((sw - 1) & 1) ^ (ADJ ? 1 : 0);
                const int o = bpar[q] ^ par ^ cs;
                if ((mk >> (2 * (S - sw) + o)) & 1u) a |= 1u << (sw - 1);
            }
            act[q][par] = a;
        }
    }

    const int tbeg = z0 - S;
    const int nsteps = (z1 - z0) + 3 * S + 1;
    const int flo = max(0, z0 - S), fhi = min(L.D, z1 + S);

    float P[PPT][NP][2];     // pressure by colour, ring of planes
    float Wc[PPT][WR ? NP : 1][2];   // WREG: omega/cnt by colour (0: never updated)
    unsigned F[PPT][(ADJ || WR) ? 1 : NP];  // else: flags by colour, byte c = the colour-c cell's
    float A[PPT][ADJ ? NP : 1][2];  // ADJ: acc by colour, ring of planes
    float2 np_[PPT], nd[PPT], na[PPT];
    unsigned nf[PPT];
#pragma unroll
    for (int q = 0; q < PPT; q++) {
#pragma unroll
        for (int a = 0; a < NP; a++) P[q][a][0] = P[q][a][1] = 0.0f;
#pragma unroll
        for (int a = 0; a < (WR ? NP : 1); a++) Wc[q][a][0] = Wc[q][a][1] = 0.0f;
#pragma unroll
        for (int a = 0; a < ((ADJ || WR) ? 1 : NP); a++) F[q][a] = 0u;
#pragma unroll
        for (int a = 0; a < (ADJ ? NP : 1); a++) A[q][a][0] = A[q][a][1] = 0.0f;
        np_[q] = make_float2(0.0f, 0.0f);
        nd[q] = np_[q];
        na[q] = np_[q];
        nf[q] = 0;
        if (pin_ok[q] && tbeg >= flo && tbeg < fhi) {
            np_[q] = __ldg(reinterpret_cast<const float2*>(pin + gaddr[q]));
            nd[q] = __ldg(reinterpret_cast<const float2*>(div + gaddr[q]));
            if (!ADJ) nf[q] = __ldg(reinterpret_cast<const unsigned short*>(flags + gaddr[q]));
        }
        if (ADJ && out_ok[q] && tbeg >= z0 && tbeg < z1) na[q] = *reinterpret_cast<const float2*>(acc + gaddr[q]);
    }

    // SPLIT: the two-step spacing of every shared-memory dependence (see the
    // barrier at the end of a step) is kept with two mbarriers instead of a
    // block barrier every two steps: a thread arrives on sbar[n & 1] when it
    // has finished step n and, before step n, waits until every thread has
    // finished step n-2, so warps may run up to a step apart.
    __shared__ uint64_t sbar[2];
    if (SPLIT) {
        if (threadIdx.x == 0) {
            sor_bar_init(&sbar[0], NT);
            sor_bar_init(&sbar[1], NT);
        }
        __syncthreads();
    }

    for (int g = 0; g < nsteps; g += NP) {
        // step n = g + qs waits for phase ((n >> 1) - 1) of sbar[n & 1]; with
        // g a multiple of NP = 2S + 2 (NP/2 odd) that parity is
        // (g / NP + qs / 2 + 1) & 1
        const uint32_t gpar = (uint32_t)(g / NP) & 1u;
#pragma unroll
        for (int qs = 0; qs < NP; qs++) {
            if (g + qs < nsteps) {
                static_assert(!SPLIT || (NP / 2) % 2 == 1, "the parity rule needs NP/2 odd");
                if (SPLIT && (qs >= 2 || g > 0))
                    sor_bar_wait(&sbar[qs & 1], gpar ^ (uint32_t)((qs / 2 + 1) & 1));
                const int t = tbeg + g + qs;
                // 1. plane t: registers by colour, and publish
#pragma unroll
                for (int q = 0; q < PPT; q++) {
                    const bool lc = (bpar[q] ^ (qs & 1)) != 0;  // the left cell is black
                    P[q][qs][0] = lc ? np_[q].y : np_[q].x;
                    P[q][qs][1] = lc ? np_[q].x : np_[q].y;
                    if (WR) {
                        const float wl = wtab[(nf[q] >> F_CNT_SHIFT) & 7u];
                        const float wr = wtab[(nf[q] >> (8 + F_CNT_SHIFT)) & 7u];
                        Wc[q][WR ? qs : 0][0] = lc ? wr : wl;
                        Wc[q][WR ? qs : 0][1] = lc ? wl : wr;
                    } else if (!ADJ) {
                        F[q][ADJ ? 0 : qs] = lc ? (((nf[q] & 0xffu) << 8) | (nf[q] >> 8)) : nf[q];
                    }
                    if (ADJ) {
                        A[q][ADJ ? qs : 0][0] = lc ? na[q].y : na[q].x;
                        A[q][ADJ ? qs : 0][1] = lc ? na[q].x : na[q].y;
                    }
                    float* Pp = sp + qs * 2 * CA + me[q];
                    float* Dp = sd + qs * 2 * CA + me[q];
                    Pp[0] = P[q][qs][0];
                    Pp[CA] = P[q][qs][1];
                    Dp[0] = lc ? nd[q].y : nd[q].x;
                    Dp[CA] = lc ? nd[q].x : nd[q].y;
                }
                // 2. prefetch plane t+1
#pragma unroll
                for (int q = 0; q < PPT; q++) {
                    gaddr[q] += plane;
                    np_[q] = make_float2(0.0f, 0.0f);
                    nd[q] = np_[q];
                    nf[q] = 0;
                    if (pin_ok[q] && t + 1 >= flo && t + 1 < fhi) {
                        np_[q] = __ldg(reinterpret_cast<const float2*>(pin + gaddr[q]));
                        nd[q] = __ldg(reinterpret_cast<const float2*>(div + gaddr[q]));
                        if (!ADJ) nf[q] = __ldg(reinterpret_cast<const unsigned short*>(flags + gaddr[q]));
                    }
                    if (ADJ) {
                        na[q] = make_float2(0.0f, 0.0f);
                        if (out_ok[q] && t + 1 >= z0 && t + 1 < z1)
                            na[q] = *reinterpret_cast<const float2*>(acc + gaddr[q]);
                    }
                }
                // 3. half-sweeps
#pragma unroll
                for (int s = 1; s <= S; s++) {
                    const int z = t - 2 * s;
                    const int r = S - s;
                    if (z >= max(z0 - r, 0) && z < min(z1 + r, L.D)) {
                        const int c = ((s - 1) & 1) ^ (ADJ ? 1 : 0);
                        const int sz = (qs - 2 * s + 2 * NP) % NP;
                        const int szm = (sz + NP - 1) % NP;
                        const int szp = (sz + 1) % NP;
#pragma unroll
                        for (int q = 0; q < PPT; q++) {
                            // weight: wt from shared memory (ADJ), omega/cnt from registers
                            // (WREG), else the stencil count from the flags and the table.
                            // Branch-free: every pair forms the update and keeps its old
                            // value where the half-sweep leaves it (outside the active ring,
                            // obstacles, the domain edge), so the independent half-sweeps of
                            // a step interleave.
                            bool on = ((act[q][qs & 1] >> (s - 1)) & 1u) != 0;
                            float wgt;
                            if (ADJ) {
                                wgt = sd[(sz * 2 + c) * CA + me[q]];
                                on = on && wgt != 0.0f;
                            } else if (WR) {
                                wgt = Wc[q][WR ? sz : 0][c];
                                on = on && wgt != 0.0f;
                            } else {
                                const unsigned cnt = (F[q][(ADJ || WR) ? 0 : sz] >> (8 * c + F_CNT_SHIFT)) & 7u;
                                on = on && cnt != 0;
                                wgt = wtab[cnt];
                            }
                            const float* Po = sp + (sz * 2 + (c ^ 1)) * CA + me[q];
                            // the x neighbour in the adjacent pair: right of the pair when
                            // bpar ^ (qs & 1) ^ c is 1, else left
                            float adj;
                            if (WR) {
                                adj = sp[(sz * 2 + (c ^ 1)) * CA + xoff[q][WR ? ((qs & 1) ^ c) : 0]];
                            } else {
                                const int o = bpar[q] ^ (qs & 1) ^ c;
                                adj = Po[o ? 1 : -1];
                            }
                            const float sum = ((P[q][sz][c ^ 1] + adj) + (Po[-PW] + Po[PW])) +
                                              (P[q][szm][c ^ 1] + P[q][szp][c ^ 1]);
                            const float old = P[q][sz][c];
                            float nv;
                            if (ADJ) {
                                nv = om1 * old + wgt * sum;
                                const float a0 = A[q][ADJ ? sz : 0][c];
                                A[q][ADJ ? sz : 0][c] = on ? a0 + old : a0;
                            } else {
                                nv = sor_update(old, sum, sd[(sz * 2 + c) * CA + me[q]], wgt, om1);
                            }
                            const float res = on ? nv : old;
                            P[q][sz][c] = res;
                            sp[(sz * 2 + c) * CA + me[q]] = res;
                        }
                    }
                }
                // 4. output plane t-2S-1
                const int zo = t - 2 * S - 1;
                if (zo >= z0 && zo < z1) {
                    const int so = (qs - 2 * S - 1 + 2 * NP) % NP;
#pragma unroll
                    for (int q = 0; q < PPT; q++) {
                        if (out_ok[q]) {
                            const bool lc = (bpar[q] ^ (qs & 1) ^ 1) != 0;  // zo = t - 2S - 1
                            const float a = lc ? P[q][so][1] : P[q][so][0];
                            const float b = lc ? P[q][so][0] : P[q][so][1];
                            *reinterpret_cast<float2*>(pout + gaddr[q] - (2 * S + 2) * plane) = make_float2(a, b);
                            if (ADJ) {
                                const float aa = lc ? A[q][ADJ ? so : 0][1] : A[q][ADJ ? so : 0][0];
                                const float ab = lc ? A[q][ADJ ? so : 0][0] : A[q][ADJ ? so : 0][1];
                                *reinterpret_cast<float2*>(acc + gaddr[q] - (2 * S + 2) * plane) =
                                    make_float2(aa, ab);
                            }
                        }
                    }
                }
                // One barrier per two steps.  Shared data written at step t is first
                // read at step t+2 (half-sweep s reads, on plane t+2-2s, the colour
                // half-sweep s-1 wrote there at step t; half-sweep 1 reads the plane
                // published at step t), and a slot's old content was last read at
                // step t-2 (the slot published at step t held plane t-NP, last read
                // by half-sweep S at step t-2).  A barrier after every odd ring slot
                // (NP is even) separates every such pair of steps.
                if (SPLIT) sor_bar_arrive(&sbar[qs & 1]);
                else if (qs & 1) __syncthreads();
            }
        }
    }
    __syncthreads();
    if (SPLIT && threadIdx.x == 0) {  // a persistent block initialises them again for its next tile
        sor_bar_inval(&sbar[0]);
        sor_bar_inval(&sbar[1]);
    }
}

// Quad form of the register-column kernel: each thread owns four x-adjacent
// cells (two of each colour) of its row, so per half-sweep it updates two
// cells whose x neighbours are, but for one, its own registers; the row's
// neighbours above and below arrive as one 8-byte shared-memory load each
// (both colour-c^1 values of the group), the divergence as one, the result
// leaves as one.  Per two updates: five shared-memory instructions instead of
// ten in the pair form.  Same schedule (S half-sweeps in flight at lags 2s,
// one barrier per two ring steps), same update arithmetic, same results.
//
// Shared memory per slot and colour c: float2 per thread, (.x, .y) = the
// group's first and second colour-c cell (x offsets {0,2} when the group's
// first cell has colour c, else {1,3}); the published pressure and the
// divergence, NP slots each.  Incoming planes are 16-byte loads (x0 - S is a
// multiple of 4 because TX and S are, as is the row pitch), flags one 4-byte
// load.
template <int S, int TX, int TY>
struct QuadShape {
    // x0 - S must be a multiple of 4 for the 16-byte plane loads and stores
    static_assert(S % 4 == 0 && TX % 4 == 0, "S and TX multiples of 4");
    static constexpr int RW = TX + 2 * S;  // multiple of 4
    static constexpr int RH = TY + 2 * S;
    static constexpr int GW = RW / 4;      // groups per row
    static constexpr int NT = GW * RH;     // threads per CTA, one group each
    static constexpr int NP = 2 * S + 2;
    // floats ahead of the ring: the row -1 (GW float2) and x -1 reads of slot 0
    static constexpr int GUARD = (2 * GW + 2 + 3) / 4 * 4;
    static constexpr size_t smem = (size_t)NP * 2 * NT * 8 * 2 + (size_t)GUARD * 4;
};

template <int S, int TX, int TY>
__device__ __forceinline__ void sor_quad_tile(const Layout& L, const float* __restrict__ pin,
                                              float* __restrict__ pout, const float* __restrict__ div,
                                              const uint8_t* __restrict__ flags, float omega, float om1, int bx,
                                              int by, int z0, int z1) {
    using Sh = QuadShape<S, TX, TY>;
    constexpr int GW = Sh::GW, NP = Sh::NP, NT = Sh::NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* pub = reinterpret_cast<float2*>(reinterpret_cast<float*>(smem_raw) + Sh::GUARD);  // [NP][2][NT]
    float2* sdv = pub + NP * 2 * NT;                                                           // [NP][2][NT]
    const float* pubf = reinterpret_cast<const float*>(pub);

    const int x0 = bx * TX, y0 = by * TY;
    const int plane = (int)L.plane;
    __shared__ float wtab[8];
    if (threadIdx.x < 8) wtab[threadIdx.x] = threadIdx.x ? omega / (float)threadIdx.x : 0.0f;
    __syncthreads();

    const int e = threadIdx.x;
    const int row = e / GW, gq = e - row * GW;
    const int xl = x0 - S + 4 * gq;  // first cell of the group (multiple of 4)
    const int j = y0 - S + row;
    const int ly = row - S, lxl = 4 * gq - S;
    const bool pin_ok = xl >= 0 && xl < L.W && j >= 0 && j < L.H;
    const bool out_ok = pin_ok && ly >= 0 && ly < TY && lxl >= 0 && lxl < TX;
    int gaddr = pin_ok ? lidx(L, xl, j, z0 - S) : 0;
    // colour of the group's first cell at ring slot qs: bpar ^ (qs & 1) (1 = black)
    const int bpar = (j + z0) & 1;
    // act[par] bit 2(s-1)+k: half-sweep s updates the k-th colour-c cell, par = qs & 1
    unsigned act[2];
#pragma unroll
    for (int par = 0; par < 2; par++) {
        unsigned a = 0;
#pragma unroll
        for (int sw = 1; sw <= S; sw++) {
            const int cs = (sw - 1) & 1;
            const int odd = bpar ^ par ^ cs;  // colour-c cells at offsets {1,3} when set
            const int r = S - sw;
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const int lx = lxl + 2 * k + odd;
                if (lx >= -r && lx < TX + r && ly >= -r && ly < TY + r) a |= 1u << (2 * (sw - 1) + k);
            }
        }
        act[par] = a;
    }
    // x neighbour outside the group: the left group's second colour-c^1 cell
    // when the colour-c cells sit at {0,2}, else the right group's first;
    // xsel[b] for b = (qs & 1) ^ c, as float offsets into the slot's array
    int xsel[2];
    xsel[0] = bpar ? 2 * (e + 1) : 2 * (e - 1) + 1;
    xsel[1] = bpar ? 2 * (e - 1) + 1 : 2 * (e + 1);

    const int tbeg = z0 - S;
    const int nsteps = (z1 - z0) + 3 * S + 1;
    const int flo = max(0, z0 - S), fhi = min(L.D, z1 + S);

    float P[NP][2][2];   // pressure: [slot][colour][k]
    float Wc[NP][2][2];  // omega/cnt: [slot][colour][k] (0: never updated)
#pragma unroll
    for (int a = 0; a < NP; a++)
#pragma unroll
        for (int c = 0; c < 2; c++) P[a][c][0] = P[a][c][1] = Wc[a][c][0] = Wc[a][c][1] = 0.0f;
    float4 np4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), nd4 = np4;
    unsigned nf = 0;
    if (pin_ok && tbeg >= flo && tbeg < fhi) {
        np4 = __ldg(reinterpret_cast<const float4*>(pin + gaddr));
        nd4 = __ldg(reinterpret_cast<const float4*>(div + gaddr));
        nf = __ldg(reinterpret_cast<const unsigned*>(flags + gaddr));
    }

    for (int g = 0; g < nsteps; g += NP) {
#pragma unroll
        for (int qs = 0; qs < NP; qs++) {
            if (g + qs < nsteps) {
                const int t = tbeg + g + qs;
                // 1. plane t into registers by colour, and publish
                {
                    const bool lc = (bpar ^ (qs & 1)) != 0;  // first cell black
                    const float w0 = wtab[(nf >> F_CNT_SHIFT) & 7u];
                    const float w1 = wtab[(nf >> (8 + F_CNT_SHIFT)) & 7u];
                    const float w2 = wtab[(nf >> (16 + F_CNT_SHIFT)) & 7u];
                    const float w3 = wtab[(nf >> (24 + F_CNT_SHIFT)) & 7u];
                    P[qs][0][0] = lc ? np4.y : np4.x;
                    P[qs][0][1] = lc ? np4.w : np4.z;
                    P[qs][1][0] = lc ? np4.x : np4.y;
                    P[qs][1][1] = lc ? np4.z : np4.w;
                    Wc[qs][0][0] = lc ? w1 : w0;
                    Wc[qs][0][1] = lc ? w3 : w2;
                    Wc[qs][1][0] = lc ? w0 : w1;
                    Wc[qs][1][1] = lc ? w2 : w3;
                    pub[(qs * 2 + 0) * NT + e] = make_float2(P[qs][0][0], P[qs][0][1]);
                    pub[(qs * 2 + 1) * NT + e] = make_float2(P[qs][1][0], P[qs][1][1]);
                    sdv[(qs * 2 + 0) * NT + e] = lc ? make_float2(nd4.y, nd4.w) : make_float2(nd4.x, nd4.z);
                    sdv[(qs * 2 + 1) * NT + e] = lc ? make_float2(nd4.x, nd4.z) : make_float2(nd4.y, nd4.w);
                }
                // 2. prefetch plane t+1
                gaddr += plane;
                np4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                nd4 = np4;
                nf = 0;
                if (pin_ok && t + 1 >= flo && t + 1 < fhi) {
                    np4 = __ldg(reinterpret_cast<const float4*>(pin + gaddr));
                    nd4 = __ldg(reinterpret_cast<const float4*>(div + gaddr));
                    nf = __ldg(reinterpret_cast<const unsigned*>(flags + gaddr));
                }
                // 3. half-sweeps (branch-free: inactive cells keep their value)
#pragma unroll
                for (int s = 1; s <= S; s++) {
                    const int z = t - 2 * s;
                    const int r = S - s;
                    if (z >= max(z0 - r, 0) && z < min(z1 + r, L.D)) {
                        const int c = (s - 1) & 1;  // red first
                        const int sz = (qs - 2 * s + 2 * NP) % NP;
                        const int szm = (sz + NP - 1) % NP;
                        const int szp = (sz + 1) % NP;
                        const bool E = ((bpar ^ (qs & 1) ^ c) == 0);  // colour-c cells at offsets {0,2}
                        const float adj = pubf[(sz * 2 + (c ^ 1)) * NT * 2 + xsel[(qs & 1) ^ c]];
                        const float2 ym = pub[(sz * 2 + (c ^ 1)) * NT + e - GW];
                        const float2 yp = pub[(sz * 2 + (c ^ 1)) * NT + e + GW];
                        const float2 dv = sdv[(sz * 2 + c) * NT + e];
                        const float v0 = P[sz][c ^ 1][0], v1 = P[sz][c ^ 1][1];
                        const float t0 = E ? adj : v1, t1 = E ? v0 : adj;
                        const float s0 = ((v0 + t0) + (ym.x + yp.x)) + (P[szm][c ^ 1][0] + P[szp][c ^ 1][0]);
                        const float s1 = ((v1 + t1) + (ym.y + yp.y)) + (P[szm][c ^ 1][1] + P[szp][c ^ 1][1]);
                        const float o0 = P[sz][c][0], o1 = P[sz][c][1];
                        const float w0 = Wc[sz][c][0], w1 = Wc[sz][c][1];
                        const float n0 = sor_update(o0, s0, dv.x, w0, om1);
                        const float n1 = sor_update(o1, s1, dv.y, w1, om1);
                        const unsigned ab = act[qs & 1] >> (2 * (s - 1));
                        const float r0 = ((ab & 1u) && w0 != 0.0f) ? n0 : o0;
                        const float r1 = ((ab & 2u) && w1 != 0.0f) ? n1 : o1;
                        P[sz][c][0] = r0;
                        P[sz][c][1] = r1;
                        pub[(sz * 2 + c) * NT + e] = make_float2(r0, r1);
                    }
                }
                // 4. output plane t-2S-1
                const int zo = t - 2 * S - 1;
                if (zo >= z0 && zo < z1 && out_ok) {
                    const int so = (qs - 2 * S - 1 + 2 * NP) % NP;
                    const bool lc = (bpar ^ (qs & 1) ^ 1) != 0;  // first cell of plane zo black
                    const float4 o = lc ? make_float4(P[so][1][0], P[so][0][0], P[so][1][1], P[so][0][1])
                                        : make_float4(P[so][0][0], P[so][1][0], P[so][0][1], P[so][1][1]);
                    *reinterpret_cast<float4*>(pout + gaddr - (2 * S + 2) * plane) = o;
                }
                // one barrier per two steps, as in sor_reg_tile
                if (qs & 1) __syncthreads();
            }
        }
    }
    __syncthreads();
}

template <int S, int TX, int TY>
__global__ void __launch_bounds__(QuadShape<S, TX, TY>::NT, 1)
    k_sor_quad(Layout L, const float* __restrict__ pin, float* __restrict__ pout, const float* __restrict__ div,
               const uint8_t* __restrict__ flags, float omega, float om1, int zc) {
    const int z0 = blockIdx.z * zc;
    sor_quad_tile<S, TX, TY>(L, pin, pout, div, flags, omega, om1, blockIdx.x, blockIdx.y, z0, min(z0 + zc, L.D));
}

// Persistent batched pass of the quad form (as k_sor_reg_batch).
template <int S, int TX, int TY>
__global__ void __launch_bounds__(QuadShape<S, TX, TY>::NT, 1) k_sor_quad_batch(BatchLaunch B, int pcur, int which) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[i];
        const int local = t - __ldg(B.pre + i);
        const int tx = (d.L.W + TX - 1) / TX, ty = (d.L.H + TY - 1) / TY;
        const int bx = local % tx, r = local / tx;
        const int by = r % ty, bz = r / ty;
        const int z0 = bz * d.zc[which];
        sor_quad_tile<S, TX, TY>(d.L, d.p[pcur], d.p[pcur ^ 1], d.div, d.flags, d.kp.omega, d.kp.om1, bx, by, z0,
                                 min(z0 + d.zc[which], d.L.D));
    }
}

template <int S, int TX, int TY, int PPT, bool WREG>
__global__ void __launch_bounds__(RegShape<S, TX, TY, PPT>::NT)
    k_sor_reg(Layout L, const float* __restrict__ pin, float* __restrict__ pout, const float* __restrict__ div,
              const uint8_t* __restrict__ flags, float omega, float om1, int zc) {
    const int z0 = blockIdx.z * zc;
    sor_reg_tile<S, TX, TY, PPT, false, WREG>(L, pin, pout, div, flags, omega, om1, blockIdx.x, blockIdx.y, z0,
                                              min(z0 + zc, L.D));
}

template <int S, int TX, int TY, int PPT>
__global__ void __launch_bounds__(RegShape<S, TX, TY, PPT>::NT)
    k_sor_reg_split(Layout L, const float* __restrict__ pin, float* __restrict__ pout, const float* __restrict__ div,
                    const uint8_t* __restrict__ flags, float omega, float om1, int zc) {
    const int z0 = blockIdx.z * zc;
    sor_reg_tile<S, TX, TY, PPT, false, true, true>(L, pin, pout, div, flags, omega, om1, blockIdx.x, blockIdx.y, z0,
                                                    min(z0 + zc, L.D));
}

// Persistent batched pass: tile t of the flat SOR tile space belongs to the
// instance found in the prefix array; pressure goes p[pcur] -> p[pcur^1], z
// chunk zc[which].
template <int S, int TX, int TY, int PPT, bool WREG, bool SPLIT = false>
__global__ void __launch_bounds__(RegShape<S, TX, TY, PPT>::NT)
    k_sor_reg_batch(BatchLaunch B, int pcur, int which) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[i];
        const int local = t - __ldg(B.pre + i);
        const int tx = (d.L.W + TX - 1) / TX, ty = (d.L.H + TY - 1) / TY;
        const int bx = local % tx, r = local / tx;
        const int by = r % ty, bz = r / ty;
        const int z0 = bz * d.zc[which];
        sor_reg_tile<S, TX, TY, PPT, false, WREG, SPLIT>(d.L, d.p[pcur], d.p[pcur ^ 1], d.div, d.flags,
                                                         d.kp.omega, d.kp.om1, bx, by, z0,
                                                         min(z0 + d.zc[which], d.L.D));
    }
}

// The reversed SOR of the adjoint (ADJ form of the tile): q ping-pongs, acc in place.
template <int S, int TX, int TY, int PPT, bool SPLIT = false>
__global__ void __launch_bounds__(RegShape<S, TX, TY, PPT>::NT)
    k_sor_reg_adj(Layout L, const float* __restrict__ qin, float* __restrict__ qout, const float* __restrict__ wt,
                  float* __restrict__ acc, float om1, int zc) {
    const int z0 = blockIdx.z * zc;
    sor_reg_tile<S, TX, TY, PPT, true, false, SPLIT>(L, qin, qout, wt, nullptr, 0.0f, om1, blockIdx.x, blockIdx.y,
                                                     z0, min(z0 + zc, L.D), acc);
}

// u -= p_R - p_L on live faces; OPEN also updates domain faces with p = 0 outside.
__device__ __forceinline__ void gradient_tile(const Layout& L, float* __restrict__ u, float* __restrict__ v,
                                              float* __restrict__ w, const float* __restrict__ p,
                                              const uint8_t* __restrict__ flags, int open, int bx, int by, int bz) {
    const int i = bx * 32 + threadIdx.x;
    const int j = by * 8 + threadIdx.y;
    const int k = bz;
    if (i > L.W || j > L.H || k > L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    const uint8_t fl = __ldg(flags + c);
    const float zero = 0.0f;
    if ((fl & F_UFACE) && (open || (i > 0 && i < L.W))) {
        float f = u[c];
        if (i == 0) f = f - (__ldg(p + c) - zero);
        else if (i == L.W) f = f - (zero - __ldg(p + c - 1));
        else f = f - (__ldg(p + c) - __ldg(p + c - 1));
        u[c] = f;
    }
    if ((fl & F_VFACE) && (open || (j > 0 && j < L.H))) {
        float f = v[c];
        if (j == 0) f = f - (__ldg(p + c) - zero);
        else if (j == L.H) f = f - (zero - __ldg(p + c - px));
        else f = f - (__ldg(p + c) - __ldg(p + c - px));
        v[c] = f;
    }
    if ((fl & F_WFACE) && (open || (k > 0 && k < L.D))) {
        float f = w[c];
        if (k == 0) f = f - (__ldg(p + c) - zero);
        else if (k == L.D) f = f - (zero - __ldg(p + c - pl));
        else f = f - (__ldg(p + c) - __ldg(p + c - pl));
        w[c] = f;
    }
}

// FP64 diagnostics per block: max|div u| and sum of squared residuals.
__global__ void k_stats(Layout L, const float* __restrict__ u, const float* __restrict__ v,
                        const float* __restrict__ w, const float* __restrict__ p, const float* __restrict__ div,
                        const uint8_t* __restrict__ flags, double* __restrict__ part) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    double mx = 0.0, r2 = 0.0, nf = 0.0;
    if (i < L.W && j < L.H && k < L.D) {
        const int c = lidx(L, i, j, k);
        const uint8_t f = flags[c];
        if (f & F_FREE) {
            const int px = L.px, pl = (int)L.plane;
            float d = ((((u[c + 1] - u[c]) + v[c + px]) - v[c]) + w[c + pl]) - w[c];
            mx = fabs((double)d);
            double s = 0.0;
            s += (double)p[c - 1];
            s += (double)p[c + 1];
            s += (double)p[c - px];
            s += (double)p[c + px];
            s += (double)p[c - pl];
            s += (double)p[c + pl];
            const int cnt = (f & F_CNT_MASK) >> F_CNT_SHIFT;
            double r = (double)div[c] - (s - (double)cnt * (double)p[c]);
            r2 = r * r;
            nf = 1.0;
        }
    }
    __shared__ double smx[256], sr2[256], snf[256];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    smx[t] = mx;
    sr2[t] = r2;
    snf[t] = nf;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o) {
            smx[t] = fmax(smx[t], smx[t + o]);
            sr2[t] += sr2[t + o];
            snf[t] += snf[t + o];
        }
        __syncthreads();
    }
    if (t == 0) {
        long long b = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
        part[3 * b] = smx[0];
        part[3 * b + 1] = sr2[0];
        part[3 * b + 2] = snf[0];
    }
}

__global__ void k_gradient(Layout L, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w,
                           const float* __restrict__ p, const uint8_t* __restrict__ flags, int open) {
    gradient_tile(L, u, v, w, p, flags, open, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ---- batched forms: one persistent launch over every instance's tiles ----

__device__ __forceinline__ void block_coords(int lt, int wx, int wy, int& bx, int& by, int& bz) {
    const int gx = (wx + 31) / 32, gy = (wy + 7) / 8;
    bx = lt % gx;
    const int r = lt / gx;
    by = r % gy;
    bz = r / gy;
}

// Divergence of every instance into div and p[0] = 0; closed instances write
// their block partials to red in the single-grid block order.
__global__ void k_divergence_batch(BatchLaunch B, int vcur) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[i];
        const int lt = t - __ldg(B.pre + i);
        int bx, by, bz;
        block_coords(lt, d.L.W, d.L.H, bx, by, bz);
        divergence_tile(d.L, d.vel[vcur][0], d.vel[vcur][1], d.vel[vcur][2], d.flags, d.div, d.p[0], d.red,
                        d.closed, bx, by, bz, lt);
    }
}

// One block per instance: the closed-solver mean of its partials (the
// reduction k_reduce_mean performs, same order).
__global__ void k_reduce_mean_batch(const InstDesc* __restrict__ desc, const int* __restrict__ cell_pre) {
    const InstDesc& d = desc[blockIdx.x];
    if (!d.closed || d.kp.mean_override) return;
    const long long nblocks = cell_pre[blockIdx.x + 1] - cell_pre[blockIdx.x];
    const double* part = d.red;
    __shared__ double ss[256], sc[256];
    double s = 0.0, c = 0.0;
    for (long long b = threadIdx.x; b < nblocks; b += 256) {
        s += part[2 * b];
        c += part[2 * b + 1];
    }
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = c;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            ss[threadIdx.x] += ss[threadIdx.x + o];
            sc[threadIdx.x] += sc[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double* out = d.red + d.red_len - 2;
        out[0] = sc[0] > 0.0 ? ss[0] / sc[0] : 0.0;
        out[1] = sc[0];
    }
}

__global__ void k_div_subtract_batch(BatchLaunch B) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int n = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[n];
        if (!d.closed) continue;
        int bx, by, bz;
        block_coords(t - __ldg(B.pre + n), d.L.W, d.L.H, bx, by, bz);
        const int i = bx * 32 + threadIdx.x, j = by * 8 + threadIdx.y, k = bz;
        if (i >= d.L.W || j >= d.L.H || k >= d.L.D) continue;
        const int c = lidx(d.L, i, j, k);
        if (__ldg(d.flags + c) & F_FREE) {
            const float m = d.kp.mean_override ? d.kp.mean_value : (float)d.red[d.red_len - 2];
            d.div[c] = d.div[c] - m;
        }
    }
}

__global__ void k_gradient_batch(BatchLaunch B, int vcur, int pfin) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[i];
        int bx, by, bz;
        block_coords(t - __ldg(B.pre + i), d.L.W + 1, d.L.H + 1, bx, by, bz);
        gradient_tile(d.L, d.vel[vcur][0], d.vel[vcur][1], d.vel[vcur][2], d.p[pfin], d.flags, d.closed ? 0 : 1, bx,
                      by, bz);
    }
}

// ---------------------------------------------------------------- host side

struct RbVariant {
    int S, TX, TY, ppt, nt;
    size_t smem;
    int ctas_per_sm;
    cudaError_t (*launch)(dim3, const Layout&, const float*, float*, const float*, const uint8_t*, float, float, int,
                          cudaStream_t);
    const void* fn;
    // batched persistent form (register-column variants only)
    cudaError_t (*launch_batch)(int, const BatchLaunch&, int, int, cudaStream_t);
    const void* fn_batch;
    int ctas_per_sm_batch;
    // reversed SOR of the adjoint (register-column variants only)
    cudaError_t (*launch_adj)(dim3, const Layout&, const float*, float*, const float*, float*, float, int,
                              cudaStream_t);
    const void* fn_adj;
    int ctas_per_sm_adj;
    int wreg;       // update weights in registers (k_sor_reg WREG form)
    int regs;       // registers per thread of fn
    int xcells = 2; // x-adjacent cells per thread (2: a red-black pair, 4: the quad form)
    int split = 0;  // 1: per-step mbarrier waits (k_sor_reg_split)
};

template <int S, int TX, int TY, int PPT>
cudaError_t rb_launch(dim3 gr, const Layout& L, const float* pin, float* pout, const float* div,
                      const uint8_t* flags, float omega, float om1, int zc, cudaStream_t st) {
    using Sh = RbShape<S, TX, TY, PPT>;
    k_sor_rb<S, TX, TY, PPT><<<gr, Sh::NT, Sh::smem, st>>>(L, pin, pout, div, flags, omega, om1, zc);
    return cudaGetLastError();
}

template <int S, int TX, int TY, int PPT>
RbVariant rb_variant() {
    using Sh = RbShape<S, TX, TY, PPT>;
    RbVariant v;
    v.S = S;
    v.TX = TX;
    v.TY = TY;
    v.ppt = PPT;
    v.nt = Sh::NT;
    v.smem = Sh::smem;
    v.ctas_per_sm = 0;
    v.launch = &rb_launch<S, TX, TY, PPT>;
    v.launch_adj = nullptr;
    v.fn_adj = nullptr;
    v.ctas_per_sm_adj = 0;
    v.launch_batch = nullptr;
    v.fn_batch = nullptr;
    v.ctas_per_sm_batch = 0;
    v.wreg = 0;
    v.regs = 0;
    v.fn = (const void*)k_sor_rb<S, TX, TY, PPT>;
    return v;
}

template <int S, int TX, int TY, int PPT, bool WREG>
cudaError_t reg_launch(dim3 gr, const Layout& L, const float* pin, float* pout, const float* div,
                       const uint8_t* flags, float omega, float om1, int zc, cudaStream_t st) {
    using Sh = RegShape<S, TX, TY, PPT>;
    k_sor_reg<S, TX, TY, PPT, WREG><<<gr, Sh::NT, Sh::smem, st>>>(L, pin, pout, div, flags, omega, om1, zc);
    return cudaGetLastError();
}

template <int S, int TX, int TY, int PPT, bool WREG, bool SPLIT = false>
cudaError_t reg_launch_batch(int blocks, const BatchLaunch& B, int pcur, int which, cudaStream_t st) {
    using Sh = RegShape<S, TX, TY, PPT>;
    k_sor_reg_batch<S, TX, TY, PPT, WREG, SPLIT><<<blocks, Sh::NT, Sh::smem, st>>>(B, pcur, which);
    return cudaGetLastError();
}

template <int S, int TX, int TY, int PPT, bool SPLIT = false>
cudaError_t reg_launch_adj(dim3 gr, const Layout& L, const float* qin, float* qout, const float* wt, float* acc,
                           float om1, int zc, cudaStream_t st) {
    using Sh = RegShape<S, TX, TY, PPT>;
    k_sor_reg_adj<S, TX, TY, PPT, SPLIT><<<gr, Sh::NT, Sh::smem, st>>>(L, qin, qout, wt, acc, om1, zc);
    return cudaGetLastError();
}

template <int S, int TX, int TY, int PPT, bool WREG = false>
RbVariant reg_variant() {
    using Sh = RegShape<S, TX, TY, PPT>;
    RbVariant v;
    v.S = S;
    v.TX = TX;
    v.TY = TY;
    v.ppt = PPT;
    v.nt = Sh::NT;
    v.smem = Sh::smem;
    v.ctas_per_sm = 0;
    v.launch = &reg_launch<S, TX, TY, PPT, WREG>;
    v.fn = (const void*)k_sor_reg<S, TX, TY, PPT, WREG>;
    v.launch_batch = &reg_launch_batch<S, TX, TY, PPT, WREG>;
    v.fn_batch = (const void*)k_sor_reg_batch<S, TX, TY, PPT, WREG>;
    v.wreg = WREG ? 1 : 0;
    v.regs = 0;
    v.ctas_per_sm_batch = 0;
    v.launch_adj = &reg_launch_adj<S, TX, TY, PPT>;
    v.fn_adj = (const void*)k_sor_reg_adj<S, TX, TY, PPT>;
    v.ctas_per_sm_adj = 0;
    return v;
}

template <int S, int TX, int TY, int PPT>
cudaError_t split_launch(dim3 gr, const Layout& L, const float* pin, float* pout, const float* div,
                         const uint8_t* flags, float omega, float om1, int zc, cudaStream_t st) {
    using Sh = RegShape<S, TX, TY, PPT>;
    k_sor_reg_split<S, TX, TY, PPT><<<gr, Sh::NT, Sh::smem, st>>>(L, pin, pout, div, flags, omega, om1, zc);
    return cudaGetLastError();
}

template <int S, int TX, int TY, int PPT>
RbVariant split_variant() {
    RbVariant v = reg_variant<S, TX, TY, PPT, true>();
    v.launch = &split_launch<S, TX, TY, PPT>;
    v.fn = (const void*)k_sor_reg_split<S, TX, TY, PPT>;
    v.launch_batch = &reg_launch_batch<S, TX, TY, PPT, true, true>;
    v.fn_batch = (const void*)k_sor_reg_batch<S, TX, TY, PPT, true, true>;
    v.launch_adj = &reg_launch_adj<S, TX, TY, PPT, true>;
    v.fn_adj = (const void*)k_sor_reg_adj<S, TX, TY, PPT, true>;
    v.split = 1;
    return v;
}

template <int S, int TX, int TY>
cudaError_t quad_launch(dim3 gr, const Layout& L, const float* pin, float* pout, const float* div,
                        const uint8_t* flags, float omega, float om1, int zc, cudaStream_t st) {
    using Sh = QuadShape<S, TX, TY>;
    k_sor_quad<S, TX, TY><<<gr, Sh::NT, Sh::smem, st>>>(L, pin, pout, div, flags, omega, om1, zc);
    return cudaGetLastError();
}

template <int S, int TX, int TY>
cudaError_t quad_launch_batch(int blocks, const BatchLaunch& B, int pcur, int which, cudaStream_t st) {
    using Sh = QuadShape<S, TX, TY>;
    k_sor_quad_batch<S, TX, TY><<<blocks, Sh::NT, Sh::smem, st>>>(B, pcur, which);
    return cudaGetLastError();
}

template <int S, int TX, int TY>
RbVariant quad_variant() {
    using Sh = QuadShape<S, TX, TY>;
    RbVariant v;
    v.S = S;
    v.TX = TX;
    v.TY = TY;
    v.ppt = 2;
    v.nt = Sh::NT;
    v.smem = Sh::smem;
    v.ctas_per_sm = 0;
    v.launch = &quad_launch<S, TX, TY>;
    v.fn = (const void*)k_sor_quad<S, TX, TY>;
    v.launch_batch = &quad_launch_batch<S, TX, TY>;
    v.fn_batch = (const void*)k_sor_quad_batch<S, TX, TY>;
    v.ctas_per_sm_batch = 0;
    v.launch_adj = nullptr;
    v.fn_adj = nullptr;
    v.ctas_per_sm_adj = 0;
    v.wreg = 1;
    v.regs = 0;
    v.xcells = 4;
    return v;
}

// The registry of fused SOR variants (temporal depth S/2, tile, pairs per thread);
// 0-9 keep every plane in shared memory (k_sor_rb), 10-17 keep the thread's own
// column in registers (k_sor_reg), 18-20 also the update weights (WREG), 21-23
// are the quad form (k_sor_quad: four x-adjacent cells per thread), 24 the
// WREG form on 32x30 tiles (nine tile rows cover 256: 144 CTAs of one SM each
// at two z chunks, where 32x32 tiles give 128).
constexpr int kNumVariants = 27;
RbVariant g_var[kNumVariants];
// default variant per depth 1..4
// (measured at 256^3 on GB300: register-column 32x32 at depth 2 with the
// weights in registers is fastest, 51.2 us per iteration; depth 1:
// register-column 64x16 at two CTAs per SM, 61.7 us)
const int kDefaultVariant[5] = {-1, 11, 18, 20, 7};
// batched default: register-column 32x32 at depth 2 with the weights in
// registers (measured on the 64-instance mixed batch: 75.2 ms per step against
// 79.1 ms for 32x16 tiles at two CTAs per SM)
const int kBatchDefaultVariant = 18;
// reversed SOR of the adjoint: register-column variants in order of preference
const int kAdjVariants[] = {13, 12, 11, 10};
int g_num_sms = 0;
// Devices (ordinals < 64) whose kernel attributes are set.  The variant table
// (occupancy, registers) and the SM count come from the first device; another
// device is accepted when it reports the same, i.e. the same GPU model.
std::atomic<unsigned long long> g_prepared_mask{0};
int g_first_device = -1;
std::mutex g_prep_mu;

// z chunk minimising the estimated pass time: waves x (chunk + pipeline fill)
int choose_zc(const Layout& L, const RbVariant& v) {
    const long long tiles = (long long)((L.W + v.TX - 1) / v.TX) * ((L.H + v.TY - 1) / v.TY);
    const long long slots = (long long)std::max(1, g_num_sms) * std::max(1, v.ctas_per_sm);
    int best = L.D;
    double best_cost = 1e300;
    for (int zc = L.D;; zc = (zc + 1) / 2) {
        long long ctas = tiles * ((L.D + zc - 1) / zc);
        long long waves = (ctas + slots - 1) / slots;
        double cost = (double)waves * (zc + 3 * v.S + 1);
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = zc;
        }
        if (zc <= 8) break;
    }
    return best;
}

// One fused pass on the uniform grid of tiles x z chunks (zc_forced 0: the
// chunk from choose_zc).
cudaError_t launch_pass(const RbVariant& v, const Layout& L, const float* pin, float* pout, const float* div,
                        const uint8_t* flags, float omega, float om1, int zc_forced, cudaStream_t s) {
    const int zc = zc_forced > 0 ? std::min(zc_forced, L.D) : choose_zc(L, v);
    dim3 gr((L.W + v.TX - 1) / v.TX, (L.H + v.TY - 1) / v.TY, (L.D + zc - 1) / zc);
    return v.launch(gr, L, pin, pout, div, flags, omega, om1, zc, s);
}

}  // namespace

int sor_prepare() {
    int dev = 0;
    ZQS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("SOR kernels: device ordinals from 64 up are not supported");
        return ZQS_EUNSUPPORTED;
    }
    if ((g_prepared_mask.load(std::memory_order_acquire) >> dev) & 1ull) return ZQS_OK;
    std::lock_guard<std::mutex> lk(g_prep_mu);
    if ((g_prepared_mask.load(std::memory_order_relaxed) >> dev) & 1ull) return ZQS_OK;
    const bool first = g_first_device < 0;
    if (first) {
        g_var[0] = rb_variant<2, 32, 16, 1>();
        g_var[1] = rb_variant<2, 32, 16, 2>();
        g_var[2] = rb_variant<2, 64, 16, 2>();
        g_var[3] = rb_variant<4, 32, 16, 1>();
        g_var[4] = rb_variant<4, 32, 16, 2>();
        g_var[5] = rb_variant<4, 64, 16, 2>();
        g_var[6] = rb_variant<6, 32, 16, 2>();
        g_var[7] = rb_variant<8, 32, 8, 2>();
        g_var[8] = rb_variant<2, 32, 32, 2>();
        g_var[9] = rb_variant<4, 32, 32, 2>();
        g_var[10] = reg_variant<2, 32, 16, 1>();
        g_var[11] = reg_variant<2, 64, 16, 1>();
        g_var[12] = reg_variant<4, 32, 16, 1>();
        g_var[13] = reg_variant<4, 64, 16, 1>();
        g_var[14] = reg_variant<4, 32, 32, 1>();
        g_var[15] = reg_variant<6, 32, 16, 1>();
        g_var[16] = reg_variant<2, 32, 16, 2>();
        g_var[17] = reg_variant<4, 32, 16, 2>();
        g_var[18] = reg_variant<4, 32, 32, 1, true>();
        g_var[19] = reg_variant<4, 64, 16, 1, true>();
        g_var[20] = reg_variant<6, 32, 16, 1, true>();
        g_var[21] = quad_variant<4, 32, 32>();
        g_var[22] = quad_variant<4, 32, 16>();
        g_var[23] = quad_variant<4, 64, 16>();
        g_var[24] = reg_variant<4, 32, 30, 1, true>();
        g_var[25] = split_variant<4, 32, 32, 1>();
        g_var[26] = split_variant<4, 32, 30, 1>();
    }
    int sms = 0;
    ZQS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    bool same = first || sms == g_num_sms;
    // attributes are per device: set them on this one, and compare occupancy
    auto setup = [&](const void* fn, int nt, size_t smem, int& ctas) -> int {
        ZQS_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int n = 0;
        ZQS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, nt, smem));
        if (first) ctas = n;  // 0: does not fit (never selected)
        else if (n != ctas) same = false;
        return ZQS_OK;
    };
    for (int i = 0; i < kNumVariants; i++) {
        RbVariant& v = g_var[i];
        int rc = setup(v.fn, v.nt, v.smem, v.ctas_per_sm);
        if (rc) return rc;
        if (first) {
            cudaFuncAttributes fa;
            ZQS_CUDA_TRY(cudaFuncGetAttributes(&fa, v.fn));
            v.regs = fa.numRegs;
        }
        if (v.fn_batch && (rc = setup(v.fn_batch, v.nt, v.smem, v.ctas_per_sm_batch))) return rc;
        if (v.fn_adj && (rc = setup(v.fn_adj, v.nt, v.smem, v.ctas_per_sm_adj))) return rc;
    }
    if (!same) {
        set_error("SOR kernels: device " + std::to_string(dev) + " differs from device " +
                  std::to_string(g_first_device) +
                  " in SM count or kernel occupancy; one GPU model per process is supported");
        return ZQS_EUNSUPPORTED;
    }
    if (first) {
        g_num_sms = sms;
        g_first_device = dev;
    }
    g_prepared_mask.fetch_or(1ull << dev, std::memory_order_release);
    return ZQS_OK;
}

int sor_variant_count() { return kNumVariants; }

int sor_sync_check() {
    unsigned int n = 0;
    ZQS_CUDA_TRY(cudaMemcpyFromSymbol(&n, g_sor_sync_timeouts, sizeof(n)));
    if (n == 0) return ZQS_OK;
    const unsigned int zero = 0;
    ZQS_CUDA_TRY(cudaMemcpyToSymbol(g_sor_sync_timeouts, &zero, sizeof(zero)));
    set_error("SOR: " + std::to_string(n) + " split-barrier waits gave up; the pressure is not valid");
    return ZQS_ETIMEOUT;
}

int sor_default_variant(int depth) { return kDefaultVariant[depth <= 0 ? 2 : std::min(depth, 4)]; }

int sor_variant_info(int i, zqs_sor_variant* out) {
    if (i < 0 || i >= kNumVariants || !out) {
        set_error("sor variant index out of range");
        return ZQS_EINVAL;
    }
    int rc = sor_prepare();
    if (rc) return rc;
    const RbVariant& v = g_var[i];
    out->depth = v.S / 2;
    out->tile_x = v.TX;
    out->tile_y = v.TY;
    out->pairs_per_thread = v.ppt;
    out->threads = v.nt;
    out->ctas_per_sm = v.ctas_per_sm;
    out->smem_bytes = (int64_t)v.smem;
    out->weights_in_registers = v.wreg;
    out->registers = v.regs;
    out->x_cells_per_thread = v.xcells;
    out->split_barrier = v.split;
    return ZQS_OK;
}

namespace {

std::mutex g_tune_mu;
std::map<std::string, SorChoice> g_tune_mem;

// ZQS_TUNE_CACHE names the file ("" disables it); else
// $XDG_CACHE_HOME/zqs_gb300/sor_tune.txt or $HOME/.cache/zqs_gb300/sor_tune.txt.
std::string tune_cache_path() {
    if (const char* e = std::getenv("ZQS_TUNE_CACHE")) return std::string(e);
    std::string base;
    if (const char* x = std::getenv("XDG_CACHE_HOME"); x && *x) base = x;
    else if (const char* h = std::getenv("HOME"); h && *h) base = std::string(h) + "/.cache";
    return base.empty() ? std::string() : base + "/zqs_gb300/sor_tune.txt";
}

// The cache key: device name and SM count, grid shape and the registry size
// (a registry change invalidates older entries).
std::string tune_key(const Layout& L) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    std::string name = "unknown";
    if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) name = prop.name;
    for (char& c : name)
        if (c == ' ' || c == '|') c = '_';
    std::ostringstream k;
    k << name << "|" << g_num_sms << "|" << L.W << "x" << L.H << "x" << L.D << "|r" << kNumVariants;
    return k.str();
}

bool choice_usable(const SorChoice& c) {
    return c.variant >= 0 && c.variant < kNumVariants && g_var[c.variant].ctas_per_sm >= 1 && c.zchunk >= 0;
}

bool tune_load(const std::string& path, const std::string& key, SorChoice& out) {
    if (path.empty()) return false;
    std::ifstream f(path);
    if (!f) return false;
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {  // the last entry of a key wins
        std::istringstream is(line);
        std::string k;
        SorChoice c;
        if (is >> k >> c.variant >> c.zchunk >> c.us_per_iter && k == key && choice_usable(c)) {
            out = c;
            found = true;
        }
    }
    return found;
}

void tune_store(const std::string& path, const std::string& key, const SorChoice& c) {
    if (path.empty()) return;
    // create the directory chain (best effort: an unwritable cache only costs a re-measure)
    for (size_t pos = path.find('/', 1); pos != std::string::npos; pos = path.find('/', pos + 1))
        mkdir(path.substr(0, pos).c_str(), 0755);
    std::ofstream f(path, std::ios::app);
    if (f) f << key << " " << c.variant << " " << c.zchunk << " " << c.us_per_iter << "\n";
}

}  // namespace

int sor_autotune(const DevGrid& g, const KParams& kp, cudaStream_t s, SorChoice& out) {
    int rc = sor_prepare();
    if (rc) return rc;
    const Layout& L = g.L;
    const std::string key = tune_key(L);
    const std::string path = tune_cache_path();
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_mem.find(key);
        if (it != g_tune_mem.end()) {
            out = it->second;
            out.source = 2;
            return ZQS_OK;
        }
        SorChoice c;
        if (tune_load(path, key, c)) {
            c.source = 3;
            g_tune_mem[key] = c;
            out = c;
            return ZQS_OK;
        }
    }
    cudaEvent_t a = nullptr, b = nullptr;
    ZQS_CUDA_TRY(cudaEventCreate(&a));
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return cuda_fail(cudaErrorUnknown, "sor_autotune: cudaEventCreate");
    }
    constexpr int kReps = 3;
    SorChoice best;
    float best_us = 1e30f;
    cudaError_t err = cudaSuccess;
    for (int vi = 0; vi < kNumVariants && err == cudaSuccess; vi++) {
        const RbVariant& v = g_var[vi];
        if (v.ctas_per_sm < 1) continue;
        std::set<int> zcs = {choose_zc(L, v)};
        for (int n : {1, 2, 3, 4, 6, 8}) zcs.insert(std::max(1, (L.D + n - 1) / n));
        for (int zc : zcs) {
            float* pin = g.p;
            float* pout = g.p2;
            err = launch_pass(v, L, pin, pout, g.div, g.flags, kp.omega, kp.om1, zc, s);  // warm-up
            if (err == cudaSuccess) err = cudaEventRecord(a, s);
            for (int r = 0; r < kReps && err == cudaSuccess; r++) {
                std::swap(pin, pout);
                err = launch_pass(v, L, pin, pout, g.div, g.flags, kp.omega, kp.om1, zc, s);
            }
            if (err == cudaSuccess) err = cudaEventRecord(b, s);
            if (err == cudaSuccess) err = cudaEventSynchronize(b);
            float ms = 0.0f;
            if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, a, b);
            if (err != cudaSuccess) break;
            const float us = 1000.0f * ms / (kReps * (v.S / 2));
            if (us < best_us) {
                best_us = us;
                best.variant = vi;
                best.zchunk = zc;
                best.us_per_iter = us;
            }
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (err != cudaSuccess) return cuda_fail(err, "sor_autotune");
    if (!choice_usable(best)) {
        set_error("sor_autotune: no fused SOR variant fits this device");
        return ZQS_EUNSUPPORTED;
    }
    best.source = 1;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_mem[key] = best;
        tune_store(path, key, best);
    }
    out = best;
    return ZQS_OK;
}

int launch_project(DevGrid& g, const KParams& kp, int K, const SorConfig& cfg, cudaStream_t s, LaunchCounter& lc,
                   float** p_final) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    if (kp.solver == ZQS_SOLVER_COARSE_OPEN) {
        // no fine pressure or right-hand side: both read back as zero
        ZQS_CUDA_TRY(cudaMemsetAsync(g.p - L.plane, 0, (size_t)L.elems * sizeof(float), s));
        ZQS_CUDA_TRY(cudaMemsetAsync(g.div - L.plane, 0, (size_t)L.elems * sizeof(float), s));
        int rc = launch_project_coarse(g, kp, K, s, lc);
        if (p_final) *p_final = g.p;
        return rc;
    }
    dim3 gc((L.W + 31) / 32, (L.H + 7) / 8, L.D);
    const bool closed = kp.solver == ZQS_SOLVER_CLOSED;
    k_divergence<<<gc, b, 0, s>>>(L, g.u, g.v, g.w, g.flags, g.div, g.p, g.red, closed ? 1 : 0);
    lc.n++;
    if (closed) {
        long long nblocks = (long long)gc.x * gc.y * gc.z;
        double* mean = g.red + g.red_len - 2;  // kept apart from the stats partials
        if (kp.mean_override) {
            k_div_subtract_const<<<gc, b, 0, s>>>(L, g.flags, g.div, kp.mean_value);
            lc.n++;
        } else {
            k_reduce_mean<<<1, 256, 0, s>>>(g.red, nblocks, mean);
            k_div_subtract_mean<<<gc, b, 0, s>>>(L, g.flags, g.div, mean);
            lc.n += 2;
        }
    }
    ZQS_LAUNCH_CHECK("divergence");
    float* cur = g.p;
    float* nxt = g.p2;
    if (cfg.split) {
        for (int it = 0; it < K; it++) {
            k_sor_colour<<<gc, b, 0, s>>>(L, cur, g.div, g.flags, 0, kp.omega, kp.om1);
            k_sor_colour<<<gc, b, 0, s>>>(L, cur, g.div, g.flags, 1, kp.omega, kp.om1);
            lc.n += 2;
        }
        ZQS_LAUNCH_CHECK("k_sor_colour");
    } else {
        int rc = sor_prepare();
        if (rc) return rc;
        const int depth = cfg.temporal_depth > 0 ? cfg.temporal_depth : 2;
        int vmain = cfg.variant >= 0 ? cfg.variant : kDefaultVariant[std::min(depth, 4)];
        if (vmain >= kNumVariants || g_var[vmain].ctas_per_sm < 1) {
            set_error("SOR variant does not fit this device");
            return ZQS_EUNSUPPORTED;
        }
        const int dmain = g_var[vmain].S / 2;
        int remaining = K;
        while (remaining > 0) {
            const int d = std::min(dmain, remaining);
            const RbVariant& v = (d == dmain) ? g_var[vmain] : g_var[kDefaultVariant[d]];
            cudaError_t e =
                launch_pass(v, L, cur, nxt, g.div, g.flags, kp.omega, kp.om1, d == dmain ? cfg.zchunk : 0, s);
            if (e != cudaSuccess) return cuda_fail(e, "k_sor_rb");
            lc.n++;
            std::swap(cur, nxt);
            remaining -= d;
        }
    }
    dim3 gf((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, L.D + 1);
    k_gradient<<<gf, b, 0, s>>>(L, g.u, g.v, g.w, cur, g.flags, closed ? 0 : 1);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_gradient");
    if (p_final) *p_final = cur;
    return ZQS_OK;
}

bool sor_variant_batchable(int variant) {
    if (sor_prepare() != ZQS_OK) return false;
    return variant >= 0 && variant < kNumVariants && g_var[variant].launch_batch &&
           g_var[variant].ctas_per_sm_batch > 0;
}

int sor_batch_plan(int variant, SorBatchPlan& out) {
    int rc = sor_prepare();
    if (rc) return rc;
    const int vm = variant >= 0 ? variant : kBatchDefaultVariant;
    if (!sor_variant_batchable(vm)) {
        set_error("SOR variant " + std::to_string(vm) + " has no batched form on this device");
        return ZQS_EUNSUPPORTED;
    }
    // remainder: the depth-1 register-column variant with the same tile, else the first depth-1 one
    int vr = -1;
    for (int i = 0; i < kNumVariants && vr < 0; i++)
        if (sor_variant_batchable(i) && g_var[i].S == 2 && g_var[i].TX == g_var[vm].TX &&
            g_var[i].TY == g_var[vm].TY && g_var[i].ppt == g_var[vm].ppt)
            vr = i;
    for (int i = 0; i < kNumVariants && vr < 0; i++)
        if (sor_variant_batchable(i) && g_var[i].S == 2) vr = i;
    if (vr < 0) {
        set_error("no depth-1 batched SOR variant fits this device");
        return ZQS_EUNSUPPORTED;
    }
    out.vmain = vm;
    out.vrem = vr;
    const int v2[2] = {vm, vr};
    for (int q = 0; q < 2; q++) {
        out.S[q] = g_var[v2[q]].S;
        out.TX[q] = g_var[v2[q]].TX;
        out.TY[q] = g_var[v2[q]].TY;
        out.slots[q] = g_num_sms * g_var[v2[q]].ctas_per_sm_batch;
    }
    return ZQS_OK;
}

int launch_project_batch(const BatchLaunch& cell, const BatchLaunch& face, const BatchLaunch& sorm,
                         const BatchLaunch& sorr, const SorBatchPlan& plan, int K, bool any_closed, int vcur,
                         int blocks, cudaStream_t s, LaunchCounter& lc, int* pfin) {
    dim3 b(32, 8, 1);
    k_divergence_batch<<<persistent_blocks((const void*)k_divergence_batch, 256, 0, std::min(blocks, cell.total)), b, 0,
                         s>>>(cell, vcur);
    lc.n++;
    if (any_closed) {
        k_reduce_mean_batch<<<cell.n, 256, 0, s>>>(cell.desc, cell.pre);
        k_div_subtract_batch<<<persistent_blocks((const void*)k_div_subtract_batch, 256, 0, std::min(blocks, cell.total)), b, 0,
                               s>>>(cell);
        lc.n += 2;
    }
    ZQS_LAUNCH_CHECK("batched divergence");
    int pcur = 0;
    const int dmain = plan.S[0] / 2;
    int remaining = K;
    while (remaining > 0) {
        const int which = remaining >= dmain ? 0 : 1;
        const RbVariant& v = g_var[which == 0 ? plan.vmain : plan.vrem];
        const BatchLaunch& B = which == 0 ? sorm : sorr;
        const int d = which == 0 ? dmain : 1;
        cudaError_t e = v.launch_batch(std::min(plan.slots[which], B.total), B, pcur, which, s);
        if (e != cudaSuccess) return cuda_fail(e, "k_sor_reg_batch");
        lc.n++;
        pcur ^= 1;
        remaining -= d;
    }
    k_gradient_batch<<<persistent_blocks((const void*)k_gradient_batch, 256, 0, std::min(blocks, face.total)), b, 0,
                       s>>>(face, vcur, pcur);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_gradient_batch");
    if (pfin) *pfin = pcur;
    return ZQS_OK;
}

cudaError_t launch_sor_batch_pass(const SorBatchPlan& plan, int which, const BatchLaunch& B, int pcur,
                                  cudaStream_t s) {
    const RbVariant& v = g_var[which == 0 ? plan.vmain : plan.vrem];
    return v.launch_batch(std::min(plan.slots[which], B.total), B, pcur, which, s);
}

namespace {
std::map<std::string, int> g_adj_tuned;  // (device, shape) -> variant of the reversed SOR's main pass (g_tune_mu)

cudaError_t adj_pass(const RbVariant& v, const Layout& L, const float* qin, float* qout, const float* wt, float* acc,
                     float om1, cudaStream_t s) {
    RbVariant occ = v;
    occ.ctas_per_sm = v.ctas_per_sm_adj;
    const int zc = choose_zc(L, occ);
    dim3 gr((L.W + v.TX - 1) / v.TX, (L.H + v.TY - 1) / v.TY, (L.D + zc - 1) / zc);
    return v.launch_adj(gr, L, qin, qout, wt, acc, om1, zc, s);
}
}  // namespace

int sor_adj_autotune(const Layout& L, float* q, float* q2, const float* wt, float* acc, float om1, cudaStream_t s) {
    int rc = sor_prepare();
    if (rc) return rc;
    const char* env = std::getenv("ZQS_AUTOTUNE");
    if (env && env[0] == '0') return ZQS_OK;
    const std::string key = tune_key(L);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (g_adj_tuned.count(key)) return ZQS_OK;
    }
    cudaEvent_t a = nullptr, b = nullptr;
    ZQS_CUDA_TRY(cudaEventCreate(&a));
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return cuda_fail(cudaErrorUnknown, "sor_adj_autotune: cudaEventCreate");
    }
    int best = -1;
    float best_us = 1e30f;
    cudaError_t err = cudaSuccess;
    for (int vi = 0; vi < kNumVariants && err == cudaSuccess; vi++) {
        const RbVariant& v = g_var[vi];
        if (!v.launch_adj || v.ctas_per_sm_adj < 1 || v.S != 4) continue;
        err = adj_pass(v, L, q, q2, wt, acc, om1, s);  // warm-up
        if (err == cudaSuccess) err = cudaEventRecord(a, s);
        for (int r = 0; r < 3 && err == cudaSuccess; r++)
            err = adj_pass(v, L, (r & 1) ? q2 : q, (r & 1) ? q : q2, wt, acc, om1, s);
        if (err == cudaSuccess) err = cudaEventRecord(b, s);
        if (err == cudaSuccess) err = cudaEventSynchronize(b);
        float ms = 0.0f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, a, b);
        if (err == cudaSuccess && ms < best_us) {
            best_us = ms;
            best = vi;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (err != cudaSuccess) return cuda_fail(err, "sor_adj_autotune");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (best >= 0) g_adj_tuned[key] = best;
    return ZQS_OK;
}

int launch_sor_adjoint_pairs(const Layout& L, float* q, float* q2, const float* wt, float* acc, float om1,
                             int npairs, cudaStream_t s, LaunchCounter& lc, float** qcur) {
    int rc = sor_prepare();
    if (rc) return rc;
    auto fits = [](int i) { return g_var[i].launch_adj && g_var[i].ctas_per_sm_adj > 0; };
    int vmain = -1, vrem = -1;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_adj_tuned.find(tune_key(L));
        if (it != g_adj_tuned.end() && fits(it->second)) vmain = it->second;
    }
    for (int i : kAdjVariants)
        if (vmain < 0 && fits(i) && g_var[i].S == 4) vmain = i;
    for (int i : kAdjVariants)
        if (vrem < 0 && fits(i) && g_var[i].S == 2) vrem = i;
    if (vrem < 0) {
        set_error("reversed SOR: no fused variant fits this device");
        return ZQS_EUNSUPPORTED;
    }
    if (vmain < 0) vmain = vrem;
    float* cur = q;
    float* nxt = q2;
    int remaining = npairs;
    while (remaining > 0) {
        const int dmain = g_var[vmain].S / 2;
        const RbVariant& v = remaining >= dmain ? g_var[vmain] : g_var[vrem];
        const int d = v.S / 2;
        cudaError_t e = adj_pass(v, L, cur, nxt, wt, acc, om1, s);
        if (e != cudaSuccess) return cuda_fail(e, "k_sor_reg_adj");
        lc.n++;
        std::swap(cur, nxt);
        remaining -= d;
    }
    *qcur = cur;
    return ZQS_OK;
}

int launch_stats(const DevGrid& g, const KParams& kp, const float* p, zqs_stats* out, cudaStream_t s) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    dim3 gc((L.W + 31) / 32, (L.H + 7) / 8, L.D);
    long long nblocks = (long long)gc.x * gc.y * gc.z;
    if (3 * nblocks + 2 > g.red_len) {
        set_error("stats: reduction scratch too small");
        return ZQS_EINVAL;
    }
    k_stats<<<gc, b, 0, s>>>(L, g.u, g.v, g.w, p, g.div, g.flags, g.red);
    ZQS_LAUNCH_CHECK("k_stats");
    std::vector<double> h(3 * nblocks);
    ZQS_CUDA_TRY(cudaMemcpyAsync(h.data(), g.red, sizeof(double) * 3 * nblocks, cudaMemcpyDeviceToHost, s));
    ZQS_CUDA_TRY(cudaStreamSynchronize(s));
    double mx = 0.0, r2 = 0.0, nf = 0.0;
    for (long long bb = 0; bb < nblocks; bb++) {
        mx = std::max(mx, h[3 * bb]);
        r2 += h[3 * bb + 1];
        nf += h[3 * bb + 2];
    }
    out->max_abs_div = mx;
    out->residual_l2 = std::sqrt(r2);
    out->free_cells = (int64_t)nf;
    (void)kp;
    return ZQS_OK;
}

}  // namespace zqs
