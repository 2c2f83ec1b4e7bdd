// Reverse mode of the smoke step (no counterpart in the reference: the
// differentiable path is new).  Each kernel is the transpose of a forward
// stage of kernels_force.cu / kernels_advect.cu / kernels_sor.cu, restated
// from the same rules as the FP64 oracle's adjoint (oracle/zqs_oracle.cpp,
// step_adjoint); stage order and buffers are listed in zqs_adjoint.h.
//
// Gather where the transpose has a fixed stencil (G^T, div^T, the face
// averaging, the curl and gradient stencils: no atomics), scatter with FP32
// atomicAdd where it does not (the transposed trilinear samples of the
// backtraces: 16-byte atomics into quad accumulators for the velocity, folded
// onto the faces afterwards by k_adj_fold; scalar atomics for the final
// scalar samples).  Discrete decisions of the forward (backtrace breaks, clamps,
// floor cells, a zero-length confinement normal) are held fixed.
#include <algorithm>

#include "zqs_adjoint.h"
#include "zqs_sample.cuh"

namespace zqs {

namespace {

// ---------------------------------------------------------------- helpers

// Gradient of the trilinear sample with respect to the texel coordinates;
// clamped axes have equal corners and so a zero derivative.
__device__ __forceinline__ void tri_grad(const float* __restrict__ f, const Corners& c, float g[3]) {
    const float c000 = __ldg(f + c.r00 + c.i0), c100 = __ldg(f + c.r00 + c.i1);
    const float c010 = __ldg(f + c.r10 + c.i0), c110 = __ldg(f + c.r10 + c.i1);
    const float c001 = __ldg(f + c.r01 + c.i0), c101 = __ldg(f + c.r01 + c.i1);
    const float c011 = __ldg(f + c.r11 + c.i0), c111 = __ldg(f + c.r11 + c.i1);
    const float c00 = lerpf(c000, c100, c.tx), c10 = lerpf(c010, c110, c.tx);
    const float c01 = lerpf(c001, c101, c.tx), c11 = lerpf(c011, c111, c.tx);
    const float c0 = lerpf(c00, c10, c.ty), c1 = lerpf(c01, c11, c.ty);
    g[0] = lerpf(lerpf(c100 - c000, c110 - c010, c.ty), lerpf(c101 - c001, c111 - c011, c.ty), c.tz);
    g[1] = lerpf(c10 - c00, c11 - c01, c.tz);
    g[2] = c1 - c0;
}

// Transposed trilinear sample: val times each corner weight, added atomically.
__device__ __forceinline__ void tri_scatter(float* __restrict__ f, const Corners& c, float val) {
    if (val == 0.0f) return;
    const float x0 = 1.0f - c.tx, x1 = c.tx, y0 = 1.0f - c.ty, y1 = c.ty, z0 = 1.0f - c.tz, z1 = c.tz;
    atomicAdd(f + c.r00 + c.i0, ((x0 * y0) * z0) * val);
    atomicAdd(f + c.r00 + c.i1, ((x1 * y0) * z0) * val);
    atomicAdd(f + c.r10 + c.i0, ((x0 * y1) * z0) * val);
    atomicAdd(f + c.r10 + c.i1, ((x1 * y1) * z0) * val);
    atomicAdd(f + c.r01 + c.i0, ((x0 * y0) * z1) * val);
    atomicAdd(f + c.r01 + c.i1, ((x1 * y0) * z1) * val);
    atomicAdd(f + c.r11 + c.i0, ((x0 * y1) * z1) * val);
    atomicAdd(f + c.r11 + c.i1, ((x1 * y1) * z1) * val);
}

// Base corner of a trilinear sample in the quad layout (tri0 in
// zqs_sample.cuh), plus the axes the clamp-to-edge rule pinned to the last
// texel (i0 == n-1).  There the clamped sample is flat along that axis (both
// corners are the same texel), so its derivative is 0; the quad form's
// unclamped +1 corner enters the value with weight t = 0 only, but would give
// a one-sided difference, which tri_grad_q replaces by that 0.
struct QC {
    int r;
    float tx, ty, tz;
    bool hx, hy, hz;
};
__device__ __forceinline__ QC qcorner(const Layout& L, int nx, int ny, int nz, float gx, float gy, float gz) {
    const Ax ax = axis(gx, nx), ay = axis(gy, ny), az = axis(gz, nz);
    QC c;
    c.r = (az.i0 * L.py + ay.i0) * L.px + ax.i0;
    c.tx = ax.t;
    c.ty = ay.t;
    c.tz = az.t;
    c.hx = ax.i0 == nx - 1;
    c.hy = ay.i0 == ny - 1;
    c.hz = az.i0 == nz - 1;
    return c;
}
__device__ __forceinline__ QC qcorner_u(const Layout& L, float x, float y, float z) {
    return qcorner(L, L.W + 1, L.H, L.D, x, y - 0.5f, z - 0.5f);
}
__device__ __forceinline__ QC qcorner_v(const Layout& L, float x, float y, float z) {
    return qcorner(L, L.W, L.H + 1, L.D, x - 0.5f, y, z - 0.5f);
}
__device__ __forceinline__ QC qcorner_w(const Layout& L, float x, float y, float z) {
    return qcorner(L, L.W, L.H, L.D + 1, x - 0.5f, y - 0.5f, z);
}

// tri_grad from the quad copy Q of the field: the eight corners are the two
// 16-byte loads Q[r] = (c000, c001, c100, c101) and Q[r + px] = (c010, c011,
// c110, c111); same expressions, and 0 along clamped axes.
__device__ __forceinline__ void tri_grad_q(const float4* __restrict__ Q, const Layout& L, const QC& c, float g[3]) {
    const float4 a = __ldg(Q + c.r);
    const float4 b = __ldg(Q + c.r + L.px);
    const float c000 = a.x, c001 = a.y, c100 = a.z, c101 = a.w;
    const float c010 = b.x, c011 = b.y, c110 = b.z, c111 = b.w;
    const float c00 = lerpf(c000, c100, c.tx), c10 = lerpf(c010, c110, c.tx);
    const float c01 = lerpf(c001, c101, c.tx), c11 = lerpf(c011, c111, c.tx);
    const float c0 = lerpf(c00, c10, c.ty), c1 = lerpf(c01, c11, c.ty);
    g[0] = c.hx ? 0.0f : lerpf(lerpf(c100 - c000, c110 - c010, c.ty), lerpf(c101 - c001, c111 - c011, c.ty), c.tz);
    g[1] = c.hy ? 0.0f : lerpf(c10 - c00, c11 - c01, c.tz);
    g[2] = c.hz ? 0.0f : c1 - c0;
}

// tri_scatter into a quad accumulator: the same eight products, as two
// 16-byte atomics (vector atomicAdd, compute capability 9.0 and up).  A
// clamped axis has t = 0, so its +1 corners receive exact zeros.
__device__ __forceinline__ void tri_scatter_q(float4* __restrict__ G, const Layout& L, const QC& c, float val) {
    if (val == 0.0f) return;
    const float x0 = 1.0f - c.tx, x1 = c.tx, y0 = 1.0f - c.ty, y1 = c.ty, z0 = 1.0f - c.tz, z1 = c.tz;
    atomicAdd(G + c.r, make_float4(((x0 * y0) * z0) * val, ((x0 * y0) * z1) * val, ((x1 * y0) * z0) * val,
                                   ((x1 * y0) * z1) * val));
    atomicAdd(G + c.r + L.px, make_float4(((x0 * y1) * z0) * val, ((x0 * y1) * z1) * val,
                                          ((x1 * y1) * z0) * val, ((x1 * y1) * z1) * val));
}

__device__ __forceinline__ Corners corners_c(const Layout& L, float x, float y, float z) {
    return corners(L, L.W, L.H, L.D, x - 0.5f, y - 0.5f, z - 0.5f);
}

__device__ __forceinline__ bool bt_ok(const Layout& L, const uint8_t* __restrict__ flags, float x, float y,
                                      float z) {
    if (!(x >= 0.0f && x <= (float)L.W && y >= 0.0f && y <= (float)L.H && z >= 0.0f && z <= (float)L.D))
        return false;
    const int i = min(max((int)floorf(x), 0), L.W - 1);
    const int j = min(max((int)floorf(y), 0), L.H - 1);
    const int k = min(max((int)floorf(z), 0), L.D - 1);
    return (__ldg(flags + lidx(L, i, j, k)) & F_FREE) != 0;
}

// The forward backtrace (zqs_sample.cuh) with every position kept in xs;
// returns m, the index of the point the forward samples at.  VelF is the
// forward's sampler (MacVelQC: the quad copies with the last quads kept in
// registers, bit-identical to the fields).
template <class VelF>
__device__ __forceinline__ int backtrace_record(const Layout& L, const uint8_t* __restrict__ flags, VelF& vel,
                                                const KParams& kp, float px, float py, float pz, float* xs) {
    float vx, vy, vz;
    vel(px, py, pz, vx, vy, vz);
    xs[0] = px;
    xs[1] = py;
    xs[2] = pz;
    const float dt = kp.dt_sub;
    int m = 0, istep = 0;
    bool broke = false;
    do {
        if (!bt_ok(L, flags, px, py, pz)) {
            broke = true;
            break;
        }
        m = istep;
        if (kp.inv_h != 0.0f) {
            px = px - (vx * dt) * kp.inv_h;
            py = py - (vy * dt) * kp.inv_h;
            pz = pz - (vz * dt) * kp.inv_h;
        } else {
            px = px - (vx * dt) / kp.h;
            py = py - (vy * dt) / kp.h;
            pz = pz - (vz * dt) / kp.h;
        }
        istep++;
        xs[3 * istep + 0] = px;
        xs[3 * istep + 1] = py;
        xs[3 * istep + 2] = pz;
        if (istep < kp.substeps) vel(px, py, pz, vx, vy, vz);
    } while (istep < kp.substeps);
    if (kp.full && !broke && bt_ok(L, flags, px, py, pz)) m = istep;
    return m;
}

// Reverse of x_{s+1} = x_s - c*vel(x_s) for s = m-1 .. 0: the velocity
// adjoint -c*gx is scattered at x_s into the quad accumulators gq and
// gx += J_vel(x_s)^T (-c*gx), with J from the quad copies q.
__device__ __forceinline__ void backtrace_adjoint(const Layout& L, const float4* const (&q)[3],
                                                  float4* const (&gq)[3], const float* xs, int m, float c,
                                                  float gx[3]) {
    for (int s = m - 1; s >= 0; s--) {
        const float x = xs[3 * s], y = xs[3 * s + 1], z = xs[3 * s + 2];
        const float g0 = -c * gx[0], g1 = -c * gx[1], g2 = -c * gx[2];
        const QC cu = qcorner_u(L, x, y, z), cv = qcorner_v(L, x, y, z), cw = qcorner_w(L, x, y, z);
        tri_scatter_q(gq[0], L, cu, g0);
        tri_scatter_q(gq[1], L, cv, g1);
        tri_scatter_q(gq[2], L, cw, g2);
        float J0[3], J1[3], J2[3];
        tri_grad_q(q[0], L, cu, J0);
        tri_grad_q(q[1], L, cv, J1);
        tri_grad_q(q[2], L, cw, J2);
        gx[0] += (J0[0] * g0 + J1[0] * g1) + J2[0] * g2;
        gx[1] += (J0[1] * g0 + J1[1] * g1) + J2[1] * g2;
        gx[2] += (J0[2] * g0 + J1[2] * g1) + J2[2] * g2;
    }
}

__device__ __forceinline__ float chain_c(const KParams& kp) {
    return kp.inv_h != 0.0f ? kp.dt_sub * kp.inv_h : kp.dt_sub / kp.h;
}

__device__ __forceinline__ bool in_source(const SourceList& src, int i, int j, int k) {
    for (int s = 0; s < src.n; s++) {
        const zqs_source& S = src.s[s];
        const float dx = ((float)i + 0.5f) - S.cx;
        const float dy = ((float)j + 0.5f) - S.cy;
        const float dz = ((float)k + 0.5f) - S.cz;
        bool in;
        if (S.shape == ZQS_SOURCE_SPHERE) in = ((dx * dx + dy * dy) + dz * dz) <= S.hx * S.hx;
        else in = fabsf(dx) <= S.hx && fabsf(dy) <= S.hy && fabsf(dz) <= S.hz;
        if (in) return true;
    }
    return false;
}

// ---------------------------------------------------------------- scalar advection

// Per cell: reinjection (sources overwrite: zero adjoint), then the transposed
// sample of the attenuated scalars and the backtrace chain through u4.
__global__ void __launch_bounds__(256) k_adj_scalar(Layout L, AdjFwd f, AdjBufs b, KParams kp, SourceList src) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    if (src.n > 0 && in_source(src, i, j, k)) return;
    const float gT = b.gT[c], gD = b.grho[c];
    if (gT == 0.0f && gD == 0.0f) return;
    float xs[3 * (kAdjMaxSubsteps + 1)];
    MacVelQC<> mv(L, f.q4[0], f.q4[1], f.q4[2]);
    const int m = backtrace_record(L, f.flags, mv, kp, (float)i + 0.5f, (float)j + 0.5f, (float)k + 0.5f, xs);
    const float x = xs[3 * m], y = xs[3 * m + 1], z = xs[3 * m + 2];
    const Corners cc = corners_c(L, x, y, z);
    const float aT = kp.temp_atten * gT, aD = kp.dens_atten * gD;
    tri_scatter(b.gTa, cc, aT);
    tri_scatter(b.grhoa, cc, aD);
    float g1[3], g2[3];
    tri_grad(f.T0, cc, g1);
    tri_grad(f.rho0, cc, g2);
    float gx[3] = {aT * g1[0] + aD * g2[0], aT * g1[1] + aD * g2[1], aT * g1[2] + aD * g2[2]};
    backtrace_adjoint(L, f.q4, b.gq, xs, m, chain_c(kp), gx);
}

// ---------------------------------------------------------------- projection

__global__ void k_adj_weights(Layout L, const uint8_t* __restrict__ flags, float omega, float* __restrict__ wt) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    const uint8_t fl = __ldg(flags + c);
    const int cnt = (fl & F_CNT_MASK) >> F_CNT_SHIFT;
    wt[c] = ((fl & F_FREE) && cnt > 0) ? omega / (float)cnt : 0.0f;
}

// Face g of the gradient subtraction's live rule (open: domain faces of free
// cells too; closed: interior faces only).
__device__ __forceinline__ float live_g(const float* __restrict__ g, const uint8_t* __restrict__ flags, int f,
                                        uint8_t bit, int along, int n, int open) {
    return face_live(__ldg(flags + f), bit, along, n, open != 0) ? g[f] : 0.0f;
}

// q = (omega/cnt) * G^T g, where u_f -= p_hi - p_lo gives gp_c = sum over the
// cell's axes of (g_hiface - g_loface).
__global__ void k_adj_gradT(Layout L, const uint8_t* __restrict__ flags, AdjBufs b, int open) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    float gp = live_g(b.gu, flags, c + 1, F_UFACE, i + 1, L.W, open) - live_g(b.gu, flags, c, F_UFACE, i, L.W, open);
    gp += live_g(b.gv, flags, c + px, F_VFACE, j + 1, L.H, open) - live_g(b.gv, flags, c, F_VFACE, j, L.H, open);
    gp += live_g(b.gw, flags, c + pl, F_WFACE, k + 1, L.D, open) - live_g(b.gw, flags, c, F_WFACE, k, L.D, open);
    b.q[c] = __ldg(b.wt + c) * gp;
    b.acc[c] = 0.0f;
}

// One in-place sweep of the reversed SOR over colour `colour` in the scaled
// variable q = (omega/cnt) gp:
//   mode 0 (head)  q += wt * sum(q_n)
//   mode 1         acc += q;  q = (1-omega) q + wt * sum(q_n)
//   mode 2 (tail)  acc += q
// Cells of the other colour are only read, so the sweep is race-free.
__global__ void k_adj_sor_sweep(Layout L, float* __restrict__ q, const float* __restrict__ wt,
                                float* __restrict__ acc, int colour, int mode, float om1) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    if (((i + j + k) & 1) != colour) return;
    const int c = lidx(L, i, j, k);
    const float wc = __ldg(wt + c);
    if (wc == 0.0f) return;
    const float qc = q[c];
    if (mode == 2) {
        acc[c] += qc;
        return;
    }
    const int px = L.px, pl = (int)L.plane;
    const float s = ((((q[c - 1] + q[c + 1]) + q[c - px]) + q[c + px]) + q[c - pl]) + q[c + pl];
    if (mode == 0) {
        q[c] = qc + wc * s;
    } else {
        acc[c] += qc;
        q[c] = om1 * qc + wc * s;
    }
}

// Closed solver: FP64 partial sums of acc over free cells per 32x8 block.
__global__ void k_adj_acc_partials(Layout L, const uint8_t* __restrict__ flags, const float* __restrict__ acc,
                                   double* __restrict__ part) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    double s = 0.0, n = 0.0;
    if (i < L.W && j < L.H && k < L.D) {
        const int c = lidx(L, i, j, k);
        if (__ldg(flags + c) & F_FREE) {
            s = (double)acc[c];
            n = 1.0;
        }
    }
    __shared__ double ss[256], sn[256];
    const int t = threadIdx.y * 32 + threadIdx.x;
    ss[t] = s;
    sn[t] = n;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o) {
            ss[t] += ss[t + o];
            sn[t] += sn[t + o];
        }
        __syncthreads();
    }
    if (t == 0) {
        const long long blk = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
        part[2 * blk] = ss[0];
        part[2 * blk + 1] = sn[0];
    }
}

__global__ void k_adj_acc_mean(const double* __restrict__ part, long long nblocks, double* __restrict__ out) {
    __shared__ double ss[256], sn[256];
    double s = 0.0, n = 0.0;
    for (long long bb = threadIdx.x; bb < nblocks; bb += 256) {
        s += part[2 * bb];
        n += part[2 * bb + 1];
    }
    ss[threadIdx.x] = s;
    sn[threadIdx.x] = n;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            ss[threadIdx.x] += ss[threadIdx.x + o];
            sn[threadIdx.x] += sn[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = sn[0] > 0.0 ? ss[0] / sn[0] : 0.0;
}

__global__ void k_adj_acc_subtract(Layout L, const uint8_t* __restrict__ flags, float* __restrict__ acc,
                                   const double* __restrict__ mean) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    if (__ldg(flags + c) & F_FREE) acc[c] = acc[c] - (float)mean[0];
}

// gu3 = gu + div^T(gdiv) with gdiv = -acc: the face between cells lo and hi
// gets acc_hi - acc_lo.  gu2 is seeded with gu3 on faces the velocity
// advection does not write (open rule) and 0 elsewhere.
__global__ void k_adj_divT(Layout L, const uint8_t* __restrict__ flags, AdjBufs b) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i > L.W || j > L.H || k > L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    const uint8_t fl = __ldg(flags + c);
    const float* acc = b.acc;
    const float a = (i < L.W && j < L.H && k < L.D) ? acc[c] : 0.0f;
    if (j < L.H && k < L.D) {
        const float lo = i > 0 ? acc[c - 1] : 0.0f;
        const float g = b.gu[c] + (a - lo);
        b.gu3[c] = g;
        b.gu2[c] = (fl & F_UFACE) ? 0.0f : g;
    }
    if (i < L.W && k < L.D) {
        const float lo = j > 0 ? acc[c - px] : 0.0f;
        const float g = b.gv[c] + (a - lo);
        b.gv3[c] = g;
        b.gv2[c] = (fl & F_VFACE) ? 0.0f : g;
    }
    if (i < L.W && j < L.H) {
        const float lo = k > 0 ? acc[c - pl] : 0.0f;
        const float g = b.gw[c] + (a - lo);
        b.gw3[c] = g;
        b.gw2[c] = (fl & F_WFACE) ? 0.0f : g;
    }
}

// ---------------------------------------------------------------- velocity advection

// Per live face (bz = 3k + comp, the three components of a plane adjacent in
// the launch order as in the forward): transposed final sample of the input
// component and the backtrace chain, all into the quad accumulators gq.
__global__ void __launch_bounds__(256) k_adj_advect_vel(Layout L, AdjFwd f, AdjBufs b, KParams kp) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z / 3;
    const int comp = blockIdx.z - 3 * k;
    int nx = L.W, ny = L.H, nz = L.D;
    if (comp == 0) nx++;
    else if (comp == 1) ny++;
    else nz++;
    if (i >= nx || j >= ny || k >= nz) return;
    const int c = lidx(L, i, j, k);
    const uint8_t bit = comp == 0 ? F_UFACE : (comp == 1 ? F_VFACE : F_WFACE);
    if (!(__ldg(f.flags + c) & bit)) return;
    const float g = comp == 0 ? b.gu3[c] : (comp == 1 ? b.gv3[c] : b.gw3[c]);
    if (g == 0.0f) return;
    const float px0 = (comp == 0) ? (float)i : (float)i + 0.5f;
    const float py0 = (comp == 1) ? (float)j : (float)j + 0.5f;
    const float pz0 = (comp == 2) ? (float)k : (float)k + 0.5f;
    float xs[3 * (kAdjMaxSubsteps + 1)];
    MacVelQC<> mv(L, f.q2[0], f.q2[1], f.q2[2]);
    const int m = backtrace_record(L, f.flags, mv, kp, px0, py0, pz0, xs);
    const float x = xs[3 * m], y = xs[3 * m + 1], z = xs[3 * m + 2];
    float gx[3];
    const QC cc = comp == 0 ? qcorner_u(L, x, y, z) : (comp == 1 ? qcorner_v(L, x, y, z) : qcorner_w(L, x, y, z));
    // (selects, not a dynamic index into the parameter arrays)
    tri_scatter_q(comp == 0 ? b.gq[0] : (comp == 1 ? b.gq[1] : b.gq[2]), L, cc, g);
    tri_grad_q(comp == 0 ? f.q2[0] : (comp == 1 ? f.q2[1] : f.q2[2]), L, cc, gx);
    gx[0] *= g;
    gx[1] *= g;
    gx[2] *= g;
    backtrace_adjoint(L, f.q2, b.gq, xs, m, chain_c(kp), gx);
}

// g += the quad accumulators folded back onto their texels (bz = 3k + comp,
// every face index): texel t collects gq[t].x + gq[t - plane].y + gq[t - 1].z
// + gq[t - plane - 1].w.  Padding entries only ever receive exact zeros.
__global__ void __launch_bounds__(256) k_adj_fold(Layout L, AdjBufs b, float* __restrict__ gu,
                                                  float* __restrict__ gv, float* __restrict__ gw) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z / 3;
    const int comp = blockIdx.z - 3 * k;
    int nx = L.W, ny = L.H, nz = L.D;
    if (comp == 0) nx++;
    else if (comp == 1) ny++;
    else nz++;
    if (i >= nx || j >= ny || k >= nz) return;
    const int c = lidx(L, i, j, k);
    const int pl = (int)L.plane;
    const float4* G = comp == 0 ? b.gq[0] : (comp == 1 ? b.gq[1] : b.gq[2]);
    const float s = (G[c].x + G[c - pl].y) + (G[c - 1].z + G[c - pl - 1].w);
    float* dst = comp == 0 ? gu : (comp == 1 ? gv : gw);
    if (s != 0.0f) dst[c] += s;
}

// ---------------------------------------------------------------- forces

// Adjoint of the face update + attenuation of one face, as seen by the cell
// force: weight * vel_atten * gu2 on live faces (dt on domain faces, dt/2
// inside), 0 elsewhere.
__device__ __forceinline__ float face_force_g(const float* __restrict__ g2, const uint8_t* __restrict__ flags,
                                              int f, uint8_t bit, int along, int n, const KParams& kp) {
    if (!(__ldg(flags + f) & bit)) return 0.0f;
    const float wgt = (along == 0 || along == n) ? kp.dt : kp.dt * 0.5f;
    return wgt * (kp.vel_atten * g2[f]);
}

// Per cell: gf (transposed face averaging), the control and buoyancy adjoints,
// and the confinement force f = cc (N x w) transposed to gN, gw; then
// N = g/|g| transposed to gg.
__global__ void k_adj_force_cell(Layout L, AdjFwd f, AdjBufs b, KParams kp) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    const float fx = face_force_g(b.gu2, f.flags, c, F_UFACE, i, L.W, kp) +
                     face_force_g(b.gu2, f.flags, c + 1, F_UFACE, i + 1, L.W, kp);
    const float fy = face_force_g(b.gv2, f.flags, c, F_VFACE, j, L.H, kp) +
                     face_force_g(b.gv2, f.flags, c + px, F_VFACE, j + 1, L.H, kp);
    const float fz = face_force_g(b.gw2, f.flags, c, F_WFACE, k, L.D, kp) +
                     face_force_g(b.gw2, f.flags, c + pl, F_WFACE, k + 1, L.D, kp);
    const long long E = L.elems;
    b.gF[c] += fx;
    b.gF[E + c] += fy;
    b.gF[2 * E + c] += fz;
    b.gT[c] = b.gTa[c] + kp.beta * fy;
    b.grho[c] = b.grhoa[c] - kp.alpha * fy;
    // normal of this cell, as the forward force_cell computes it
    auto S = [&](int o) -> float { return __ldg(&f.vort[o].w); };
    float gx, gy, gz;
    if (i == 0) gx = S(c + 1) - S(c);
    else if (i == L.W - 1) gx = S(c) - S(c - 1);
    else gx = 0.5f * (S(c + 1) - S(c - 1));
    if (j == 0) gy = S(c + px) - S(c);
    else if (j == L.H - 1) gy = S(c) - S(c - px);
    else gy = 0.5f * (S(c + px) - S(c - px));
    if (k == 0) gz = S(c + pl) - S(c);
    else if (k == L.D - 1) gz = S(c) - S(c - pl);
    else gz = 0.5f * (S(c + pl) - S(c - pl));
    const float len = sqrtf((gx * gx + gy * gy) + gz * gz);
    float Nx = gx, Ny = gy, Nz = gz;
    if (len != 0.0f) {
        Nx = gx / len;
        Ny = gy / len;
        Nz = gz / len;
    }
    const float4 o = __ldg(&f.vort[c]);
    const float cc = kp.cc;
    const float gNx = cc * (o.y * fz - o.z * fy), gNy = cc * (o.z * fx - o.x * fz), gNz = cc * (o.x * fy - o.y * fx);
    b.gom4[c] = make_float4(cc * (Nz * fy - Ny * fz), cc * (Nx * fz - Nz * fx), cc * (Ny * fx - Nx * fy), 0.0f);
    float4 gg = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (len != 0.0f) {
        const float dot = (Nx * gNx + Ny * gNy) + Nz * gNz;
        gg.x = (gNx - Nx * dot) / len;
        gg.y = (gNy - Ny * dot) / len;
        gg.z = (gNz - Nz * dot) / len;
    }
    b.gg4[c] = gg;
}

// Transposed |w|-gradient stencil along one axis at index a of n cells: the
// adjoint of |w| at this cell from gg of itself and its two neighbours.
__device__ __forceinline__ float grad_T(float g_self, float g_lo, float g_hi, int a, int n) {
    float s = 0.0f;
    if (a == 0) s -= g_self;
    if (a == n - 1) s += g_self;
    if (a - 1 >= 0) s += (a - 1 == 0) ? g_lo : 0.5f * g_lo;
    if (a + 1 <= n - 1) s -= (a + 1 == n - 1) ? g_hi : 0.5f * g_hi;
    return s;
}

// Per cell: g|w| from the gradient stencil, then gw_total = gw + (w/|w|) g|w|
// on interior cells (the vorticity is a constant 0 elsewhere), divided by 2h.
__global__ void k_adj_vs(Layout L, AdjFwd f, AdjBufs b, float twoh) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    float4 r = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (i >= 1 && i <= L.W - 2 && j >= 1 && j <= L.H - 2 && k >= 1 && k <= L.D - 2) {
        const float gvs = (grad_T(b.gg4[c].x, b.gg4[c - 1].x, b.gg4[c + 1].x, i, L.W) +
                           grad_T(b.gg4[c].y, b.gg4[c - px].y, b.gg4[c + px].y, j, L.H)) +
                          grad_T(b.gg4[c].z, b.gg4[c - pl].z, b.gg4[c + pl].z, k, L.D);
        const float4 o = __ldg(&f.vort[c]);
        float4 go = b.gom4[c];
        if (o.w != 0.0f) {
            go.x += o.x / o.w * gvs;
            go.y += o.y / o.w * gvs;
            go.z += o.z / o.w * gvs;
        }
        r = make_float4(go.x / twoh, go.y / twoh, go.z / twoh, 0.0f);
    }
    b.gw4[c] = r;
}

// Per cell: adjoint of the cell-centre velocity from the curl stencil
// (gw4 is zero outside the interior and in the padding).
__global__ void k_adj_centre(Layout L, AdjBufs b) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    const float4* g = b.gw4;
    const float gU = ((g[c - pl].y - g[c + pl].y) - g[c - px].z) + g[c + px].z;
    const float gV = ((g[c + pl].x - g[c - pl].x) + g[c - 1].z) - g[c + 1].z;
    const float gW = ((g[c - px].x - g[c + px].x) - g[c - 1].y) + g[c + 1].y;
    b.gom4[c] = make_float4(gU, gV, gW, 0.0f);
}

// Per face: gu = gu1 + 0.5 * (gcentre_lo + gcentre_hi), gu1 = vel_atten * gu2
// on live faces (the face update is the identity in the velocity).
__global__ void k_adj_faces(Layout L, const uint8_t* __restrict__ flags, AdjBufs b, float vel_atten) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i > L.W || j > L.H || k > L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    const uint8_t fl = __ldg(flags + c);
    const float4* gc = b.gom4;
    if (j < L.H && k < L.D) {
        const float g1 = (fl & F_UFACE) ? vel_atten * b.gu2[c] : b.gu2[c];
        const float lo = i > 0 ? gc[c - 1].x : 0.0f, hi = i < L.W ? gc[c].x : 0.0f;
        b.gu[c] = g1 + (0.5f * lo + 0.5f * hi);
    }
    if (i < L.W && k < L.D) {
        const float g1 = (fl & F_VFACE) ? vel_atten * b.gv2[c] : b.gv2[c];
        const float lo = j > 0 ? gc[c - px].y : 0.0f, hi = j < L.H ? gc[c].y : 0.0f;
        b.gv[c] = g1 + (0.5f * lo + 0.5f * hi);
    }
    if (i < L.W && j < L.H) {
        const float g1 = (fl & F_WFACE) ? vel_atten * b.gw2[c] : b.gw2[c];
        const float lo = k > 0 ? gc[c - pl].z : 0.0f, hi = k < L.D ? gc[c].z : 0.0f;
        b.gw[c] = g1 + (0.5f * lo + 0.5f * hi);
    }
}

}  // namespace

// ---------------------------------------------------------------- host side

int launch_adj_weights(const Layout& L, const uint8_t* flags, float omega, float* wt, cudaStream_t s,
                       LaunchCounter& lc) {
    dim3 b(32, 8, 1), gc((L.W + 31) / 32, (L.H + 7) / 8, L.D);
    k_adj_weights<<<gc, b, 0, s>>>(L, flags, omega, wt);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_adj_weights");
    return ZQS_OK;
}

int launch_adj_step(const Layout& L, const AdjFwd& f, const AdjBufs& b, const KParams& kp, const SourceList& src,
                    int K, cudaStream_t s, LaunchCounter& lc) {
    if (kp.substeps > kAdjMaxSubsteps) {
        set_error("adjoint: at most 32 backtrace substeps are supported");
        return ZQS_EUNSUPPORTED;
    }
    dim3 blk(32, 8, 1);
    dim3 gc((L.W + 31) / 32, (L.H + 7) / 8, L.D);
    dim3 gf((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, L.D + 1);
    dim3 ga((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, 3 * (L.D + 1));
    dim3 gq3((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, 3 * (L.D + 1));
    const size_t cell_bytes = (size_t)L.elems * 4;
    // the three quad accumulators are contiguous, each with a float4 before
    // its leading guard plane and one spare after it
    const size_t gq_bytes = 3 * (size_t)(L.elems + 2) * 16;
    float4* gq_base = b.gq[0] - L.plane - 1;
    // scalar advection + reinjection
    ZQS_CUDA_TRY(cudaMemsetAsync(b.gTa - L.plane, 0, cell_bytes, s));
    ZQS_CUDA_TRY(cudaMemsetAsync(b.grhoa - L.plane, 0, cell_bytes, s));
    ZQS_CUDA_TRY(cudaMemsetAsync(gq_base, 0, gq_bytes, s));
    k_adj_scalar<<<gc, blk, 0, s>>>(L, f, b, kp, src);
    k_adj_fold<<<gq3, blk, 0, s>>>(L, b, b.gu, b.gv, b.gw);
    lc.n += 2;
    ZQS_LAUNCH_CHECK("k_adj_scalar");
    // projection: G^T, reversed SOR, div^T
    const int open = kp.solver == ZQS_SOLVER_OPEN ? 1 : 0;
    k_adj_gradT<<<gc, blk, 0, s>>>(L, f.flags, b, open);
    lc.n++;
    if (K > 0) {
        // forward order per iteration: red (0) then black (1); reversed: the
        // head red gather, K-1 black/red pairs (fused, temporally blocked),
        // the last black sweep, then the red tail
        k_adj_sor_sweep<<<gc, blk, 0, s>>>(L, b.q, b.wt, b.acc, 0, 0, kp.om1);
        lc.n++;
        float* qc = b.q;
        if (K > 1) {
            int rc = launch_sor_adjoint_pairs(L, b.q, b.q2, b.wt, b.acc, kp.om1, K - 1, s, lc, &qc);
            if (rc) return rc;
        }
        k_adj_sor_sweep<<<gc, blk, 0, s>>>(L, qc, b.wt, b.acc, 1, 1, kp.om1);
        k_adj_sor_sweep<<<gc, blk, 0, s>>>(L, qc, b.wt, b.acc, 0, 2, kp.om1);
        lc.n += 2;
    }
    ZQS_LAUNCH_CHECK("k_adj_sor_sweep");
    if (!open && !kp.mean_override) {
        const long long nblocks = (long long)gc.x * gc.y * gc.z;
        if (2 * nblocks + 1 > b.red_len) {
            set_error("adjoint: reduction scratch too small");
            return ZQS_EINVAL;
        }
        double* mean = b.red + 2 * nblocks;
        k_adj_acc_partials<<<gc, blk, 0, s>>>(L, f.flags, b.acc, b.red);
        k_adj_acc_mean<<<1, 256, 0, s>>>(b.red, nblocks, mean);
        k_adj_acc_subtract<<<gc, blk, 0, s>>>(L, f.flags, b.acc, mean);
        lc.n += 3;
        ZQS_LAUNCH_CHECK("adjoint closed mean");
    }
    k_adj_divT<<<gf, blk, 0, s>>>(L, f.flags, b);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_adj_divT");
    // velocity advection
    ZQS_CUDA_TRY(cudaMemsetAsync(gq_base, 0, gq_bytes, s));
    k_adj_advect_vel<<<ga, blk, 0, s>>>(L, f, b, kp);
    k_adj_fold<<<gq3, blk, 0, s>>>(L, b, b.gu2, b.gv2, b.gw2);
    lc.n += 2;
    ZQS_LAUNCH_CHECK("k_adj_advect_vel");
    // forces (+ attenuation)
    k_adj_force_cell<<<gc, blk, 0, s>>>(L, f, b, kp);
    k_adj_vs<<<gc, blk, 0, s>>>(L, f, b, kp.twoh);
    k_adj_centre<<<gc, blk, 0, s>>>(L, b);
    k_adj_faces<<<gf, blk, 0, s>>>(L, f.flags, b, kp.vel_atten);
    lc.n += 4;
    ZQS_LAUNCH_CHECK("adjoint force kernels");
    return ZQS_OK;
}

}  // namespace zqs
