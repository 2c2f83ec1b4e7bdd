// Semi-Lagrangian advection of velocity and scalars (gather form).
//
// Restates the backtrace kernels of ZQ_CUDA_Advection3D.cu (MAC in/out
// :232-377, regular in / MAC out :115-230, regular in/out :76-113, scalars
// :379-469) and the open/closed write-back (:471-650).  The reference samples
// 3D textures with hardware linear filtering (9-bit weights, clamp addressing,
// :654-993); here every sample is an exact FP32 trilinear interpolation over
// the padded arrays, read through the read-only data path, with the same
// clamp-to-edge rule and the same expression order as the oracle.
//
// Per-step fusions: the write-back mask is applied in the epilogue (no
// separate Apply_* launches), and the scalar pass folds in the temperature /
// density attenuation factors (multiplying each interpolation corner, which is
// what attenuating the field first computes) and the source reinjection of
// ZQ_ReinjectTemperatureDensity3D (ZQ_SmokeSimulationUtils3D.cpp:3842-3882).
#include <algorithm>

#include "zqs_batch.h"
#include "zqs_sample.cuh"

namespace zqs {

namespace {

// Quad copies (zqs_sample.cuh, tri0_quad) of the three face components, one
// thread per face index (i <= W, j <= H, k <= D): q[c][r] = (f[r],
// f[r + plane], f[r + 1], f[r + plane + 1]).
__device__ __forceinline__ void mac_quads_tile(const Layout& L, const float* __restrict__ u,
                                               const float* __restrict__ v, const float* __restrict__ w,
                                               float4* __restrict__ qu, float4* __restrict__ qv,
                                               float4* __restrict__ qw, int bx, int by, int bz) {
    const int i = bx * 32 + threadIdx.x;
    const int j = by * 8 + threadIdx.y;
    const int k = bz;
    if (i > L.W || j > L.H || k > L.D) return;
    const int c = lidx(L, i, j, k);
    const int pl = (int)L.plane;
    qu[c] = make_float4(__ldg(u + c), __ldg(u + c + pl), __ldg(u + c + 1), __ldg(u + c + pl + 1));
    qv[c] = make_float4(__ldg(v + c), __ldg(v + c + pl), __ldg(v + c + 1), __ldg(v + c + pl + 1));
    qw[c] = make_float4(__ldg(w + c), __ldg(w + c + pl), __ldg(w + c + 1), __ldg(w + c + pl + 1));
}

__global__ void __launch_bounds__(256) k_mac_quads(Layout L, const float* __restrict__ u,
                                                   const float* __restrict__ v, const float* __restrict__ w,
                                                   float4* __restrict__ qu, float4* __restrict__ qv,
                                                   float4* __restrict__ qw) {
    mac_quads_tile(L, u, v, w, qu, qv, qw, blockIdx.x, blockIdx.y, blockIdx.z);
}

// One thread per face: bz = comp*(D+1) + k, comp 0/1/2 = u/v/w.
// REGIN selects the regular (cell-centre float4) velocity for both the
// backtrace and the final sample (inRegular_outMAC), else MAC (inMAC_outMAC),
// whose samples read the quad copies q (built from u, v, w).
template <bool REGIN>
__device__ __forceinline__ void advect_vel_macout_tile(const Layout& L, const float* __restrict__ u,
                                                       const float* __restrict__ v, const float* __restrict__ w,
                                                       const float4* __restrict__ vel4, const float4* const* q,
                                                       const uint8_t* __restrict__ flags, float* __restrict__ u2,
                                                       float* __restrict__ v2, float* __restrict__ w2,
                                                       const KParams& kp, int open, int bx, int by, int bz) {
    const int i = bx * 32 + threadIdx.x;
    const int j = by * 8 + threadIdx.y;
    const int comp = bz / (L.D + 1);
    const int k = bz - comp * (L.D + 1);
    int nx = L.W, ny = L.H, nz = L.D;
    if (comp == 0) nx++;
    else if (comp == 1) ny++;
    else nz++;
    if (i >= nx || j >= ny || k >= nz) return;
    const int c = lidx(L, i, j, k);
    const uint8_t fl = __ldg(flags + c);
    const float* src = comp == 0 ? u : (comp == 1 ? v : w);
    float* dst = comp == 0 ? u2 : (comp == 1 ? v2 : w2);
    const uint8_t bit = comp == 0 ? F_UFACE : (comp == 1 ? F_VFACE : F_WFACE);
    const int along = comp == 0 ? i : (comp == 1 ? j : k);
    const int n = comp == 0 ? L.W : (comp == 1 ? L.H : L.D);
    float out = __ldg(src + c);
    if (face_live(fl, bit, along, n, open != 0)) {
        float px = (comp == 0) ? (float)i : (float)i + 0.5f;
        float py = (comp == 1) ? (float)j : (float)j + 0.5f;
        float pz = (comp == 2) ? (float)k : (float)k + 0.5f;
        if (REGIN) {
            RegVel rv{L, vel4};
            backtrace(L, flags, rv, kp, px, py, pz);
            out = tri4c(vel4, comp, corners(L, L.W, L.H, L.D, px - 0.5f, py - 0.5f, pz - 0.5f));
        } else {
            const MacVelQ mv{L, {q[0]}, {q[1]}, {q[2]}};
            backtrace(L, flags, mv, kp, px, py, pz);
            if (comp == 0) out = tri0_quad(q[0], L, tri0(L, L.W + 1, L.H, L.D, px, py - 0.5f, pz - 0.5f));
            else if (comp == 1) out = tri0_quad(q[1], L, tri0(L, L.W, L.H + 1, L.D, px - 0.5f, py, pz - 0.5f));
            else out = tri0_quad(q[2], L, tri0(L, L.W, L.H, L.D + 1, px - 0.5f, py - 0.5f, pz));
        }
    }
    dst[c] = out;
}

struct Quads {
    const float4* q[3];
};

template <bool REGIN>
__global__ void __launch_bounds__(256) k_advect_vel_macout(Layout L, const float* __restrict__ u,
                                                           const float* __restrict__ v, const float* __restrict__ w,
                                                           const float4* __restrict__ vel4, Quads Q,
                                                           const uint8_t* __restrict__ flags, float* __restrict__ u2,
                                                           float* __restrict__ v2, float* __restrict__ w2, KParams kp,
                                                           int open) {
    advect_vel_macout_tile<REGIN>(L, u, v, w, vel4, Q.q, flags, u2, v2, w2, kp, open, blockIdx.x, blockIdx.y,
                                  blockIdx.z);
}

// Advect_Velocity_inRegular_outRegular_Kernel (Adv3D:76-113): per cell.
__global__ void __launch_bounds__(256) k_advect_vel_regreg(Layout L, const float4* __restrict__ vel4,
                                                           const uint8_t* __restrict__ flags,
                                                           float4* __restrict__ out4, KParams kp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    float px = (float)i + 0.5f, py = (float)j + 0.5f, pz = (float)k + 0.5f;
    RegVel rv{L, vel4};
    backtrace(L, flags, rv, kp, px, py, pz);
    float3 r = tri4(vel4, corners(L, L.W, L.H, L.D, px - 0.5f, py - 0.5f, pz - 0.5f));
    out4[lidx(L, i, j, k)] = make_float4(r.x, r.y, r.z, 0.0f);
}

// Regular4_to_MAC (ZQ_CUDA_MACtoRegular.cu:29-99) fused with the write-back.
__global__ void k_reg4_to_mac_apply(Layout L, const float4* __restrict__ c4, const uint8_t* __restrict__ flags,
                                    const float* __restrict__ u, const float* __restrict__ v,
                                    const float* __restrict__ w, float* __restrict__ u2, float* __restrict__ v2,
                                    float* __restrict__ w2, int open) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > L.W || j > L.H || k > L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    const uint8_t fl = __ldg(flags + c);
    if (j < L.H && k < L.D) {
        float o = __ldg(u + c);
        if (face_live(fl, F_UFACE, i, L.W, open != 0)) {
            if (i == 0) o = __ldg(&c4[c].x);
            else if (i == L.W) o = __ldg(&c4[c - 1].x);
            else o = 0.5f * (__ldg(&c4[c].x) + __ldg(&c4[c - 1].x));
        }
        u2[c] = o;
    }
    if (i < L.W && k < L.D) {
        float o = __ldg(v + c);
        if (face_live(fl, F_VFACE, j, L.H, open != 0)) {
            if (j == 0) o = __ldg(&c4[c].y);
            else if (j == L.H) o = __ldg(&c4[c - px].y);
            else o = 0.5f * (__ldg(&c4[c].y) + __ldg(&c4[c - px].y));
        }
        v2[c] = o;
    }
    if (i < L.W && j < L.H) {
        float o = __ldg(w + c);
        if (face_live(fl, F_WFACE, k, L.D, open != 0)) {
            if (k == 0) o = __ldg(&c4[c].z);
            else if (k == L.D) o = __ldg(&c4[c - pl].z);
            else o = 0.5f * (__ldg(&c4[c].z) + __ldg(&c4[c - pl].z));
        }
        w2[c] = o;
    }
}

__device__ __forceinline__ void reinject_cell(const SourceList& src, int i, int j, int k, float& T, float& rho) {
    for (int s = 0; s < src.n; s++) {
        const zqs_source& S = src.s[s];
        float dx = ((float)i + 0.5f) - S.cx;
        float dy = ((float)j + 0.5f) - S.cy;
        float dz = ((float)k + 0.5f) - S.cz;
        bool in;
        if (S.shape == ZQS_SOURCE_SPHERE) in = ((dx * dx + dy * dy) + dz * dz) <= S.hx * S.hx;
        else in = fabsf(dx) <= S.hx && fabsf(dy) <= S.hy && fabsf(dz) <= S.hz;
        if (in) {
            rho = S.density;
            T = S.temperature;
        }
    }
}

// Advect_Scalar_{MAC,Regular}_Velocity_Kernel (Adv3D:379-469) with the
// attenuation factors applied to the interpolation corners and the sources
// reinjected in the epilogue.
template <bool REGIN>
__device__ __forceinline__ void advect_scalar_tile(const Layout& L, const float4* __restrict__ vel4,
                                                   const float4* const* q, const uint8_t* __restrict__ flags,
                                                   const float* __restrict__ T, const float* __restrict__ rho,
                                                   float* __restrict__ T2, float* __restrict__ rho2,
                                                   const KParams& kp, float aT, float aD, const SourceList& src,
                                                   int bx, int by, int bz) {
    const int i = bx * 32 + threadIdx.x;
    const int j = by * 8 + threadIdx.y;
    const int k = bz;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    float px = (float)i + 0.5f, py = (float)j + 0.5f, pz = (float)k + 0.5f;
    if (REGIN) {
        RegVel rv{L, vel4};
        backtrace(L, flags, rv, kp, px, py, pz);
    } else {
        const MacVelQ mv{L, {q[0]}, {q[1]}, {q[2]}};
        backtrace(L, flags, mv, kp, px, py, pz);
    }
    const Tri0 cs = tri0(L, L.W, L.H, L.D, px - 0.5f, py - 0.5f, pz - 0.5f);
    float t = tri0_sample(T, L, cs, aT);
    float d = tri0_sample(rho, L, cs, aD);
    if (src.n > 0) reinject_cell(src, i, j, k, t, d);
    const int c = lidx(L, i, j, k);
    T2[c] = t;
    rho2[c] = d;
}

template <bool REGIN>
__global__ void __launch_bounds__(256) k_advect_scalar(Layout L, const float4* __restrict__ vel4, Quads Q,
                                                       const uint8_t* __restrict__ flags,
                                                       const float* __restrict__ T, const float* __restrict__ rho,
                                                       float* __restrict__ T2, float* __restrict__ rho2, KParams kp,
                                                       float aT, float aD, SourceList src) {
    advect_scalar_tile<REGIN>(L, vel4, Q.q, flags, T, rho, T2, rho2, kp, aT, aD, src, blockIdx.x, blockIdx.y,
                              blockIdx.z);
}

// ---- batched forms (MAC velocity) ----

// Quad copies of velocity buffer vcur, over the FACE tile class.
__global__ void __launch_bounds__(256) k_mac_quads_batch(BatchLaunch B, int vcur) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[i];
        const int lt = t - __ldg(B.pre + i);
        const int gx = (d.L.W + 1 + 31) / 32, gy = (d.L.H + 1 + 7) / 8;
        const int bx = lt % gx, r = lt / gx, by = r % gy, bz = r / gy;
        mac_quads_tile(d.L, d.vel[vcur][0], d.vel[vcur][1], d.vel[vcur][2], d.q4[0], d.q4[1], d.q4[2], bx, by, bz);
    }
}

__global__ void __launch_bounds__(256) k_advect_vel_batch(BatchLaunch B, int vcur) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[i];
        const int lt = t - __ldg(B.pre + i);
        const int gx = (d.L.W + 1 + 31) / 32, gy = (d.L.H + 1 + 7) / 8;
        const int bx = lt % gx, r = lt / gx, by = r % gy, bz = r / gy;
        const KParams kp = d.kp;
        const int nxt = vcur ^ 1;
        const float4* q[3] = {d.q4[0], d.q4[1], d.q4[2]};
        advect_vel_macout_tile<false>(d.L, d.vel[vcur][0], d.vel[vcur][1], d.vel[vcur][2], d.t4a, q, d.flags,
                                      d.vel[nxt][0], d.vel[nxt][1], d.vel[nxt][2], kp, 1, bx, by, bz);
    }
}

__global__ void __launch_bounds__(256) k_advect_scalar_batch(BatchLaunch B, int vcur, int scur) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[i];
        const int lt = t - __ldg(B.pre + i);
        const int gx = (d.L.W + 31) / 32, gy = (d.L.H + 7) / 8;
        const int bx = lt % gx, r = lt / gx, by = r % gy, bz = r / gy;
        const KParams kp = d.kp;
        const int nxt = scur ^ 1;
        const float4* q[3] = {d.q4[0], d.q4[1], d.q4[2]};
        advect_scalar_tile<false>(d.L, d.t4a, q, d.flags, d.sca[scur][0], d.sca[scur][1], d.sca[nxt][0],
                                  d.sca[nxt][1], kp, kp.temp_atten, kp.dens_atten, d.src, bx, by, bz);
    }
}

__global__ void k_reinject(Layout L, float* __restrict__ T, float* __restrict__ rho, SourceList src) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    float t = T[c], d = rho[c];
    reinject_cell(src, i, j, k, t, d);
    T[c] = t;
    rho[c] = d;
}

}  // namespace

int launch_mac_quads(const DevGrid& g, cudaStream_t s, LaunchCounter& lc) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    dim3 gf((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, L.D + 1);
    k_mac_quads<<<gf, b, 0, s>>>(L, g.u, g.v, g.w, g.qu, g.qv, g.qw);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_mac_quads");
    return ZQS_OK;
}

int launch_advect_velocity(DevGrid& g, const KParams& kp, int mode, bool open, cudaStream_t s, LaunchCounter& lc) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    if (mode == ZQS_ADV_VEL_INMAC_OUTMAC || mode == ZQS_ADV_VEL_INREG_OUTMAC) {
        int nxb = (L.W + 1 + 31) / 32, nyb = (L.H + 1 + 7) / 8;
        dim3 gr(nxb, nyb, 3 * (L.D + 1));
        const Quads Q{{g.qu, g.qv, g.qw}};
        if (mode == ZQS_ADV_VEL_INREG_OUTMAC) {
            int rc = launch_mac_to_reg4(g, g.u, g.v, g.w, g.t4a, s, lc);
            if (rc) return rc;
            k_advect_vel_macout<true><<<gr, b, 0, s>>>(L, g.u, g.v, g.w, g.t4a, Q, g.flags, g.u2, g.v2, g.w2, kp,
                                                       open);
        } else {
            int rc = launch_mac_quads(g, s, lc);
            if (rc) return rc;
            k_advect_vel_macout<false><<<gr, b, 0, s>>>(L, g.u, g.v, g.w, g.t4a, Q, g.flags, g.u2, g.v2, g.w2, kp,
                                                        open);
        }
        lc.n++;
        ZQS_LAUNCH_CHECK("k_advect_vel_macout");
        return ZQS_OK;
    }
    if (mode == ZQS_ADV_VEL_INREG_OUTREG) {
        int rc = launch_mac_to_reg4(g, g.u, g.v, g.w, g.t4a, s, lc);
        if (rc) return rc;
        dim3 gc((L.W + 31) / 32, (L.H + 7) / 8, L.D);
        k_advect_vel_regreg<<<gc, b, 0, s>>>(L, g.t4a, g.flags, g.t4b, kp);
        dim3 gf((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, L.D + 1);
        k_reg4_to_mac_apply<<<gf, b, 0, s>>>(L, g.t4b, g.flags, g.u, g.v, g.w, g.u2, g.v2, g.w2, open);
        lc.n += 2;
        ZQS_LAUNCH_CHECK("k_advect_vel_regreg");
        return ZQS_OK;
    }
    set_error("advect_velocity: mode " + std::to_string(mode) + " (BFECC) is not implemented");
    return ZQS_EUNSUPPORTED;
}

int launch_advect_scalar(const DevGrid& g, const KParams& kp, int mode, bool fold_atten, const SourceList* src,
                         cudaStream_t s, LaunchCounter& lc) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    dim3 gc((L.W + 31) / 32, (L.H + 7) / 8, L.D);
    SourceList none;
    none.n = 0;
    const SourceList& sl = src ? *src : none;
    float aT = fold_atten ? kp.temp_atten : 1.0f;
    float aD = fold_atten ? kp.dens_atten : 1.0f;
    const Quads Q{{g.qu, g.qv, g.qw}};
    if (mode == ZQS_ADV_SCA_MAC) {
        int rc = launch_mac_quads(g, s, lc);
        if (rc) return rc;
        k_advect_scalar<false><<<gc, b, 0, s>>>(L, g.t4a, Q, g.flags, g.T, g.rho, g.T2, g.rho2, kp, aT, aD, sl);
    } else if (mode == ZQS_ADV_SCA_REG) {
        DevGrid& gm = const_cast<DevGrid&>(g);
        int rc = launch_mac_to_reg4(gm, g.u, g.v, g.w, g.t4a, s, lc);
        if (rc) return rc;
        k_advect_scalar<true><<<gc, b, 0, s>>>(L, g.t4a, Q, g.flags, g.T, g.rho, g.T2, g.rho2, kp, aT, aD, sl);
    } else {
        set_error("advect_scalar: mode " + std::to_string(mode) + " (BFECC) is not implemented");
        return ZQS_EUNSUPPORTED;
    }
    lc.n++;
    ZQS_LAUNCH_CHECK("k_advect_scalar");
    return ZQS_OK;
}

int launch_mac_quads_batch(const BatchLaunch& face, int vcur, int blocks, cudaStream_t s, LaunchCounter& lc) {
    dim3 b(32, 8, 1);
    k_mac_quads_batch<<<std::min(blocks, face.total), b, 0, s>>>(face, vcur);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_mac_quads_batch");
    return ZQS_OK;
}

int launch_advect_velocity_batch(const BatchLaunch& advf, int vcur, int blocks, cudaStream_t s, LaunchCounter& lc) {
    dim3 b(32, 8, 1);
    k_advect_vel_batch<<<std::min(blocks, advf.total), b, 0, s>>>(advf, vcur);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_advect_vel_batch");
    return ZQS_OK;
}

int launch_advect_scalar_batch(const BatchLaunch& cell, int vcur, int scur, int blocks, cudaStream_t s,
                               LaunchCounter& lc) {
    dim3 b(32, 8, 1);
    k_advect_scalar_batch<<<std::min(blocks, cell.total), b, 0, s>>>(cell, vcur, scur);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_advect_scalar_batch");
    return ZQS_OK;
}

int launch_reinject(const DevGrid& g, const SourceList& src, cudaStream_t s, LaunchCounter& lc) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    dim3 gc((L.W + 31) / 32, (L.H + 7) / 8, L.D);
    k_reinject<<<gc, b, 0, s>>>(L, g.T, g.rho, src);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_reinject");
    return ZQS_OK;
}

}  // namespace zqs
