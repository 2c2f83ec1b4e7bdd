// Forces (vorticity confinement + buoyancy + density weight) and attenuation.
//
// Restates cu_AddForce3D (ZQ_CUDA_AddForce3D.cu:510-556) and Attenuation3D
// (ZQ_CUDA_Attenuation3D.cu:8-116) on the padded device layout.  Three
// launches replace the reference's five kernels and seven allocations:
//   vorticity    faces -> (wx, wy, wz, |w|) per cell        (:11-34)
//   force_cell   |w| halo + w + T + rho -> force per cell    (:64-111, :161-184)
//   force_faces  force -> face update, velocity attenuation fused (:211-385)
// The expression order of every float operation matches the oracle
// (oracle/zqs_oracle.cpp, add_force/attenuate) so FP32 results agree exactly.
// Each stage is a tile function over one 32x8 block of (i,j) at plane k,
// launched directly for one grid or through the batch work list.
#include <algorithm>

#include "zqs_batch.h"

namespace zqs {

namespace {

__device__ __forceinline__ float ctr_u(const float* __restrict__ u, int c) {
    return 0.5f * (__ldg(u + c) + __ldg(u + c + 1));
}
__device__ __forceinline__ float ctr_v(const float* __restrict__ v, int c, int px) {
    return 0.5f * (__ldg(v + c) + __ldg(v + c + px));
}
__device__ __forceinline__ float ctr_w(const float* __restrict__ w, int c, int pl) {
    return 0.5f * (__ldg(w + c) + __ldg(w + c + pl));
}

// Vorticity of the cell-centre velocity on cells with every index in [1,N-2]
// (ZQ_CUDA_AddForce3D.cu:11-34); other cells get 0 as the reference memsets.
__device__ __forceinline__ void vorticity_tile(const Layout& L, const float* __restrict__ u,
                                               const float* __restrict__ v, const float* __restrict__ w,
                                               float4* __restrict__ vort, float twoh, int bx, int by, int bz) {
    int i = bx * 32 + threadIdx.x;
    int j = by * 8 + threadIdx.y;
    int k = bz;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i >= 1 && i <= L.W - 2 && j >= 1 && j <= L.H - 2 && k >= 1 && k <= L.D - 2) {
        float ox = (((ctr_w(w, c + px, pl) - ctr_w(w, c - px, pl)) - ctr_v(v, c + pl, px)) + ctr_v(v, c - pl, px)) / twoh;
        float oy = (((ctr_u(u, c + pl) - ctr_u(u, c - pl)) - ctr_w(w, c + 1, pl)) + ctr_w(w, c - 1, pl)) / twoh;
        float oz = (((ctr_v(v, c + 1, px) - ctr_v(v, c - 1, px)) - ctr_u(u, c + px)) + ctr_u(u, c - px)) / twoh;
        r.x = ox;
        r.y = oy;
        r.z = oz;
        r.w = sqrtf((ox * ox + oy * oy) + oz * oz);
    }
    vort[c] = r;
}

// N = normalised gradient of |w| (ZQ_CUDA_AddForce3D.cu:64-111) and
// f = (eps*h)*(N x w); f_y += beta*(T-Tamb); f_y -= alpha*rho (:161-184).
__device__ __forceinline__ void force_cell_tile(const Layout& L, const float4* __restrict__ vort,
                                                const float* __restrict__ T, const float* __restrict__ rho,
                                                float4* __restrict__ force, const KParams& kp, int bx, int by,
                                                int bz) {
    int i = bx * 32 + threadIdx.x;
    int j = by * 8 + threadIdx.y;
    int k = bz;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    auto S = [&](int o) -> float { return __ldg(&vort[o].w); };
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
    float len = sqrtf((gx * gx + gy * gy) + gz * gz);
    if (len != 0.0f) {
        gx = gx / len;
        gy = gy / len;
        gz = gz / len;
    }
    float4 o = vort[c];
    float fx = kp.cc * (gy * o.z - gz * o.y);
    float fy = kp.cc * (gz * o.x - gx * o.z);
    float fz = kp.cc * (gx * o.y - gy * o.x);
    fy = fy + kp.beta * (__ldg(T + c) - kp.tamb);
    fy = fy - kp.alpha * __ldg(rho + c);
    if (kp.fext) {
        fx = fx + __ldg(kp.fext + c);
        fy = fy + __ldg(kp.fext + L.elems + c);
        fz = fz + __ldg(kp.fext + 2 * L.elems + c);
    }
    force[c] = make_float4(fx, fy, fz, 0.0f);
}

// Face update (ZQ_CUDA_AddForce3D.cu:211-385, w per-slice form :387-420);
// ATTEN also multiplies live faces by vel_atten, which is the next stage of
// the reference step (ZQ_CUDA_Attenuation3D.cu:8-98) applied to the same faces.
template <bool ATTEN>
__device__ __forceinline__ void force_faces_tile(const Layout& L, float* __restrict__ u, float* __restrict__ v,
                                                 float* __restrict__ w, const uint8_t* __restrict__ flags,
                                                 const float4* __restrict__ force, const KParams& kp, int bx,
                                                 int by, int bz) {
    int i = bx * 32 + threadIdx.x;
    int j = by * 8 + threadIdx.y;
    int k = bz;
    if (i > L.W || j > L.H || k > L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    const uint8_t fl = __ldg(flags + c);
    const float dt = kp.dt;
    const float hdt = dt * 0.5f;
    if (fl & F_UFACE) {
        float f = u[c];
        if (i == 0) f = f + dt * __ldg(&force[c].x);
        else if (i == L.W) f = f + dt * __ldg(&force[c - 1].x);
        else f = f + hdt * (__ldg(&force[c].x) + __ldg(&force[c - 1].x));
        if (ATTEN) f = f * kp.vel_atten;
        u[c] = f;
    }
    if (fl & F_VFACE) {
        float f = v[c];
        if (j == 0) f = f + dt * __ldg(&force[c].y);
        else if (j == L.H) f = f + dt * __ldg(&force[c - px].y);
        else f = f + hdt * (__ldg(&force[c].y) + __ldg(&force[c - px].y));
        if (ATTEN) f = f * kp.vel_atten;
        v[c] = f;
    }
    if (fl & F_WFACE) {
        float f = w[c];
        if (k == 0) f = f + dt * __ldg(&force[c].z);
        else if (k == L.D) f = f + dt * __ldg(&force[c - pl].z);
        else f = f + hdt * (__ldg(&force[c].z) + __ldg(&force[c - pl].z));
        if (ATTEN) f = f * kp.vel_atten;
        w[c] = f;
    }
}

__global__ void k_vorticity(Layout L, const float* __restrict__ u, const float* __restrict__ v,
                            const float* __restrict__ w, float4* __restrict__ vort, float twoh) {
    vorticity_tile(L, u, v, w, vort, twoh, blockIdx.x, blockIdx.y, blockIdx.z);
}

__global__ void k_force_cell(Layout L, const float4* __restrict__ vort, const float* __restrict__ T,
                             const float* __restrict__ rho, float4* __restrict__ force, KParams kp) {
    force_cell_tile(L, vort, T, rho, force, kp, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <bool ATTEN>
__global__ void k_force_faces(Layout L, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w,
                              const uint8_t* __restrict__ flags, const float4* __restrict__ force, KParams kp) {
    force_faces_tile<ATTEN>(L, u, v, w, flags, force, kp, blockIdx.x, blockIdx.y, blockIdx.z);
}

// Attenuation3D as a stage of its own (ZQ_CUDA_Attenuation3D.cu:8-116).
__global__ void k_attenuate(Layout L, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w,
                            float* __restrict__ T, float* __restrict__ rho, const uint8_t* __restrict__ flags,
                            KParams kp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i > L.W || j > L.H || k > L.D) return;
    const int c = lidx(L, i, j, k);
    const uint8_t fl = __ldg(flags + c);
    if (fl & F_UFACE) u[c] = u[c] * kp.vel_atten;
    if (fl & F_VFACE) v[c] = v[c] * kp.vel_atten;
    if (fl & F_WFACE) w[c] = w[c] * kp.vel_atten;
    if (i < L.W && j < L.H && k < L.D) {
        T[c] = T[c] * kp.temp_atten;
        rho[c] = rho[c] * kp.dens_atten;
    }
}

// ---- batched forms: one persistent launch over every instance's tiles ----

__device__ __forceinline__ void tile_coords(const Layout& L, int lt, int wx, int wy, int& bx, int& by, int& bz) {
    const int gx = (wx + 31) / 32, gy = (wy + 7) / 8;
    bx = lt % gx;
    const int r = lt / gx;
    by = r % gy;
    bz = r / gy;
}

__global__ void k_vorticity_batch(BatchLaunch B, int vcur) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[i];
        int bx, by, bz;
        tile_coords(d.L, t - __ldg(B.pre + i), d.L.W, d.L.H, bx, by, bz);
        vorticity_tile(d.L, d.vel[vcur][0], d.vel[vcur][1], d.vel[vcur][2], d.t4a, d.kp.twoh, bx, by, bz);
    }
}

__global__ void k_force_cell_batch(BatchLaunch B, int scur) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[i];
        int bx, by, bz;
        tile_coords(d.L, t - __ldg(B.pre + i), d.L.W, d.L.H, bx, by, bz);
        const KParams kp = d.kp;
        force_cell_tile(d.L, d.t4a, d.sca[scur][0], d.sca[scur][1], d.t4b, kp, bx, by, bz);
    }
}

__global__ void k_force_faces_batch(BatchLaunch B, int vcur) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[i];
        int bx, by, bz;
        tile_coords(d.L, t - __ldg(B.pre + i), d.L.W + 1, d.L.H + 1, bx, by, bz);
        const KParams kp = d.kp;
        force_faces_tile<true>(d.L, d.vel[vcur][0], d.vel[vcur][1], d.vel[vcur][2], d.flags, d.t4b, kp, bx, by,
                               bz);
    }
}

}  // namespace

int launch_force(const DevGrid& g, const KParams& kp, bool fuse_vel_atten, cudaStream_t s, LaunchCounter& lc) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    dim3 gc((L.W + 31) / 32, (L.H + 7) / 8, L.D);
    dim3 gf((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, L.D + 1);
    k_vorticity<<<gc, b, 0, s>>>(L, g.u, g.v, g.w, g.t4a, kp.twoh);
    k_force_cell<<<gc, b, 0, s>>>(L, g.t4a, g.T, g.rho, g.t4b, kp);
    if (fuse_vel_atten) k_force_faces<true><<<gf, b, 0, s>>>(L, g.u, g.v, g.w, g.flags, g.t4b, kp);
    else k_force_faces<false><<<gf, b, 0, s>>>(L, g.u, g.v, g.w, g.flags, g.t4b, kp);
    lc.n += 3;
    ZQS_LAUNCH_CHECK("force kernels");
    return ZQS_OK;
}

int launch_attenuate(const DevGrid& g, const KParams& kp, cudaStream_t s, LaunchCounter& lc) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    dim3 gf((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, L.D + 1);
    k_attenuate<<<gf, b, 0, s>>>(L, g.u, g.v, g.w, g.T, g.rho, g.flags, kp);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_attenuate");
    return ZQS_OK;
}

int launch_force_batch(const BatchLaunch& cell, const BatchLaunch& face, int vcur, int scur, int blocks,
                       cudaStream_t s, LaunchCounter& lc) {
    dim3 b(32, 8, 1);
    k_vorticity_batch<<<persistent_blocks((const void*)k_vorticity_batch, 256, 0, std::min(blocks, cell.total)), b, 0,
                        s>>>(cell, vcur);
    k_force_cell_batch<<<persistent_blocks((const void*)k_force_cell_batch, 256, 0, std::min(blocks, cell.total)), b, 0,
                         s>>>(cell, scur);
    k_force_faces_batch<<<persistent_blocks((const void*)k_force_faces_batch, 256, 0, std::min(blocks, face.total)), b, 0,
                          s>>>(face, vcur);
    lc.n += 3;
    ZQS_LAUNCH_CHECK("batched force kernels");
    return ZQS_OK;
}

}  // namespace zqs
