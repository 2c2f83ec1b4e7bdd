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

namespace zqs {

namespace {

struct Ax {
    int i0, i1;
    float t;
};

// Clamp-to-edge linear filter along one axis; g in texel-index units.
__device__ __forceinline__ Ax axis(float g, int n) {
    g = fminf(fmaxf(g, -1.0f), (float)n);
    float f = floorf(g);
    Ax a;
    a.t = g - f;
    int i = (int)f;
    a.i0 = min(max(i, 0), n - 1);
    a.i1 = min(max(i + 1, 0), n - 1);
    return a;
}

__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + t * (b - a); }

struct Corners {
    int r00, r10, r01, r11;  // row offsets (j0,k0) (j1,k0) (j0,k1) (j1,k1)
    int i0, i1;
    float tx, ty, tz;
};

__device__ __forceinline__ Corners corners(const Layout& L, int nx, int ny, int nz, float gx, float gy, float gz) {
    Ax ax = axis(gx, nx), ay = axis(gy, ny), az = axis(gz, nz);
    Corners c;
    c.r00 = (az.i0 * L.py + ay.i0) * L.px;
    c.r10 = (az.i0 * L.py + ay.i1) * L.px;
    c.r01 = (az.i1 * L.py + ay.i0) * L.px;
    c.r11 = (az.i1 * L.py + ay.i1) * L.px;
    c.i0 = ax.i0;
    c.i1 = ax.i1;
    c.tx = ax.t;
    c.ty = ay.t;
    c.tz = az.t;
    return c;
}

// x, then y, then z (same tree as the oracle's trilinear()).
__device__ __forceinline__ float tri(const float* __restrict__ f, const Corners& c, float scale) {
    float c00 = lerpf(__ldg(f + c.r00 + c.i0) * scale, __ldg(f + c.r00 + c.i1) * scale, c.tx);
    float c10 = lerpf(__ldg(f + c.r10 + c.i0) * scale, __ldg(f + c.r10 + c.i1) * scale, c.tx);
    float c01 = lerpf(__ldg(f + c.r01 + c.i0) * scale, __ldg(f + c.r01 + c.i1) * scale, c.tx);
    float c11 = lerpf(__ldg(f + c.r11 + c.i0) * scale, __ldg(f + c.r11 + c.i1) * scale, c.tx);
    float c0 = lerpf(c00, c10, c.ty);
    float c1 = lerpf(c01, c11, c.ty);
    return lerpf(c0, c1, c.tz);
}
__device__ __forceinline__ float tri_unscaled(const float* __restrict__ f, const Corners& c) {
    float c00 = lerpf(__ldg(f + c.r00 + c.i0), __ldg(f + c.r00 + c.i1), c.tx);
    float c10 = lerpf(__ldg(f + c.r10 + c.i0), __ldg(f + c.r10 + c.i1), c.tx);
    float c01 = lerpf(__ldg(f + c.r01 + c.i0), __ldg(f + c.r01 + c.i1), c.tx);
    float c11 = lerpf(__ldg(f + c.r11 + c.i0), __ldg(f + c.r11 + c.i1), c.tx);
    float c0 = lerpf(c00, c10, c.ty);
    float c1 = lerpf(c01, c11, c.ty);
    return lerpf(c0, c1, c.tz);
}
__device__ __forceinline__ float3 tri4(const float4* __restrict__ f, const Corners& c) {
    float4 a00 = __ldg(f + c.r00 + c.i0), b00 = __ldg(f + c.r00 + c.i1);
    float4 a10 = __ldg(f + c.r10 + c.i0), b10 = __ldg(f + c.r10 + c.i1);
    float4 a01 = __ldg(f + c.r01 + c.i0), b01 = __ldg(f + c.r01 + c.i1);
    float4 a11 = __ldg(f + c.r11 + c.i0), b11 = __ldg(f + c.r11 + c.i1);
    float3 r;
    {
        float c00 = lerpf(a00.x, b00.x, c.tx), c10 = lerpf(a10.x, b10.x, c.tx);
        float c01 = lerpf(a01.x, b01.x, c.tx), c11 = lerpf(a11.x, b11.x, c.tx);
        r.x = lerpf(lerpf(c00, c10, c.ty), lerpf(c01, c11, c.ty), c.tz);
    }
    {
        float c00 = lerpf(a00.y, b00.y, c.tx), c10 = lerpf(a10.y, b10.y, c.tx);
        float c01 = lerpf(a01.y, b01.y, c.tx), c11 = lerpf(a11.y, b11.y, c.tx);
        r.y = lerpf(lerpf(c00, c10, c.ty), lerpf(c01, c11, c.ty), c.tz);
    }
    {
        float c00 = lerpf(a00.z, b00.z, c.tx), c10 = lerpf(a10.z, b10.z, c.tx);
        float c01 = lerpf(a01.z, b01.z, c.tx), c11 = lerpf(a11.z, b11.z, c.tx);
        r.z = lerpf(lerpf(c00, c10, c.ty), lerpf(c01, c11, c.ty), c.tz);
    }
    return r;
}
__device__ __forceinline__ float tri4c(const float4* __restrict__ f4, int q, const Corners& c) {
    const float* f = reinterpret_cast<const float*>(f4);
    auto at = [&](int o) -> float { return __ldg(f + (size_t)o * 4 + q); };
    float c00 = lerpf(at(c.r00 + c.i0), at(c.r00 + c.i1), c.tx);
    float c10 = lerpf(at(c.r10 + c.i0), at(c.r10 + c.i1), c.tx);
    float c01 = lerpf(at(c.r01 + c.i0), at(c.r01 + c.i1), c.tx);
    float c11 = lerpf(at(c.r11 + c.i0), at(c.r11 + c.i1), c.tx);
    return lerpf(lerpf(c00, c10, c.ty), lerpf(c01, c11, c.ty), c.tz);
}

struct MacVel {
    Layout L;
    const float *u, *v, *w;
    __device__ __forceinline__ void operator()(float px, float py, float pz, float& vx, float& vy, float& vz) const {
        vx = tri_unscaled(u, corners(L, L.W + 1, L.H, L.D, px, py - 0.5f, pz - 0.5f));
        vy = tri_unscaled(v, corners(L, L.W, L.H + 1, L.D, px - 0.5f, py, pz - 0.5f));
        vz = tri_unscaled(w, corners(L, L.W, L.H, L.D + 1, px - 0.5f, py - 0.5f, pz));
    }
};
struct RegVel {
    Layout L;
    const float4* vel4;
    __device__ __forceinline__ void operator()(float px, float py, float pz, float& vx, float& vy, float& vz) const {
        float3 r = tri4(vel4, corners(L, L.W, L.H, L.D, px - 0.5f, py - 0.5f, pz - 0.5f));
        vx = r.x;
        vy = r.y;
        vz = r.z;
    }
};

// The reference backtrace (e.g. ZQ_CUDA_Advection3D.cu:253-273): test the
// point (inside [0,W]x[0,H]x[0,D] and its clamped floor cell free), remember
// it, move by -(vel*dt_sub)/h, resample; `steps` moves at most.  The result
// is the last point that passed the test before the final move.  The velocity
// after the final move is never used, so it is not sampled.
template <class VelF>
__device__ __forceinline__ void backtrace(const Layout& L, const uint8_t* __restrict__ flags, const VelF& vel,
                                          const KParams& kp, float& px, float& py, float& pz) {
    float vx, vy, vz;
    vel(px, py, pz, vx, vy, vz);
    float lx = px, ly = py, lz = pz;
    const float Wf = (float)L.W, Hf = (float)L.H, Df = (float)L.D;
    auto ok = [&](float x, float y, float z) -> bool {
        if (!(x >= 0.0f && x <= Wf && y >= 0.0f && y <= Hf && z >= 0.0f && z <= Df)) return false;
        int i = min(max((int)floorf(x), 0), L.W - 1);
        int j = min(max((int)floorf(y), 0), L.H - 1);
        int k = min(max((int)floorf(z), 0), L.D - 1);
        return (__ldg(flags + lidx(L, i, j, k)) & F_FREE) != 0;
    };
    const float dt = kp.dt_sub;
    int istep = 0;
    bool broke = false;
    do {
        if (!ok(px, py, pz)) {
            broke = true;
            break;
        }
        lx = px;
        ly = py;
        lz = pz;
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
        if (istep < kp.substeps) vel(px, py, pz, vx, vy, vz);
    } while (istep < kp.substeps);
    if (kp.full && !broke && ok(px, py, pz)) {
        lx = px;
        ly = py;
        lz = pz;
    }
    px = lx;
    py = ly;
    pz = lz;
}

__device__ __forceinline__ bool face_live(uint8_t fl, uint8_t bit, int idx, int n, bool open) {
    if (!(fl & bit)) return false;
    return open || (idx > 0 && idx < n);
}

// One thread per face: bz = comp*(D+1) + k, comp 0/1/2 = u/v/w.
// REGIN selects the regular (cell-centre float4) velocity for both the
// backtrace and the final sample (inRegular_outMAC), else MAC (inMAC_outMAC).
template <bool REGIN>
__device__ __forceinline__ void advect_vel_macout_tile(const Layout& L, const float* __restrict__ u,
                                                       const float* __restrict__ v, const float* __restrict__ w,
                                                       const float4* __restrict__ vel4,
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
            MacVel mv{L, u, v, w};
            backtrace(L, flags, mv, kp, px, py, pz);
            if (comp == 0) out = tri_unscaled(u, corners(L, L.W + 1, L.H, L.D, px, py - 0.5f, pz - 0.5f));
            else if (comp == 1) out = tri_unscaled(v, corners(L, L.W, L.H + 1, L.D, px - 0.5f, py, pz - 0.5f));
            else out = tri_unscaled(w, corners(L, L.W, L.H, L.D + 1, px - 0.5f, py - 0.5f, pz));
        }
    }
    dst[c] = out;
}

template <bool REGIN>
__global__ void __launch_bounds__(256) k_advect_vel_macout(Layout L, const float* __restrict__ u,
                                                           const float* __restrict__ v, const float* __restrict__ w,
                                                           const float4* __restrict__ vel4,
                                                           const uint8_t* __restrict__ flags, float* __restrict__ u2,
                                                           float* __restrict__ v2, float* __restrict__ w2, KParams kp,
                                                           int open) {
    advect_vel_macout_tile<REGIN>(L, u, v, w, vel4, flags, u2, v2, w2, kp, open, blockIdx.x, blockIdx.y, blockIdx.z);
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
__device__ __forceinline__ void advect_scalar_tile(const Layout& L, const float* __restrict__ u,
                                                   const float* __restrict__ v, const float* __restrict__ w,
                                                   const float4* __restrict__ vel4, const uint8_t* __restrict__ flags,
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
        MacVel mv{L, u, v, w};
        backtrace(L, flags, mv, kp, px, py, pz);
    }
    Corners cs = corners(L, L.W, L.H, L.D, px - 0.5f, py - 0.5f, pz - 0.5f);
    float t = tri(T, cs, aT);
    float d = tri(rho, cs, aD);
    if (src.n > 0) reinject_cell(src, i, j, k, t, d);
    const int c = lidx(L, i, j, k);
    T2[c] = t;
    rho2[c] = d;
}

template <bool REGIN>
__global__ void __launch_bounds__(256) k_advect_scalar(Layout L, const float* __restrict__ u,
                                                       const float* __restrict__ v, const float* __restrict__ w,
                                                       const float4* __restrict__ vel4,
                                                       const uint8_t* __restrict__ flags,
                                                       const float* __restrict__ T, const float* __restrict__ rho,
                                                       float* __restrict__ T2, float* __restrict__ rho2, KParams kp,
                                                       float aT, float aD, SourceList src) {
    advect_scalar_tile<REGIN>(L, u, v, w, vel4, flags, T, rho, T2, rho2, kp, aT, aD, src, blockIdx.x, blockIdx.y,
                              blockIdx.z);
}

// ---- batched forms (MAC velocity) ----

__global__ void __launch_bounds__(256) k_advect_vel_batch(BatchLaunch B, int vcur) {
    for (int t = blockIdx.x; t < B.total; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const InstDesc& d = B.desc[i];
        const int lt = t - __ldg(B.pre + i);
        const int gx = (d.L.W + 1 + 31) / 32, gy = (d.L.H + 1 + 7) / 8;
        const int bx = lt % gx, r = lt / gx, by = r % gy, bz = r / gy;
        const KParams kp = d.kp;
        const int nxt = vcur ^ 1;
        advect_vel_macout_tile<false>(d.L, d.vel[vcur][0], d.vel[vcur][1], d.vel[vcur][2], d.t4a, d.flags,
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
        advect_scalar_tile<false>(d.L, d.vel[vcur][0], d.vel[vcur][1], d.vel[vcur][2], d.t4a, d.flags,
                                  d.sca[scur][0], d.sca[scur][1], d.sca[nxt][0], d.sca[nxt][1], kp, kp.temp_atten,
                                  kp.dens_atten, d.src, bx, by, bz);
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

int launch_advect_velocity(DevGrid& g, const KParams& kp, int mode, bool open, cudaStream_t s, LaunchCounter& lc) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    if (mode == ZQS_ADV_VEL_INMAC_OUTMAC || mode == ZQS_ADV_VEL_INREG_OUTMAC) {
        int nxb = (L.W + 1 + 31) / 32, nyb = (L.H + 1 + 7) / 8;
        dim3 gr(nxb, nyb, 3 * (L.D + 1));
        if (mode == ZQS_ADV_VEL_INREG_OUTMAC) {
            int rc = launch_mac_to_reg4(g, g.u, g.v, g.w, g.t4a, s, lc);
            if (rc) return rc;
            k_advect_vel_macout<true><<<gr, b, 0, s>>>(L, g.u, g.v, g.w, g.t4a, g.flags, g.u2, g.v2, g.w2, kp, open);
        } else {
            k_advect_vel_macout<false><<<gr, b, 0, s>>>(L, g.u, g.v, g.w, g.t4a, g.flags, g.u2, g.v2, g.w2, kp, open);
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
    if (mode == ZQS_ADV_SCA_MAC) {
        k_advect_scalar<false><<<gc, b, 0, s>>>(L, g.u, g.v, g.w, g.t4a, g.flags, g.T, g.rho, g.T2, g.rho2, kp, aT,
                                                aD, sl);
    } else if (mode == ZQS_ADV_SCA_REG) {
        DevGrid& gm = const_cast<DevGrid&>(g);
        int rc = launch_mac_to_reg4(gm, g.u, g.v, g.w, g.t4a, s, lc);
        if (rc) return rc;
        k_advect_scalar<true><<<gc, b, 0, s>>>(L, g.u, g.v, g.w, g.t4a, g.flags, g.T, g.rho, g.T2, g.rho2, kp, aT,
                                               aD, sl);
    } else {
        set_error("advect_scalar: mode " + std::to_string(mode) + " (BFECC) is not implemented");
        return ZQS_EUNSUPPORTED;
    }
    lc.n++;
    ZQS_LAUNCH_CHECK("k_advect_scalar");
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
