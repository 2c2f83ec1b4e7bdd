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

// Buffers of one velocity advection pass.
struct VelPass {
    const float4* q[3];   // MAC velocity as quad copies (zqs_sample.cuh, tri0_quad)
    const float4* vel4;   // regular velocity (REGIN)
    const float* in[3];   // MAC input sampled at the end point (SEPIN), else the velocity itself
    const float4* in4;    // regular input (REGIN)
    const float* keep[3]; // value of a face the write-back leaves alone
    float* out[3];
};

// One thread per face: bz = 3*k + comp, comp 0/1/2 = u/v/w.  The three
// components of a plane are adjacent in the launch order, so the CTAs resident
// together sample the velocity around the same few planes and every quad line
// comes from DRAM about once (component-major order streamed the three quad
// arrays once per component).
// REGIN: the regular (cell-centre float4) velocity for the backtrace and the
// regular input for the final sample (inRegular_outMAC), else MAC velocity
// read through its quad copies (inMAC_outMAC).  RAW: every face of the
// component is backtraced and written (a BFECC pass), else the open/closed
// write-back keeps keep[] on faces it leaves alone.  NEG: through the negated
// velocity.  SEPIN: the MAC input is in[] rather than the velocity itself.
template <bool REGIN, bool RAW, bool NEG, bool SEPIN>
__device__ __forceinline__ void advect_vel_macout_tile(const Layout& L, const VelPass& P,
                                                       const uint8_t* __restrict__ flags, const KParams& kp,
                                                       int open, int bx, int by, int bz) {
    const int i = bx * 32 + threadIdx.x;
    const int j = by * 8 + threadIdx.y;
    const int k = bz / 3;
    const int comp = bz - 3 * k;
    int nx = L.W, ny = L.H, nz = L.D;
    if (comp == 0) nx++;
    else if (comp == 1) ny++;
    else nz++;
    if (i >= nx || j >= ny || k >= nz) return;
    const int c = lidx(L, i, j, k);
    // per-component pointers by select (a dynamic index into P would copy it
    // to local memory)
    auto pick = [comp](auto a, auto b, auto c) { return comp == 0 ? a : (comp == 1 ? b : c); };
    float* dst = pick(P.out[0], P.out[1], P.out[2]);
    bool live = true;
    if (!RAW) {
        const uint8_t fl = __ldg(flags + c);
        const uint8_t bit = comp == 0 ? F_UFACE : (comp == 1 ? F_VFACE : F_WFACE);
        const int along = comp == 0 ? i : (comp == 1 ? j : k);
        const int n = comp == 0 ? L.W : (comp == 1 ? L.H : L.D);
        live = face_live(fl, bit, along, n, open != 0);
    }
    float out;
    if (live) {
        float px = (comp == 0) ? (float)i : (float)i + 0.5f;
        float py = (comp == 1) ? (float)j : (float)j + 0.5f;
        float pz = (comp == 2) ? (float)k : (float)k + 0.5f;
        if (REGIN) {
            const RegVelT<NEG> rv{L, P.vel4};
            backtrace(L, flags, rv, kp, px, py, pz);
            out = tri4c(P.in4, comp, corners(L, L.W, L.H, L.D, px - 0.5f, py - 0.5f, pz - 0.5f));
        } else {
            MacVelQC<NEG> mv(L, P.q[0], P.q[1], P.q[2]);
            backtrace(L, flags, mv, kp, px, py, pz);
            Tri0 t;
            if (comp == 0) t = tri0(L, L.W + 1, L.H, L.D, px, py - 0.5f, pz - 0.5f);
            else if (comp == 1) t = tri0(L, L.W, L.H + 1, L.D, px - 0.5f, py, pz - 0.5f);
            else t = tri0(L, L.W, L.H, L.D + 1, px - 0.5f, py - 0.5f, pz);
            out = SEPIN ? tri0_sample(pick(P.in[0], P.in[1], P.in[2]), L, t)
                        : mv.sample(comp, pick(P.q[0], P.q[1], P.q[2]), t);
        }
    } else {
        out = __ldg(pick(P.keep[0], P.keep[1], P.keep[2]) + c);
    }
    dst[c] = out;
}

template <bool REGIN, bool RAW, bool NEG, bool SEPIN>
__global__ void __launch_bounds__(256) k_advect_vel_macout(Layout L, VelPass P, const uint8_t* __restrict__ flags,
                                                           KParams kp, int open) {
    advect_vel_macout_tile<REGIN, RAW, NEG, SEPIN>(L, P, flags, kp, open, blockIdx.x, blockIdx.y, blockIdx.z);
}

// Advect_Velocity_inRegular_outRegular_Kernel (Adv3D:76-113): per cell,
// through the (NEG: negated) regular velocity, sampling the regular input.
template <bool NEG>
__global__ void __launch_bounds__(256) k_advect_vel_regreg(Layout L, const float4* __restrict__ vel4,
                                                           const float4* __restrict__ in4,
                                                           const uint8_t* __restrict__ flags,
                                                           float4* __restrict__ out4, KParams kp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    float px = (float)i + 0.5f, py = (float)j + 0.5f, pz = (float)k + 0.5f;
    const RegVelT<NEG> rv{L, vel4};
    backtrace(L, flags, rv, kp, px, py, pz);
    float3 r = tri4(in4, corners(L, L.W, L.H, L.D, px - 0.5f, py - 0.5f, pz - 0.5f));
    out4[lidx(L, i, j, k)] = make_float4(r.x, r.y, r.z, 0.0f);
}

// BFECC corrections (Input_Increment_Kernel / _4channels_Kernel, Adv3D:56-74).
// The float-array kernel multiplies by double constants, so the expression is
// evaluated in double and rounded once; the float4 kernel rounds each float
// operation.  Faces: every face of the three components, s <- 1.5 b - 0.5 s.
__device__ __forceinline__ float bfecc_inc(float b, float s) {
    return __double2float_rn(__dsub_rn(__dmul_rn((double)b, 1.5), __dmul_rn((double)s, 0.5)));
}
__device__ __forceinline__ float bfecc_inc4(float b, float s) {
    return __fsub_rn(__fmul_rn(b, 1.5f), __fmul_rn(s, 0.5f));
}
__global__ void k_bfecc_inc_faces(Layout L, const float* __restrict__ bu, const float* __restrict__ bv,
                                  const float* __restrict__ bw, float* __restrict__ su, float* __restrict__ sv,
                                  float* __restrict__ sw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > L.W || j > L.H || k > L.D) return;
    const int c = lidx(L, i, j, k);
    if (j < L.H && k < L.D) su[c] = bfecc_inc(__ldg(bu + c), su[c]);
    if (i < L.W && k < L.D) sv[c] = bfecc_inc(__ldg(bv + c), sv[c]);
    if (i < L.W && j < L.H) sw[c] = bfecc_inc(__ldg(bw + c), sw[c]);
}
// Regular cells, every channel.
__global__ void k_bfecc_inc_reg4(Layout L, const float4* __restrict__ b4, float4* __restrict__ s4) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    const float4 b = __ldg(b4 + c);
    float4 x = s4[c];
    x.x = bfecc_inc4(b.x, x.x);
    x.y = bfecc_inc4(b.y, x.y);
    x.z = bfecc_inc4(b.z, x.z);
    x.w = bfecc_inc4(b.w, x.w);
    s4[c] = x;
}
// Scalar cells: the input is the attenuated field fl(T * aT) (what the
// separate attenuation pass leaves), corrected with the backward result s.
__global__ void k_bfecc_inc_cells(Layout L, const float* __restrict__ T, const float* __restrict__ rho, float aT,
                                  float aD, float* __restrict__ sT, float* __restrict__ sD) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    sT[c] = bfecc_inc(__fmul_rn(__ldg(T + c), aT), sT[c]);
    sD[c] = bfecc_inc(__fmul_rn(__ldg(rho + c), aD), sD[c]);
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

struct Quads {
    const float4* q[3];
};

// Advect_Scalar_{MAC,Regular}_Velocity_Kernel (Adv3D:379-469) with the
// attenuation factors applied to the interpolation corners and the sources
// reinjected in the epilogue.  NEG: through the negated velocity.
template <bool REGIN, bool NEG = false>
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
        const RegVelT<NEG> rv{L, vel4};
        backtrace(L, flags, rv, kp, px, py, pz);
    } else {
        MacVelQC<NEG> mv(L, q[0], q[1], q[2]);
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

template <bool REGIN, bool NEG>
__global__ void __launch_bounds__(256) k_advect_scalar(Layout L, const float4* __restrict__ vel4, Quads Q,
                                                       const uint8_t* __restrict__ flags,
                                                       const float* __restrict__ T, const float* __restrict__ rho,
                                                       float* __restrict__ T2, float* __restrict__ rho2, KParams kp,
                                                       float aT, float aD, SourceList src) {
    advect_scalar_tile<REGIN, NEG>(L, vel4, Q.q, flags, T, rho, T2, rho2, kp, aT, aD, src, blockIdx.x,
                                   blockIdx.y, blockIdx.z);
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

static_assert(sizeof(AdvHotTable) + 64 <= 32764, "the hot table must fit the kernel parameter space");

// Batched velocity advection over the tiles [t0, t1) of one table chunk
// (launched with one CTA per tile; the loop also serves smaller grids).
__global__ void __launch_bounds__(256, 4) k_advect_vel_batch(BatchLaunch B, const __grid_constant__ AdvHotTable T,
                                                         int vcur, int t0, int t1) {
    for (int t = t0 + blockIdx.x; t < t1; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const AdvHot& d = T.h[i - T.base];
        const int lt = t - __ldg(B.pre + i);
        const int gx = (d.L.W + 1 + 31) / 32, gy = (d.L.H + 1 + 7) / 8;
        const int bx = lt % gx, r = lt / gx, by = r % gy, bz = r / gy;
        const int nxt = vcur ^ 1;
        VelPass P;
        for (int m = 0; m < 3; m++) {
            P.q[m] = d.q[m];
            P.in[m] = d.vel[vcur][m];
            P.keep[m] = d.vel[vcur][m];
            P.out[m] = d.vel[nxt][m];
        }
        P.vel4 = P.in4 = nullptr;  // MAC velocity only
        advect_vel_macout_tile<false, false, false, false>(d.L, P, d.flags, d.kp, 1, bx, by, bz);
    }
}

// Batched scalar advection (+ attenuation, + reinjection) over the tiles
// [t0, t1) of one table chunk; the sources come from the instance descriptor.
__global__ void __launch_bounds__(256, 4) k_advect_scalar_batch(BatchLaunch B, const __grid_constant__ AdvHotTable T,
                                                            int vcur, int scur, int t0, int t1) {
    for (int t = t0 + blockIdx.x; t < t1; t += gridDim.x) {
        const int i = batch_find(B.pre, B.n, t);
        const AdvHot& d = T.h[i - T.base];
        const int lt = t - __ldg(B.pre + i);
        const int gx = (d.L.W + 31) / 32, gy = (d.L.H + 7) / 8;
        const int bx = lt % gx, r = lt / gx, by = r % gy, bz = r / gy;
        const int nxt = scur ^ 1;
        advect_scalar_tile<false>(d.L, nullptr, d.q, d.flags, d.sca[scur][0], d.sca[scur][1], d.sca[nxt][0],
                                  d.sca[nxt][1], d.kp, d.kp.temp_atten, d.kp.dens_atten, B.desc[i].src, bx, by,
                                  bz);
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

namespace {

// Float field m (0..3) carved from a float4 field's storage, with its own
// leading guard plane: one float4 field holds four padded float fields.
float* f4_slot(float4* t4, const Layout& L, int m) {
    return reinterpret_cast<float*>(t4 - L.plane) + (size_t)m * L.elems + L.plane;
}
// Zero a float4 field's whole storage (padding and guard planes included), so
// float fields carved from it read zero outside what a pass writes.
cudaError_t zero_f4(float4* t4, const Layout& L, cudaStream_t s) {
    return cudaMemsetAsync(t4 - L.plane, 0, (size_t)L.elems * sizeof(float4), s);
}

}  // namespace

// Advect_Velocity (Adv3D:1686-1749): the six modes.  BFECC (Adv3D:1108-1182,
// 1240-1336, 1389-1474) runs a forward pass, a pass through the negated
// velocity from its result, the correction in~ = 1.5 in - 0.5 in**, and a
// forward pass from in~, all through the original velocity.  The MAC form
// corrects u, v, w themselves in the reference, so faces the write-back leaves
// alone end with the corrected value; here the corrected field sits in t4b's
// storage and is what the write-back keeps.  Scratch: t4a / t4b (float4 or
// three float fields each) and the quad storage qu as a float4 field when the
// velocity is regular.
int launch_advect_velocity(DevGrid& g, const KParams& kp, int mode, bool open, cudaStream_t s, LaunchCounter& lc) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    const dim3 gr((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, 3 * (L.D + 1));  // faces, one z block per component plane
    const dim3 gc((L.W + 31) / 32, (L.H + 7) / 8, L.D);                    // cells
    const dim3 gf((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, L.D + 1);        // the face index box
    const int op = open ? 1 : 0;
    VelPass P;
    float* vel[3] = {g.u, g.v, g.w};
    float* out[3] = {g.u2, g.v2, g.w2};
    const float4* quads[3] = {g.qu, g.qv, g.qw};
    for (int m = 0; m < 3; m++) {
        P.q[m] = quads[m];
        P.in[m] = vel[m];
        P.keep[m] = vel[m];
        P.out[m] = out[m];
    }
    P.vel4 = P.in4 = g.t4a;
    int rc = ZQS_OK;
    switch (mode) {
        case ZQS_ADV_VEL_INMAC_OUTMAC:
            if ((rc = launch_mac_quads(g, s, lc))) return rc;
            k_advect_vel_macout<false, false, false, false><<<gr, b, 0, s>>>(L, P, g.flags, kp, op);
            lc.n++;
            break;
        case ZQS_ADV_VEL_INMAC_OUTMAC_BFECC: {
            if ((rc = launch_mac_quads(g, s, lc))) return rc;
            ZQS_CUDA_TRY(zero_f4(g.t4a, L, s));
            ZQS_CUDA_TRY(zero_f4(g.t4b, L, s));
            VelPass P1 = P, P2 = P, P3 = P;
            for (int m = 0; m < 3; m++) {
                P1.out[m] = f4_slot(g.t4a, L, m);                 // u* = A(u; u)
                P2.in[m] = P1.out[m];
                P2.out[m] = f4_slot(g.t4b, L, m);                 // u** = A(u*; -u)
                P3.in[m] = P3.keep[m] = P2.out[m];                // u~ = 1.5 u - 0.5 u**
            }
            k_advect_vel_macout<false, true, false, false><<<gr, b, 0, s>>>(L, P1, g.flags, kp, op);
            k_advect_vel_macout<false, true, true, true><<<gr, b, 0, s>>>(L, P2, g.flags, kp, op);
            k_bfecc_inc_faces<<<gf, b, 0, s>>>(L, g.u, g.v, g.w, P2.out[0], P2.out[1], P2.out[2]);
            k_advect_vel_macout<false, false, false, true><<<gr, b, 0, s>>>(L, P3, g.flags, kp, op);
            lc.n += 4;
            break;
        }
        case ZQS_ADV_VEL_INREG_OUTMAC:
            if ((rc = launch_mac_to_reg4(g, g.u, g.v, g.w, g.t4a, s, lc))) return rc;
            k_advect_vel_macout<true, false, false, false><<<gr, b, 0, s>>>(L, P, g.flags, kp, op);
            lc.n++;
            break;
        case ZQS_ADV_VEL_INREG_OUTMAC_BFECC: {
            if ((rc = launch_mac_to_reg4(g, g.u, g.v, g.w, g.t4a, s, lc))) return rc;
            VelPass P1 = P, P2 = P, P3 = P;
            for (int m = 0; m < 3; m++) P1.out[m] = P2.out[m] = f4_slot(g.t4b, L, m);
            P2.in4 = P3.in4 = g.qu;
            k_advect_vel_macout<true, true, false, false><<<gr, b, 0, s>>>(L, P1, g.flags, kp, op);
            lc.n++;
            if ((rc = launch_mac_to_reg4(g, P1.out[0], P1.out[1], P1.out[2], g.qu, s, lc))) return rc;
            k_advect_vel_macout<true, true, true, false><<<gr, b, 0, s>>>(L, P2, g.flags, kp, op);
            lc.n++;
            if ((rc = launch_mac_to_reg4(g, P2.out[0], P2.out[1], P2.out[2], g.qu, s, lc))) return rc;
            k_bfecc_inc_reg4<<<gc, b, 0, s>>>(L, g.t4a, g.qu);
            k_advect_vel_macout<true, false, false, false><<<gr, b, 0, s>>>(L, P3, g.flags, kp, op);
            lc.n += 2;
            break;
        }
        case ZQS_ADV_VEL_INREG_OUTREG:
        case ZQS_ADV_VEL_INREG_OUTREG_BFECC: {
            if ((rc = launch_mac_to_reg4(g, g.u, g.v, g.w, g.t4a, s, lc))) return rc;
            if (mode == ZQS_ADV_VEL_INREG_OUTREG) {
                k_advect_vel_regreg<false><<<gc, b, 0, s>>>(L, g.t4a, g.t4a, g.flags, g.t4b, kp);
                lc.n++;
            } else {
                k_advect_vel_regreg<false><<<gc, b, 0, s>>>(L, g.t4a, g.t4a, g.flags, g.t4b, kp);
                k_advect_vel_regreg<true><<<gc, b, 0, s>>>(L, g.t4a, g.t4b, g.flags, g.qu, kp);
                k_bfecc_inc_reg4<<<gc, b, 0, s>>>(L, g.t4a, g.qu);
                k_advect_vel_regreg<false><<<gc, b, 0, s>>>(L, g.t4a, g.qu, g.flags, g.t4b, kp);
                lc.n += 4;
            }
            k_reg4_to_mac_apply<<<gf, b, 0, s>>>(L, g.t4b, g.flags, g.u, g.v, g.w, g.u2, g.v2, g.w2, op);
            lc.n++;
            break;
        }
        default:
            set_error("advect_velocity: unknown mode " + std::to_string(mode));
            return ZQS_EINVAL;
    }
    ZQS_LAUNCH_CHECK("advect_velocity");
    return ZQS_OK;
}

// Advect_Scalar (Adv3D:1751-1821) through MAC or regular velocity; BFECC as
// cu_Advect_Scalar_{MAC,Regular}_Velocity_BFECC (Adv3D:1507-1554, 1586-1648):
// forward pass (attenuation folded into the corners), negated-velocity pass
// from its result, the correction of the attenuated inputs, forward pass from
// the corrected fields with the sources reinjected.  (The reference's entry
// point never reaches those functions for the BFECC types and returns zeros,
// Adv3D:1786-1794.)
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
    DevGrid& gm = const_cast<DevGrid&>(g);
    const bool reg = mode == ZQS_ADV_SCA_REG || mode == ZQS_ADV_SCA_REG_BFECC;
    const bool bfecc = mode == ZQS_ADV_SCA_MAC_BFECC || mode == ZQS_ADV_SCA_REG_BFECC;
    if (mode < ZQS_ADV_SCA_MAC || mode > ZQS_ADV_SCA_REG_BFECC) {
        set_error("advect_scalar: unknown mode " + std::to_string(mode));
        return ZQS_EINVAL;
    }
    int rc = reg ? launch_mac_to_reg4(gm, g.u, g.v, g.w, g.t4a, s, lc) : launch_mac_quads(g, s, lc);
    if (rc) return rc;
    auto pass = [&](bool neg, const float* ti, const float* di, float* to, float* dout, float st, float sd,
                    const SourceList& sr) {
        if (reg && !neg) k_advect_scalar<true, false><<<gc, b, 0, s>>>(L, g.t4a, Q, g.flags, ti, di, to, dout, kp, st, sd, sr);
        if (reg && neg) k_advect_scalar<true, true><<<gc, b, 0, s>>>(L, g.t4a, Q, g.flags, ti, di, to, dout, kp, st, sd, sr);
        if (!reg && !neg) k_advect_scalar<false, false><<<gc, b, 0, s>>>(L, g.t4a, Q, g.flags, ti, di, to, dout, kp, st, sd, sr);
        if (!reg && neg) k_advect_scalar<false, true><<<gc, b, 0, s>>>(L, g.t4a, Q, g.flags, ti, di, to, dout, kp, st, sd, sr);
        lc.n++;
    };
    if (!bfecc) {
        pass(false, g.T, g.rho, g.T2, g.rho2, aT, aD, sl);
    } else {
        ZQS_CUDA_TRY(zero_f4(g.t4b, L, s));
        float* xT = f4_slot(g.t4b, L, 0);
        float* xD = f4_slot(g.t4b, L, 1);
        pass(false, g.T, g.rho, g.T2, g.rho2, aT, aD, none);  // phi* = A(a phi; v)
        pass(true, g.T2, g.rho2, xT, xD, 1.0f, 1.0f, none);   // phi** = A(phi*; -v)
        k_bfecc_inc_cells<<<gc, b, 0, s>>>(L, g.T, g.rho, aT, aD, xT, xD);
        lc.n++;
        pass(false, xT, xD, g.T2, g.rho2, 1.0f, 1.0f, sl);    // A(1.5 a phi - 0.5 phi**; v)
    }
    ZQS_LAUNCH_CHECK("k_advect_scalar");
    return ZQS_OK;
}

int launch_mac_quads_batch(const BatchLaunch& face, int vcur, int blocks, cudaStream_t s, LaunchCounter& lc) {
    dim3 b(32, 8, 1);
    k_mac_quads_batch<<<persistent_blocks((const void*)k_mac_quads_batch, 256, 0, std::min(blocks, face.total)), b, 0,
                        s>>>(face, vcur);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_mac_quads_batch");
    return ZQS_OK;
}

int launch_advect_velocity_batch(const BatchLaunch& advf, const std::vector<AdvHotTable>& hot, int vcur,
                                 cudaStream_t s, LaunchCounter& lc) {
    dim3 b(32, 8, 1);
    for (const AdvHotTable& T : hot) {
        const int t0 = advf.pre_host[T.base], t1 = advf.pre_host[T.base + T.n];
        if (t1 <= t0) continue;
        // one CTA per tile: backtrace costs vary across tiles (plume against
        // still air), and the block scheduler balances them as CTAs finish
        k_advect_vel_batch<<<t1 - t0, b, 0, s>>>(advf, T, vcur, t0, t1);
        lc.n++;
    }
    ZQS_LAUNCH_CHECK("k_advect_vel_batch");
    return ZQS_OK;
}

int launch_advect_scalar_batch(const BatchLaunch& cell, const std::vector<AdvHotTable>& hot, int vcur, int scur,
                               cudaStream_t s, LaunchCounter& lc) {
    dim3 b(32, 8, 1);
    for (const AdvHotTable& T : hot) {
        const int t0 = cell.pre_host[T.base], t1 = cell.pre_host[T.base + T.n];
        if (t1 <= t0) continue;
        k_advect_scalar_batch<<<t1 - t0, b, 0, s>>>(cell, T, vcur, scur, t0, t1);  // one CTA per tile
        lc.n++;
    }
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
