// Device helpers of the semi-Lagrangian advection, shared by the forward
// kernels (kernels_advect.cu) and their reverse mode (kernels_adjoint.cu).
// Internal header.
#pragma once

#include "zqs_internal.h"

namespace zqs {

struct Ax {
    int i0, i1;
    float t;
};

// Clamp-to-edge linear filter along one axis; g in texel-index units.  g is
// clamped to [0, n-1] first (NaN -> 0): outside that range clamp-to-edge
// filtering returns the edge texel, which the clamped coordinate gives with
// t = 0 (or with i0 == i1), so only i1 needs a bound.
__device__ __forceinline__ Ax axis(float g, int n) {
    g = fminf(fmaxf(g, 0.0f), (float)(n - 1));
    const float f = floorf(g);
    Ax a;
    a.t = g - f;
    a.i0 = (int)f;
    a.i1 = min(a.i0 + 1, n - 1);
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
__device__ __forceinline__ float3 tri4(const float4* __restrict__ f, const Corners& c);
__device__ __forceinline__ float tri4c(const float4* __restrict__ f4, int q, const Corners& c) {
    const float* f = reinterpret_cast<const float*>(f4);
    auto at = [&](int o) -> float { return __ldg(f + (size_t)o * 4 + q); };
    float c00 = lerpf(at(c.r00 + c.i0), at(c.r00 + c.i1), c.tx);
    float c10 = lerpf(at(c.r10 + c.i0), at(c.r10 + c.i1), c.tx);
    float c01 = lerpf(at(c.r01 + c.i0), at(c.r01 + c.i1), c.tx);
    float c11 = lerpf(at(c.r11 + c.i0), at(c.r11 + c.i1), c.tx);
    return lerpf(lerpf(c00, c10, c.ty), lerpf(c01, c11, c.ty), c.tz);
}

// Forward-only trilinear sample with the upper corners at lower + 1 along
// every axis, unclamped: one base offset plus {0, 1, px, plane} combinations.
// axis() leaves i1 != i0 + 1 only at the upper edge, where t is exactly 0, and
// the padded layout keeps that neighbour in bounds (padding column or row,
// the next row or plane, or the trailing guard plane) and finite, so the value
// equals the clamp-to-edge sample (up to the sign of an exact zero).
struct Tri0 {
    int r;
    float tx, ty, tz;
};
__device__ __forceinline__ Tri0 tri0(const Layout& L, int nx, int ny, int nz, float gx, float gy, float gz) {
    const Ax ax = axis(gx, nx), ay = axis(gy, ny), az = axis(gz, nz);
    Tri0 c;
    c.r = (az.i0 * L.py + ay.i0) * L.px + ax.i0;
    c.tx = ax.t;
    c.ty = ay.t;
    c.tz = az.t;
    return c;
}
// x, then y, then z; each corner times scale first (attenuation folding).
__device__ __forceinline__ float tri0_sample(const float* __restrict__ f, const Layout& L, const Tri0& c,
                                             float scale) {
    const float* p = f + c.r;
    const int px = L.px, pl = (int)L.plane;
    const float c00 = lerpf(__ldg(p) * scale, __ldg(p + 1) * scale, c.tx);
    const float c10 = lerpf(__ldg(p + px) * scale, __ldg(p + px + 1) * scale, c.tx);
    const float c01 = lerpf(__ldg(p + pl) * scale, __ldg(p + pl + 1) * scale, c.tx);
    const float c11 = lerpf(__ldg(p + pl + px) * scale, __ldg(p + pl + px + 1) * scale, c.tx);
    return lerpf(lerpf(c00, c10, c.ty), lerpf(c01, c11, c.ty), c.tz);
}
__device__ __forceinline__ float tri0_sample(const float* __restrict__ f, const Layout& L, const Tri0& c) {
    const float* p = f + c.r;
    const int px = L.px, pl = (int)L.plane;
    const float c00 = lerpf(__ldg(p), __ldg(p + 1), c.tx);
    const float c10 = lerpf(__ldg(p + px), __ldg(p + px + 1), c.tx);
    const float c01 = lerpf(__ldg(p + pl), __ldg(p + pl + 1), c.tx);
    const float c11 = lerpf(__ldg(p + pl + px), __ldg(p + pl + px + 1), c.tx);
    return lerpf(lerpf(c00, c10, c.ty), lerpf(c01, c11, c.ty), c.tz);
}

// Quad copy of a face component for the forward sampler:
//   Q[r] = (f[r], f[r + plane], f[r + 1], f[r + plane + 1])
// so the eight corners of tri0_sample at base r are the two 16-byte loads
// Q[r] and Q[r + px]; the interpolation tree is tri0_sample's.  Q is built for
// every face index (i <= W, j <= H, k <= D) and zero elsewhere; Q[r + px] at
// j = H lies in the next plane's first row, or in the zero tail after the
// last face plane, and enters only with weight ty = 0.
//
// The x and y steps pair two interpolations each on the Blackwell FP32x2
// instructions: the differences and the products are packed (sub/mul
// .rn.f32x2), the final sums stay scalar (__fadd_rn).  A packed multiply
// followed by a packed add is contracted into a packed fma by the assembler,
// which would round once instead of twice; scalar adds of the product's
// halves are not, so every value is the separately rounded a + t*(b - a) of
// lerpf, bit for bit.
__device__ __forceinline__ unsigned long long pack2(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 unpack2(unsigned long long r) {
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
// (t0 * (b0 - a0), t1 * (b1 - a1)), each rounded once per operation
__device__ __forceinline__ float2 lerp_step2(float a0, float a1, float b0, float b1, float t0, float t1) {
    unsigned long long d, m;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pack2(b0, b1)), "l"(pack2(a0, a1)));
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(m) : "l"(pack2(t0, t1)), "l"(d));
    return unpack2(m);
}

// x, then y, then z per component as in tri(); the x and y components go
// through the packed sub/mul of lerp_step2 (same roundings), z stays scalar.
__device__ __forceinline__ float3 tri4(const float4* __restrict__ f, const Corners& c) {
    const float4 a00 = __ldg(f + c.r00 + c.i0), b00 = __ldg(f + c.r00 + c.i1);
    const float4 a10 = __ldg(f + c.r10 + c.i0), b10 = __ldg(f + c.r10 + c.i1);
    const float4 a01 = __ldg(f + c.r01 + c.i0), b01 = __ldg(f + c.r01 + c.i1);
    const float4 a11 = __ldg(f + c.r11 + c.i0), b11 = __ldg(f + c.r11 + c.i1);
    // along x: (x, y) packed, z scalar
    auto lx = [&](const float4& a, const float4& b, float& ox, float& oy, float& oz) {
        const float2 m = lerp_step2(a.x, a.y, b.x, b.y, c.tx, c.tx);
        ox = __fadd_rn(a.x, m.x);
        oy = __fadd_rn(a.y, m.y);
        oz = lerpf(a.z, b.z, c.tx);
    };
    float x00, y00, z00, x10, y10, z10, x01, y01, z01, x11, y11, z11;
    lx(a00, b00, x00, y00, z00);
    lx(a10, b10, x10, y10, z10);
    lx(a01, b01, x01, y01, z01);
    lx(a11, b11, x11, y11, z11);
    // along y
    const float2 m0 = lerp_step2(x00, y00, x10, y10, c.ty, c.ty);
    const float2 m1 = lerp_step2(x01, y01, x11, y11, c.ty, c.ty);
    const float x0 = __fadd_rn(x00, m0.x), y0 = __fadd_rn(y00, m0.y), z0 = lerpf(z00, z10, c.ty);
    const float x1 = __fadd_rn(x01, m1.x), y1 = __fadd_rn(y01, m1.y), z1 = lerpf(z01, z11, c.ty);
    // along z
    const float2 mz = lerp_step2(x0, y0, x1, y1, c.tz, c.tz);
    float3 r;
    r.x = __fadd_rn(x0, mz.x);
    r.y = __fadd_rn(y0, mz.y);
    r.z = lerpf(z0, z1, c.tz);
    return r;
}
// tri0_quad on the two quads already loaded (a = Q[r], b = Q[r + px]).
__device__ __forceinline__ float tri0_quad_ab(const float4& a, const float4& b, const Tri0& c) {
    const float2 ma = lerp_step2(a.x, a.y, a.z, a.w, c.tx, c.tx);
    const float2 mb = lerp_step2(b.x, b.y, b.z, b.w, c.tx, c.tx);
    const float c00 = __fadd_rn(a.x, ma.x), c01 = __fadd_rn(a.y, ma.y);  // lerpf(a.x, a.z), lerpf(a.y, a.w)
    const float c10 = __fadd_rn(b.x, mb.x), c11 = __fadd_rn(b.y, mb.y);  // lerpf(b.x, b.z), lerpf(b.y, b.w)
    const float2 my = lerp_step2(c00, c01, c10, c11, c.ty, c.ty);
    const float c0 = __fadd_rn(c00, my.x), c1 = __fadd_rn(c01, my.y);  // lerpf(c00, c10), lerpf(c01, c11)
    return lerpf(c0, c1, c.tz);
}
__device__ __forceinline__ float tri0_quad(const float4* __restrict__ q, const Layout& L, const Tri0& c) {
    return tri0_quad_ab(__ldg(q + c.r), __ldg(q + c.r + L.px), c);
}

// Corner fetch policies of the MAC sampler: the field itself, or its quads.
struct FieldTri {
    const float* f;
    __device__ __forceinline__ float operator()(const Layout& L, const Tri0& c) const {
        return tri0_sample(f, L, c);
    }
};
struct QuadTri {
    const float4* q;
    __device__ __forceinline__ float operator()(const Layout& L, const Tri0& c) const { return tri0_quad(q, L, c); }
};

// NEG samples the negated field (the BFECC backward pass); negation is exact
// and commutes with the interpolation, so this equals sampling -u, -v, -w.
template <class Tri, bool NEG = false>
struct MacVelT {
    Layout L;
    Tri u, v, w;
    __device__ __forceinline__ void operator()(float px, float py, float pz, float& vx, float& vy, float& vz) const {
        vx = u(L, tri0(L, L.W + 1, L.H, L.D, px, py - 0.5f, pz - 0.5f));
        vy = v(L, tri0(L, L.W, L.H + 1, L.D, px - 0.5f, py, pz - 0.5f));
        vz = w(L, tri0(L, L.W, L.H, L.D + 1, px - 0.5f, py - 0.5f, pz));
        if (NEG) {
            vx = -vx;
            vy = -vy;
            vz = -vz;
        }
    }
    // Also returns the cell containing the point when it lies in the domain:
    // the u grid's x corner floor(clamp(x, 0, W)), the v grid's y and the w
    // grid's z corners, bounded by the last cell (x = W lies in cell W-1).
    __device__ __forceinline__ void operator()(float px, float py, float pz, float& vx, float& vy, float& vz,
                                               int& ci, int& cj, int& ck) const {
        const Ax xu = axis(px, L.W + 1), xc = axis(px - 0.5f, L.W);
        const Ax yv = axis(py, L.H + 1), yc = axis(py - 0.5f, L.H);
        const Ax zw = axis(pz, L.D + 1), zc = axis(pz - 0.5f, L.D);
        const int rcc = zc.i0 * L.py;  // plane row of the cell-centred z corner
        Tri0 cu, cv, cw;
        cu.r = (rcc + yc.i0) * L.px + xu.i0;
        cu.tx = xu.t;
        cu.ty = yc.t;
        cu.tz = zc.t;
        cv.r = (rcc + yv.i0) * L.px + xc.i0;
        cv.tx = xc.t;
        cv.ty = yv.t;
        cv.tz = zc.t;
        cw.r = (zw.i0 * L.py + yc.i0) * L.px + xc.i0;
        cw.tx = xc.t;
        cw.ty = yc.t;
        cw.tz = zw.t;
        vx = u(L, cu);
        vy = v(L, cv);
        vz = w(L, cw);
        if (NEG) {
            vx = -vx;
            vy = -vy;
            vz = -vz;
        }
        ci = min(xu.i0, L.W - 1);
        cj = min(yv.i0, L.H - 1);
        ck = min(zw.i0, L.D - 1);
    }
};
// MacVelT<QuadTri> that keeps each component's last two quads (and the last
// occupancy byte) in registers: while a backtrace stays inside the same
// interpolation cells from one substep to the next (everywhere the flow moves
// less than a cell per step) the samples reuse them instead of gathering
// through L1 again.  Same values into the same arithmetic: bit-identical to
// MacVelT<QuadTri>.  One instance per thread and backtrace.
template <bool NEG = false>
struct MacVelQC {
    Layout L;
    const float4 *qu, *qv, *qw;
    int ru = -1, rv = -1, rw = -1, rf = -1;
    float4 au, bu, av, bv, aw, bw;
    uint8_t fl = 0;
    __device__ __forceinline__ MacVelQC(const Layout& L_, const float4* u, const float4* v, const float4* w)
        : L(L_), qu(u), qv(v), qw(w) {}
    __device__ __forceinline__ void operator()(float px, float py, float pz, float& vx, float& vy, float& vz,
                                               int& ci, int& cj, int& ck) {
        const Ax xu = axis(px, L.W + 1), xc = axis(px - 0.5f, L.W);
        const Ax yv = axis(py, L.H + 1), yc = axis(py - 0.5f, L.H);
        const Ax zw = axis(pz, L.D + 1), zc = axis(pz - 0.5f, L.D);
        const int rcc = zc.i0 * L.py;
        Tri0 cu, cv, cw;
        cu.r = (rcc + yc.i0) * L.px + xu.i0;
        cu.tx = xu.t;
        cu.ty = yc.t;
        cu.tz = zc.t;
        cv.r = (rcc + yv.i0) * L.px + xc.i0;
        cv.tx = xc.t;
        cv.ty = yv.t;
        cv.tz = zc.t;
        cw.r = (zw.i0 * L.py + yc.i0) * L.px + xc.i0;
        cw.tx = xc.t;
        cw.ty = yc.t;
        cw.tz = zw.t;
        if (cu.r != ru) {
            ru = cu.r;
            au = __ldg(qu + ru);
            bu = __ldg(qu + ru + L.px);
        }
        if (cv.r != rv) {
            rv = cv.r;
            av = __ldg(qv + rv);
            bv = __ldg(qv + rv + L.px);
        }
        if (cw.r != rw) {
            rw = cw.r;
            aw = __ldg(qw + rw);
            bw = __ldg(qw + rw + L.px);
        }
        vx = tri0_quad_ab(au, bu, cu);
        vy = tri0_quad_ab(av, bv, cv);
        vz = tri0_quad_ab(aw, bw, cw);
        if (NEG) {
            vx = -vx;
            vy = -vy;
            vz = -vz;
        }
        ci = min(xu.i0, L.W - 1);
        cj = min(yv.i0, L.H - 1);
        ck = min(zw.i0, L.D - 1);
    }
    __device__ __forceinline__ void operator()(float px, float py, float pz, float& vx, float& vy, float& vz) {
        int ci, cj, ck;
        (*this)(px, py, pz, vx, vy, vz, ci, cj, ck);
    }
    // tri0_quad of component comp (quad copy q) at c, from the cache when
    // its last sample of that component had the same base
    __device__ __forceinline__ float sample(int comp, const float4* __restrict__ q, const Tri0& c) const {
        if (comp == 0 && c.r == ru) return tri0_quad_ab(au, bu, c);
        if (comp == 1 && c.r == rv) return tri0_quad_ab(av, bv, c);
        if (comp == 2 && c.r == rw) return tri0_quad_ab(aw, bw, c);
        return tri0_quad(q, L, c);
    }
    // occupancy byte of cell (i, j, k), reloaded only when the cell changes
    __device__ __forceinline__ uint8_t flag(const uint8_t* __restrict__ flags, int i, int j, int k) {
        const int c = lidx(L, i, j, k);
        if (c != rf) {
            rf = c;
            fl = __ldg(flags + c);
        }
        return fl;
    }
};

using MacVel = MacVelT<FieldTri>;   // corners from the fields
using MacVelQ = MacVelT<QuadTri>;   // corners from the quad copies
template <bool NEG = false>
struct RegVelT {
    Layout L;
    const float4* vel4;
    __device__ __forceinline__ void operator()(float px, float py, float pz, float& vx, float& vy, float& vz) const {
        float3 r = tri4(vel4, corners(L, L.W, L.H, L.D, px - 0.5f, py - 0.5f, pz - 0.5f));
        vx = NEG ? -r.x : r.x;
        vy = NEG ? -r.y : r.y;
        vz = NEG ? -r.z : r.z;
    }
};
using RegVel = RegVelT<false>;

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

// backtrace() for the MAC sampler: the occupancy test reuses the cell index
// that the velocity sample at the same point already floored.
template <class Tri, bool NEG>
__device__ __forceinline__ void backtrace(const Layout& L, const uint8_t* __restrict__ flags,
                                          const MacVelT<Tri, NEG>& vel, const KParams& kp, float& px, float& py,
                                          float& pz) {
    float vx, vy, vz;
    int ci, cj, ck;
    vel(px, py, pz, vx, vy, vz, ci, cj, ck);
    float lx = px, ly = py, lz = pz;
    const float Wf = (float)L.W, Hf = (float)L.H, Df = (float)L.D;
    auto inside = [&](float x, float y, float z) -> bool {
        return x >= 0.0f && x <= Wf && y >= 0.0f && y <= Hf && z >= 0.0f && z <= Df;
    };
    const float dt = kp.dt_sub;
    int istep = 0;
    bool broke = false;
    do {
        if (!inside(px, py, pz) || !(__ldg(flags + lidx(L, ci, cj, ck)) & F_FREE)) {
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
        if (istep < kp.substeps) vel(px, py, pz, vx, vy, vz, ci, cj, ck);
    } while (istep < kp.substeps);
    if (kp.full && !broke && inside(px, py, pz)) {
        const int i = min((int)floorf(px), L.W - 1), j = min((int)floorf(py), L.H - 1);
        const int k = min((int)floorf(pz), L.D - 1);
        if (__ldg(flags + lidx(L, i, j, k)) & F_FREE) {
            lx = px;
            ly = py;
            lz = pz;
        }
    }
    px = lx;
    py = ly;
    pz = lz;
}

// backtrace() for the caching MAC sampler: the same loop as above, the
// occupancy test through the sampler's cached byte.
template <bool NEG>
__device__ __forceinline__ void backtrace(const Layout& L, const uint8_t* __restrict__ flags, MacVelQC<NEG>& vel,
                                          const KParams& kp, float& px, float& py, float& pz) {
    float vx, vy, vz;
    int ci, cj, ck;
    vel(px, py, pz, vx, vy, vz, ci, cj, ck);
    float lx = px, ly = py, lz = pz;
    const float Wf = (float)L.W, Hf = (float)L.H, Df = (float)L.D;
    auto inside = [&](float x, float y, float z) -> bool {
        return x >= 0.0f && x <= Wf && y >= 0.0f && y <= Hf && z >= 0.0f && z <= Df;
    };
    const float dt = kp.dt_sub;
    int istep = 0;
    bool broke = false;
    do {
        if (!inside(px, py, pz) || !(vel.flag(flags, ci, cj, ck) & F_FREE)) {
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
        if (istep < kp.substeps) vel(px, py, pz, vx, vy, vz, ci, cj, ck);
    } while (istep < kp.substeps);
    if (kp.full && !broke && inside(px, py, pz)) {
        const int i = min((int)floorf(px), L.W - 1), j = min((int)floorf(py), L.H - 1);
        const int k = min((int)floorf(pz), L.D - 1);
        if (vel.flag(flags, i, j, k) & F_FREE) {
            lx = px;
            ly = py;
            lz = pz;
        }
    }
    px = lx;
    py = ly;
    pz = lz;
}

__device__ __forceinline__ bool face_live(uint8_t fl, uint8_t bit, int idx, int n, bool open) {
    if (!(fl & bit)) return false;
    return open || (idx > 0 && idx < n);
}

}  // namespace zqs
