/*
 * zqs_oracle.cpp -- CPU ORACLE for the 3D smoke step.  TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C++ templated on the arithmetic type R
 * (float or double), the per-timestep path of ZQ_SmokeSimulation3D as the
 * reference computes it.  It is the checker for the CUDA library: only the
 * tests, the smoke check and bench.py's CPU-baseline / reference arm may load
 * it.  Nothing in the product links or calls it.
 *
 * Parity status: UNPINNED by the reference.  The reference ships no tests or
 * golden outputs, cannot be built here (Windows/VS2015, legacy texture
 * references, missing ZQlib/ZQlibCuda), and its SOR solver lives in the
 * un-vendored ZQlibCuda library; see the per-function citations for the
 * in-tree evidence each rule is restated from.
 *
 * Arithmetic contract (shared with the CUDA kernels so FP32 results can match
 * bit for bit): no contraction (built with -ffp-contract=off; kernels with
 * -fmad=false), IEEE division and square root, and the association order
 * written out explicitly in every expression below.  Hardware texture
 * filtering of the reference (9-bit weights) is replaced by exact trilinear
 * interpolation lerp(a,b,t) = a + t*(b-a), x then y then z.
 *
 * Layout: unpadded reference layouts, x fastest
 *   cell (i,j,k)  ((k*H)+j)*W + i          u (i<=W) ((k*H)+j)*(W+1) + i
 *   v (j<=H)      ((k*(H+1))+j)*W + i      w (k<=D) ((k*H)+j)*W + i
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/zqs_capi.h"

namespace zqo {

struct Dims {
    int W, H, D;
    size_t cell(int i, int j, int k) const { return ((size_t)k * H + j) * W + i; }
    size_t uix(int i, int j, int k) const { return ((size_t)k * H + j) * (W + 1) + i; }
    size_t vix(int i, int j, int k) const { return ((size_t)k * (H + 1) + j) * W + i; }
    size_t wix(int i, int j, int k) const { return ((size_t)k * H + j) * W + i; }
    size_t ncell() const { return (size_t)W * H * D; }
    size_t nu() const { return (size_t)(W + 1) * H * D; }
    size_t nv() const { return (size_t)W * (H + 1) * D; }
    size_t nw() const { return (size_t)W * H * (D + 1); }
};

static inline int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

template <class R> static inline R lerp(R a, R b, R t) { return a + t * (b - a); }

/* One axis of clamp-to-edge linear filtering: the coordinate g is in texel
 * index units (texel n has its centre at g = n).  g is first clamped to
 * [-1, n] (which does not change the filtered value and makes NaN/inf safe:
 * fmax/fmin return the non-NaN operand), then split into floor and fraction.
 * Mirrors cudaAddressModeClamp + cudaFilterModeLinear of the reference's
 * textures (ZQ_CUDA_Advection3D.cu:654-993). */
template <class R> struct Axis {
    int i0, i1;
    R t;
};
template <class R> static inline Axis<R> axis(R g, int n) {
    g = std::fmin(std::fmax(g, R(-1)), R(n));
    R f = std::floor(g);
    Axis<R> a;
    a.t = g - f;
    int i = (int)f;
    a.i0 = clampi(i, 0, n - 1);
    a.i1 = clampi(i + 1, 0, n - 1);
    return a;
}

/* Trilinear sample of a field with dims nx*ny*nz, element (i,j,k) at
 * base[(((size_t)k*ny)+j)*nx + i)*stride + comp]. */
template <class R, class S>
static inline R trilinear(const S* base, int nx, int ny, int nz, int stride, int comp, R gx, R gy, R gz) {
    Axis<R> ax = axis(gx, nx), ay = axis(gy, ny), az = axis(gz, nz);
    auto at = [&](int i, int j, int k) -> R {
        return (R)base[((((size_t)k * ny) + j) * nx + i) * stride + comp];
    };
    R c00 = lerp(at(ax.i0, ay.i0, az.i0), at(ax.i1, ay.i0, az.i0), ax.t);
    R c10 = lerp(at(ax.i0, ay.i1, az.i0), at(ax.i1, ay.i1, az.i0), ax.t);
    R c01 = lerp(at(ax.i0, ay.i0, az.i1), at(ax.i1, ay.i0, az.i1), ax.t);
    R c11 = lerp(at(ax.i0, ay.i1, az.i1), at(ax.i1, ay.i1, az.i1), ax.t);
    R c0 = lerp(c00, c10, ay.t);
    R c1 = lerp(c01, c11, ay.t);
    return lerp(c0, c1, az.t);
}

/* ---------------------------------------------------------------------- */
/* MAC <-> cell-centre velocity                                            */
/* ---------------------------------------------------------------------- */

/* ZQ_CUDA_MACtoRegular.cu:9-27 (MAC_to_Regular4_Kernel): centre = 0.5*(lo+hi). */
template <class R>
void mac_to_regular4(const Dims& d, const R* u, const R* v, const R* w, R* vel4) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < d.D; k++)
        for (int j = 0; j < d.H; j++)
            for (int i = 0; i < d.W; i++) {
                size_t c = d.cell(i, j, k);
                vel4[c * 4 + 0] = R(0.5) * (u[d.uix(i, j, k)] + u[d.uix(i + 1, j, k)]);
                vel4[c * 4 + 1] = R(0.5) * (v[d.vix(i, j, k)] + v[d.vix(i, j + 1, k)]);
                vel4[c * 4 + 2] = R(0.5) * (w[d.wix(i, j, k)] + w[d.wix(i, j, k + 1)]);
                vel4[c * 4 + 3] = R(0);
            }
}

/* ZQ_CUDA_MACtoRegular.cu:29-99 (Regular4_to_MAC_{u,v,w}_Kernel): interior
 * faces average the two cells, domain faces copy the inner cell.  (The CPU
 * Regular4toMAC of Utils3D:377-416 writes mac_v at x=W instead of mac_u; the
 * GPU semantics are the intended ones and are followed here.) */
template <class R>
void regular4_to_mac(const Dims& d, const R* vel4, R* u, R* v, R* w) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < d.D; k++)
        for (int j = 0; j < d.H; j++)
            for (int i = 0; i <= d.W; i++) {
                R val;
                if (i == 0) val = vel4[d.cell(0, j, k) * 4 + 0];
                else if (i == d.W) val = vel4[d.cell(d.W - 1, j, k) * 4 + 0];
                else val = R(0.5) * (vel4[d.cell(i, j, k) * 4 + 0] + vel4[d.cell(i - 1, j, k) * 4 + 0]);
                u[d.uix(i, j, k)] = val;
            }
#pragma omp parallel for schedule(static)
    for (int k = 0; k < d.D; k++)
        for (int j = 0; j <= d.H; j++)
            for (int i = 0; i < d.W; i++) {
                R val;
                if (j == 0) val = vel4[d.cell(i, 0, k) * 4 + 1];
                else if (j == d.H) val = vel4[d.cell(i, d.H - 1, k) * 4 + 1];
                else val = R(0.5) * (vel4[d.cell(i, j, k) * 4 + 1] + vel4[d.cell(i, j - 1, k) * 4 + 1]);
                v[d.vix(i, j, k)] = val;
            }
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= d.D; k++)
        for (int j = 0; j < d.H; j++)
            for (int i = 0; i < d.W; i++) {
                R val;
                if (k == 0) val = vel4[d.cell(i, j, 0) * 4 + 2];
                else if (k == d.D) val = vel4[d.cell(i, j, d.D - 1) * 4 + 2];
                else val = R(0.5) * (vel4[d.cell(i, j, k) * 4 + 2] + vel4[d.cell(i, j, k - 1) * 4 + 2]);
                w[d.wix(i, j, k)] = val;
            }
}

/* ---------------------------------------------------------------------- */
/* Face masks shared by force, attenuation and the advection write-back   */
/* ---------------------------------------------------------------------- */

/* Open rule (ZQ_CUDA_Advection3D.cu:471-575, ZQ_CUDA_AddForce3D.cu:211-385,
 * ZQ_CUDA_Attenuation3D.cu:8-98): an interior face is live when both cells
 * are free, a domain face when its inner cell is free.  Closed rule
 * (ZQ_CUDA_Advection3D.cu:577-650): domain faces are never written. */
static inline bool u_live(const Dims& d, const uint8_t* occ, int i, int j, int k, bool open) {
    if (i == 0) return open && !occ[d.cell(0, j, k)];
    if (i == d.W) return open && !occ[d.cell(d.W - 1, j, k)];
    return !occ[d.cell(i, j, k)] && !occ[d.cell(i - 1, j, k)];
}
static inline bool v_live(const Dims& d, const uint8_t* occ, int i, int j, int k, bool open) {
    if (j == 0) return open && !occ[d.cell(i, 0, k)];
    if (j == d.H) return open && !occ[d.cell(i, d.H - 1, k)];
    return !occ[d.cell(i, j, k)] && !occ[d.cell(i, j - 1, k)];
}
static inline bool w_live(const Dims& d, const uint8_t* occ, int i, int j, int k, bool open) {
    if (k == 0) return open && !occ[d.cell(i, j, 0)];
    if (k == d.D) return open && !occ[d.cell(i, j, d.D - 1)];
    return !occ[d.cell(i, j, k)] && !occ[d.cell(i, j, k - 1)];
}

/* ApplyAdvectVelocityResult (Utils3D:419-474; GPU Adv3D:471-650). */
template <class R>
void apply_advect_result(const Dims& d, const uint8_t* occ, const R* au, const R* av, const R* aw,
                         R* u, R* v, R* w, bool open) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= d.D; k++)
        for (int j = 0; j <= d.H; j++)
            for (int i = 0; i <= d.W; i++) {
                if (j < d.H && k < d.D && u_live(d, occ, i, j, k, open)) u[d.uix(i, j, k)] = au[d.uix(i, j, k)];
                if (i < d.W && k < d.D && v_live(d, occ, i, j, k, open)) v[d.vix(i, j, k)] = av[d.vix(i, j, k)];
                if (i < d.W && j < d.H && w_live(d, occ, i, j, k, open)) w[d.wix(i, j, k)] = aw[d.wix(i, j, k)];
            }
}

/* ---------------------------------------------------------------------- */
/* Forces: vorticity confinement + buoyancy (+ density weight)            */
/* ---------------------------------------------------------------------- */

/* cu_AddForce3D (ZQ_CUDA_AddForce3D.cu:510-556):
 *  1. cell-centre velocity (cu_MAC_to_Regular_vel, restated as MAC_to_Regular4)
 *  2. vorticity on cells with every index in [1,N-2], zero elsewhere (:11-34):
 *       wx = (((w[y+1]-w[y-1]) - v[z+1]) + v[z-1]) / (2h)   (centre values)
 *       wy = (((u[z+1]-u[z-1]) - w[x+1]) + w[x-1]) / (2h)
 *       wz = (((v[x+1]-v[x-1]) - u[y+1]) + u[y-1]) / (2h)
 *       |w| = sqrt((wx*wx + wy*wy) + wz*wz)
 *  3. N = grad|w| (0.5*central inside, one-sided on the domain boundary),
 *     normalised when its length is nonzero (:64-111)
 *  4. f = (eps*h)*(N x w);  f_y += beta*(T - Tamb);  f_y -= alpha*rho (:161-184;
 *     the alpha term is an addition of this build, alpha = 0 reproduces it)
 *  5. faces: u += (dt*0.5)*(f_R + f_L) when both cells are free, u += dt*f_in on
 *     domain faces whose inner cell is free (:211-385; the w kernel at :360-385
 *     reads occupy[-1 plane] for z=0, its per-slice twin :387-420 is followed). */
/* Vorticity (wx, wy, wz) and |w| of the cell-centre velocity, nonzero only on
 * cells with every index in [1,N-2] (ZQ_CUDA_AddForce3D.cu:11-34). */
template <class R>
void vorticity(const Dims& d, const R* u, const R* v, const R* w, R h, R* vort, R* vs) {
    const size_t n = d.ncell();
    const int W = d.W, H = d.H, D = d.D;
    const size_t sy = (size_t)W, sz = (size_t)W * H;
    std::vector<R> vel4(n * 4);
    mac_to_regular4(d, u, v, w, vel4.data());
    std::fill(vort, vort + n * 3, R(0));
    std::fill(vs, vs + n, R(0));
    const R twoh = R(2) * h;
#pragma omp parallel for schedule(static)
    for (int k = 1; k < D - 1; k++)
        for (int j = 1; j < H - 1; j++)
            for (int i = 1; i < W - 1; i++) {
                size_t c = d.cell(i, j, k);
                auto U = [&](size_t o) { return vel4[o * 4 + 0]; };
                auto V = [&](size_t o) { return vel4[o * 4 + 1]; };
                auto Wc = [&](size_t o) { return vel4[o * 4 + 2]; };
                R ox = (((Wc(c + sy) - Wc(c - sy)) - V(c + sz)) + V(c - sz)) / twoh;
                R oy = (((U(c + sz) - U(c - sz)) - Wc(c + 1)) + Wc(c - 1)) / twoh;
                R oz = (((V(c + 1) - V(c - 1)) - U(c + sy)) + U(c - sy)) / twoh;
                vort[c * 3 + 0] = ox;
                vort[c * 3 + 1] = oy;
                vort[c * 3 + 2] = oz;
                vs[c] = std::sqrt((ox * ox + oy * oy) + oz * oz);
            }
}

template <class R>
void add_force(const Dims& d, R* u, R* v, R* w, const uint8_t* occ, const R* T, const R* rho,
               const zqs_params& P) {
    const size_t n = d.ncell();
    const int W = d.W, H = d.H, D = d.D;
    const size_t sy = (size_t)W, sz = (size_t)W * H;
    std::vector<R> vort(n * 3, R(0)), vs(n, R(0)), grad(n * 3, R(0)), force(n * 3, R(0));
    const R h = (R)P.voxel_size;
    vorticity(d, u, v, w, h, vort.data(), vs.data());
#pragma omp parallel for schedule(static)
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                size_t c = d.cell(i, j, k);
                R gx, gy, gz;
                if (i == 0) gx = vs[c + 1] - vs[c];
                else if (i == W - 1) gx = vs[c] - vs[c - 1];
                else gx = R(0.5) * (vs[c + 1] - vs[c - 1]);
                if (j == 0) gy = vs[c + sy] - vs[c];
                else if (j == H - 1) gy = vs[c] - vs[c - sy];
                else gy = R(0.5) * (vs[c + sy] - vs[c - sy]);
                if (k == 0) gz = vs[c + sz] - vs[c];
                else if (k == D - 1) gz = vs[c] - vs[c - sz];
                else gz = R(0.5) * (vs[c + sz] - vs[c - sz]);
                R len = std::sqrt((gx * gx + gy * gy) + gz * gz);
                if (len != R(0)) {
                    gx = gx / len;
                    gy = gy / len;
                    gz = gz / len;
                }
                grad[c * 3 + 0] = gx;
                grad[c * 3 + 1] = gy;
                grad[c * 3 + 2] = gz;
            }
    const R cc = (R)P.confine * h;
    const R beta = (R)P.buoyancy, alpha = (R)P.gravity, tamb = (R)P.tamb;
#pragma omp parallel for schedule(static)
    for (size_t c = 0; c < n; c++) {
        R gx = grad[c * 3 + 0], gy = grad[c * 3 + 1], gz = grad[c * 3 + 2];
        R ox = vort[c * 3 + 0], oy = vort[c * 3 + 1], oz = vort[c * 3 + 2];
        R fx = cc * (gy * oz - gz * oy);
        R fy = cc * (gz * ox - gx * oz);
        R fz = cc * (gx * oy - gy * ox);
        fy = fy + beta * (T[c] - tamb);
        fy = fy - alpha * rho[c];
        force[c * 3 + 0] = fx;
        force[c * 3 + 1] = fy;
        force[c * 3 + 2] = fz;
    }
    const R dt = (R)P.step_time;
    const R hdt = dt * R(0.5);
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= D; k++)
        for (int j = 0; j <= H; j++)
            for (int i = 0; i <= W; i++) {
                if (j < H && k < D && u_live(d, occ, i, j, k, true)) {
                    R& f = u[d.uix(i, j, k)];
                    if (i == 0) f = f + dt * force[d.cell(0, j, k) * 3 + 0];
                    else if (i == W) f = f + dt * force[d.cell(W - 1, j, k) * 3 + 0];
                    else f = f + hdt * (force[d.cell(i, j, k) * 3 + 0] + force[d.cell(i - 1, j, k) * 3 + 0]);
                }
                if (i < W && k < D && v_live(d, occ, i, j, k, true)) {
                    R& f = v[d.vix(i, j, k)];
                    if (j == 0) f = f + dt * force[d.cell(i, 0, k) * 3 + 1];
                    else if (j == H) f = f + dt * force[d.cell(i, H - 1, k) * 3 + 1];
                    else f = f + hdt * (force[d.cell(i, j, k) * 3 + 1] + force[d.cell(i, j - 1, k) * 3 + 1]);
                }
                if (i < W && j < H && w_live(d, occ, i, j, k, true)) {
                    R& f = w[d.wix(i, j, k)];
                    if (k == 0) f = f + dt * force[d.cell(i, j, 0) * 3 + 2];
                    else if (k == D) f = f + dt * force[d.cell(i, j, D - 1) * 3 + 2];
                    else f = f + hdt * (force[d.cell(i, j, k) * 3 + 2] + force[d.cell(i, j, k - 1) * 3 + 2]);
                }
            }
}

/* Attenuation3D (ZQ_CUDA_Attenuation3D.cu:8-116; factors from Utils3D:2098-2100):
 * live faces (open rule) times vel_atten, every cell's T and rho times theirs. */
template <class R>
void attenuate(const Dims& d, R* u, R* v, R* w, R* T, R* rho, const uint8_t* occ, const zqs_params& P) {
    const R av = (R)P.vel_atten, at = (R)P.temp_atten, ad = (R)P.dens_atten;
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= d.D; k++)
        for (int j = 0; j <= d.H; j++)
            for (int i = 0; i <= d.W; i++) {
                if (j < d.H && k < d.D && u_live(d, occ, i, j, k, true)) u[d.uix(i, j, k)] = u[d.uix(i, j, k)] * av;
                if (i < d.W && k < d.D && v_live(d, occ, i, j, k, true)) v[d.vix(i, j, k)] = v[d.vix(i, j, k)] * av;
                if (i < d.W && j < d.H && w_live(d, occ, i, j, k, true)) w[d.wix(i, j, k)] = w[d.wix(i, j, k)] * av;
                if (i < d.W && j < d.H && k < d.D) {
                    size_t c = d.cell(i, j, k);
                    T[c] = T[c] * at;
                    rho[c] = rho[c] * ad;
                }
            }
}

/* ---------------------------------------------------------------------- */
/* Semi-Lagrangian advection                                              */
/* ---------------------------------------------------------------------- */

/* Velocity samplers.  MAC: u texel (i,j,k) sits at (i, j+.5, k+.5), so the
 * texel-index coordinate of a point p is (p.x, p.y-.5, p.z-.5); v and w
 * likewise (ZQ_CUDA_Advection3D.cu:244-246 normalised by W+1 etc.).
 * Regular: the float4 centre field sits at (i+.5, j+.5, k+.5). */
template <class R> struct MacSampler {
    Dims d;
    const R *u, *v, *w;
    void operator()(R px, R py, R pz, R& vx, R& vy, R& vz) const {
        const R hf = R(0.5);
        vx = trilinear<R>(u, d.W + 1, d.H, d.D, 1, 0, px, py - hf, pz - hf);
        vy = trilinear<R>(v, d.W, d.H + 1, d.D, 1, 0, px - hf, py, pz - hf);
        vz = trilinear<R>(w, d.W, d.H, d.D + 1, 1, 0, px - hf, py - hf, pz);
    }
};
template <class R> struct RegSampler {
    Dims d;
    const R* vel4;
    void operator()(R px, R py, R pz, R& vx, R& vy, R& vz) const {
        const R hf = R(0.5);
        R gx = px - hf, gy = py - hf, gz = pz - hf;
        vx = trilinear<R>(vel4, d.W, d.H, d.D, 4, 0, gx, gy, gz);
        vy = trilinear<R>(vel4, d.W, d.H, d.D, 4, 1, gx, gy, gz);
        vz = trilinear<R>(vel4, d.W, d.H, d.D, 4, 2, gx, gy, gz);
    }
};

/* The backtrace loop of every advection kernel (e.g. ZQ_CUDA_Advection3D.cu:253-273):
 *   do { if p is outside [0,W]x[0,H]x[0,D] or occupy[floor(p) clamped]: break;
 *        last = p;  p -= (vel(p)*dt_sub)/h;  vel = sample(p);  } while (++n < steps);
 * and the result is sampled at `last`, i.e. at the last point that passed the
 * test BEFORE the final move.  With backtrace_full the final point is also
 * tested and, when it passes, used. */
template <class R, class VelF>
static inline void backtrace(const Dims& d, const uint8_t* occ, const VelF& vel, int steps, R dt, R h,
                             bool full, R& px, R& py, R& pz) {
    R vx, vy, vz;
    vel(px, py, pz, vx, vy, vz);
    R lx = px, ly = py, lz = pz;
    const R Wf = (R)d.W, Hf = (R)d.H, Df = (R)d.D;
    auto ok = [&](R x, R y, R z) -> bool {
        if (!(x >= R(0) && x <= Wf && y >= R(0) && y <= Hf && z >= R(0) && z <= Df)) return false;
        int i = clampi((int)std::floor(x), 0, d.W - 1);
        int j = clampi((int)std::floor(y), 0, d.H - 1);
        int k = clampi((int)std::floor(z), 0, d.D - 1);
        return occ[d.cell(i, j, k)] == 0;
    };
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
        px = px - (vx * dt) / h;
        py = py - (vy * dt) / h;
        pz = pz - (vz * dt) / h;
        vel(px, py, pz, vx, vy, vz);
        istep++;
    } while (istep < steps);
    if (full && !broke && ok(px, py, pz)) {
        lx = px;
        ly = py;
        lz = pz;
    }
    px = lx;
    py = ly;
    pz = lz;
}

template <class R> struct AdvCtx {
    int steps;
    R dt, h;
    bool full;
};
template <class R> static AdvCtx<R> adv_ctx(const zqs_params& P) {
    AdvCtx<R> c;
    c.steps = P.substeps;
    /* deltatt = stepTime / steps, computed in float on the host (Utils3D:2155) */
    c.dt = (R)((float)P.step_time / (float)P.substeps);
    if (sizeof(R) == 8) c.dt = (R)P.step_time / (R)P.substeps;
    c.h = (R)P.voxel_size;
    c.full = P.backtrace_full != 0;
    return c;
}

/* Advect_Velocity (ZQ_CUDA_Advection3D.cu:1686-1749) for the three non-BFECC
 * modes; the write-back follows cu_Apply_Advect_Velocity_Result_{Open,Closed}. */
template <class R>
int advect_velocity(const Dims& d, R* u, R* v, R* w, const uint8_t* occ, const zqs_params& P, int mode,
                    bool open) {
    AdvCtx<R> a = adv_ctx<R>(P);
    std::vector<R> ou(d.nu(), R(0)), ov(d.nv(), R(0)), ow(d.nw(), R(0));
    const R hf = R(0.5);
    if (mode == ZQS_ADV_VEL_INMAC_OUTMAC) {
        /* Advect_Velocity_inMAC_outMAC_{u,v,w}_Kernel, Adv3D:232-377 */
        MacSampler<R> s{d, u, v, w};
#pragma omp parallel for schedule(dynamic, 1)
        for (int k = 0; k <= d.D; k++)
            for (int j = 0; j <= d.H; j++)
                for (int i = 0; i <= d.W; i++) {
                    if (j < d.H && k < d.D) {
                        R px = (R)i, py = (R)j + hf, pz = (R)k + hf;
                        backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                        ou[d.uix(i, j, k)] = trilinear<R>(u, d.W + 1, d.H, d.D, 1, 0, px, py - hf, pz - hf);
                    }
                    if (i < d.W && k < d.D) {
                        R px = (R)i + hf, py = (R)j, pz = (R)k + hf;
                        backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                        ov[d.vix(i, j, k)] = trilinear<R>(v, d.W, d.H + 1, d.D, 1, 0, px - hf, py, pz - hf);
                    }
                    if (i < d.W && j < d.H) {
                        R px = (R)i + hf, py = (R)j + hf, pz = (R)k;
                        backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                        ow[d.wix(i, j, k)] = trilinear<R>(w, d.W, d.H, d.D + 1, 1, 0, px - hf, py - hf, pz);
                    }
                }
    } else if (mode == ZQS_ADV_VEL_INREG_OUTMAC) {
        /* Advect_Velocity_inRegular_outMAC_{u,v,w}_Kernel, Adv3D:115-230 */
        std::vector<R> vel4(d.ncell() * 4);
        mac_to_regular4(d, u, v, w, vel4.data());
        RegSampler<R> s{d, vel4.data()};
#pragma omp parallel for schedule(dynamic, 1)
        for (int k = 0; k <= d.D; k++)
            for (int j = 0; j <= d.H; j++)
                for (int i = 0; i <= d.W; i++) {
                    if (j < d.H && k < d.D) {
                        R px = (R)i, py = (R)j + hf, pz = (R)k + hf;
                        backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                        ou[d.uix(i, j, k)] =
                            trilinear<R>(vel4.data(), d.W, d.H, d.D, 4, 0, px - hf, py - hf, pz - hf);
                    }
                    if (i < d.W && k < d.D) {
                        R px = (R)i + hf, py = (R)j, pz = (R)k + hf;
                        backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                        ov[d.vix(i, j, k)] =
                            trilinear<R>(vel4.data(), d.W, d.H, d.D, 4, 1, px - hf, py - hf, pz - hf);
                    }
                    if (i < d.W && j < d.H) {
                        R px = (R)i + hf, py = (R)j + hf, pz = (R)k;
                        backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                        ow[d.wix(i, j, k)] =
                            trilinear<R>(vel4.data(), d.W, d.H, d.D, 4, 2, px - hf, py - hf, pz - hf);
                    }
                }
    } else if (mode == ZQS_ADV_VEL_INREG_OUTREG) {
        /* Advect_Velocity_inRegular_outRegular_Kernel (Adv3D:76-113), then
         * Regular4_to_MAC and the write-back (Adv3D:1061-1106) */
        std::vector<R> vel4(d.ncell() * 4), out4(d.ncell() * 4);
        mac_to_regular4(d, u, v, w, vel4.data());
        RegSampler<R> s{d, vel4.data()};
#pragma omp parallel for schedule(dynamic, 1)
        for (int k = 0; k < d.D; k++)
            for (int j = 0; j < d.H; j++)
                for (int i = 0; i < d.W; i++) {
                    R px = (R)i + hf, py = (R)j + hf, pz = (R)k + hf;
                    backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                    size_t c = d.cell(i, j, k);
                    for (int q = 0; q < 3; q++)
                        out4[c * 4 + q] = trilinear<R>(vel4.data(), d.W, d.H, d.D, 4, q, px - hf, py - hf, pz - hf);
                    out4[c * 4 + 3] = R(0);
                }
        regular4_to_mac(d, out4.data(), ou.data(), ov.data(), ow.data());
    } else {
        return ZQS_EUNSUPPORTED;
    }
    apply_advect_result(d, occ, ou.data(), ov.data(), ow.data(), u, v, w, open);
    return ZQS_OK;
}

/* Advect_Scalar (Adv3D:1751-1821): backtrace from cell centres through MAC
 * (Adv3D:420-469) or regular (Adv3D:379-418) velocity, sample T and rho at the
 * final point; every cell is written, occupied ones included. */
template <class R>
int advect_scalar(const Dims& d, const R* u, const R* v, const R* w, const uint8_t* occ, const R* Tin,
                  const R* Din, R* Tout, R* Dout, const zqs_params& P, int mode) {
    AdvCtx<R> a = adv_ctx<R>(P);
    const R hf = R(0.5);
    std::vector<R> tt(d.ncell()), dd(d.ncell());
    std::vector<R> vel4;
    if (mode == ZQS_ADV_SCA_REG) {
        vel4.resize(d.ncell() * 4);
        mac_to_regular4(d, u, v, w, vel4.data());
    } else if (mode != ZQS_ADV_SCA_MAC) {
        return ZQS_EUNSUPPORTED;
    }
    MacSampler<R> ms{d, u, v, w};
    RegSampler<R> rs{d, vel4.data()};
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < d.D; k++)
        for (int j = 0; j < d.H; j++)
            for (int i = 0; i < d.W; i++) {
                R px = (R)i + hf, py = (R)j + hf, pz = (R)k + hf;
                if (mode == ZQS_ADV_SCA_MAC) backtrace(d, occ, ms, a.steps, a.dt, a.h, a.full, px, py, pz);
                else backtrace(d, occ, rs, a.steps, a.dt, a.h, a.full, px, py, pz);
                size_t c = d.cell(i, j, k);
                tt[c] = trilinear<R>(Tin, d.W, d.H, d.D, 1, 0, px - hf, py - hf, pz - hf);
                dd[c] = trilinear<R>(Din, d.W, d.H, d.D, 1, 0, px - hf, py - hf, pz - hf);
            }
    std::copy(tt.begin(), tt.end(), Tout);
    std::copy(dd.begin(), dd.end(), Dout);
    return ZQS_OK;
}

/* ZQ_ReinjectTemperatureDensity3D (Utils3D:3842-3882): cells inside a source
 * get density and temperature overwritten; sources in order, the last wins.
 * Box test |i+.5-cx| <= hx (per axis); sphere test (new in this build)
 * ((dx*dx + dy*dy) + dz*dz) <= r*r with dx = (i+.5) - cx. */
template <class R>
void reinject(const Dims& d, R* T, R* rho, const zqs_params& P) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < d.D; k++)
        for (int j = 0; j < d.H; j++)
            for (int i = 0; i < d.W; i++) {
                size_t c = d.cell(i, j, k);
                for (int s = 0; s < P.n_sources; s++) {
                    const zqs_source& S = P.sources[s];
                    float dx = ((float)i + 0.5f) - S.cx;
                    float dy = ((float)j + 0.5f) - S.cy;
                    float dz = ((float)k + 0.5f) - S.cz;
                    bool in;
                    if (S.shape == ZQS_SOURCE_SPHERE) in = ((dx * dx + dy * dy) + dz * dz) <= S.hx * S.hx;
                    else in = std::fabs(dx) <= S.hx && std::fabs(dy) <= S.hy && std::fabs(dz) <= S.hz;
                    if (in) {
                        rho[c] = (R)S.density;
                        T[c] = (R)S.temperature;
                    }
                }
            }
}

/* ---------------------------------------------------------------------- */
/* Pressure projection: fixed-K red-black SOR                              */
/* ---------------------------------------------------------------------- */

/* Restatement of ZQ_CUDA_PoissonSolver3D::Solve{Open,Closed}PoissonRedBlackwithOccupy3D_MAC,
 * whose source is not in the reference tree.  Evidence used:
 *   divergence  u[i+1]-u[i] + v[j+1]-v[j] + w[k+1]-w[k]       Utils3D:2310-2312, 2410-2412
 *   closed: subtract the mean divergence over free cells      Utils3D:2368-2440
 *   stencil weights: free in-domain neighbour 1; occupied 0;
 *     outside the domain 1 with p=0 (open) / 0 (closed)       Utils3D:476-601 (count = 6 - #in-domain), 603-747
 *   red cells (i+j+k)%2==0 first, then black                  ZQ_SmokeOctreeGrid3D.cpp:6378
 *   update p = (sum w*p_n - div) / sum w                      CPU_PoissonSolver3D_OpenOctreePoisson.cpp:401-440
 *   gradient: u -= p_R - p_L on faces between free cells, open
 *     domain faces use p=0 outside                            Utils3D:2794-2926
 * Added: over-relaxation p <- (1-omega)*p + omega*GS (omega=1 gives GS
 * exactly), cold start p=0, neighbours summed in the order x-,x+,y-,y+,z-,z+.
 * Stats: max|div| after projection and ||div - Lp||_2, both in FP64. */
template <class R>
void project(const Dims& d, R* u, R* v, R* w, const uint8_t* occ, const zqs_params& P, R* p_out,
             R* div_out, zqs_stats* st) {
    const int W = d.W, H = d.H, D = d.D;
    const size_t n = d.ncell();
    const bool open = P.solver == ZQS_SOLVER_OPEN;
    std::vector<R> div(n, R(0)), p(n, R(0));
    std::vector<R> cnt(n, R(0));
    auto divergence = [&](int i, int j, int k) -> R {
        return ((((u[d.uix(i + 1, j, k)] - u[d.uix(i, j, k)]) + v[d.vix(i, j + 1, k)]) - v[d.vix(i, j, k)]) +
                w[d.wix(i, j, k + 1)]) -
               w[d.wix(i, j, k)];
    };
#pragma omp parallel for schedule(static)
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                size_t c = d.cell(i, j, k);
                if (occ[c]) continue;
                div[c] = divergence(i, j, k);
                int nin = 0, nfree = 0;
                const int di[6] = {-1, 1, 0, 0, 0, 0}, dj[6] = {0, 0, -1, 1, 0, 0}, dk[6] = {0, 0, 0, 0, -1, 1};
                for (int q = 0; q < 6; q++) {
                    int a = i + di[q], b = j + dj[q], e = k + dk[q];
                    if (a < 0 || a >= W || b < 0 || b >= H || e < 0 || e >= D) continue;
                    nin++;
                    if (!occ[d.cell(a, b, e)]) nfree++;
                }
                cnt[c] = open ? (R)(6 - (nin - nfree)) : (R)nfree;
            }
    double mean_removed = 0.0;
    int64_t nfree_cells = 0;
    if (!open) {
        /* FP64 mean: per-plane partial sums combined in plane order */
        std::vector<double> part(D, 0.0);
        std::vector<int64_t> pc(D, 0);
#pragma omp parallel for schedule(static)
        for (int k = 0; k < D; k++) {
            double s = 0.0;
            int64_t c0 = 0;
            for (int j = 0; j < H; j++)
                for (int i = 0; i < W; i++) {
                    size_t c = d.cell(i, j, k);
                    if (occ[c]) continue;
                    s += (double)div[c];
                    c0++;
                }
            part[k] = s;
            pc[k] = c0;
        }
        double s = 0.0;
        int64_t c0 = 0;
        for (int k = 0; k < D; k++) {
            s += part[k];
            c0 += pc[k];
        }
        if (c0 > 0) {
            R mean = (R)(s / (double)c0);
            mean_removed = (double)mean;
#pragma omp parallel for schedule(static)
            for (size_t c = 0; c < n; c++)
                if (!occ[c]) div[c] = div[c] - mean;
        }
    }
    const R omega = (R)P.omega;
    const R om1 = R(1) - omega;
    const size_t sy = (size_t)W, sz = (size_t)W * H;
    for (int it = 0; it < P.sor_iters; it++) {
        for (int colour = 0; colour < 2; colour++) {
#pragma omp parallel for schedule(static)
            for (int k = 0; k < D; k++)
                for (int j = 0; j < H; j++)
                    for (int i = (j + k + colour) & 1; i < W; i += 2) {
                        size_t c = d.cell(i, j, k);
                        if (occ[c] || cnt[c] == R(0)) continue;
                        R s = R(0);
                        if (i > 0 && !occ[c - 1]) s = s + p[c - 1];
                        if (i < W - 1 && !occ[c + 1]) s = s + p[c + 1];
                        if (j > 0 && !occ[c - sy]) s = s + p[c - sy];
                        if (j < H - 1 && !occ[c + sy]) s = s + p[c + sy];
                        if (k > 0 && !occ[c - sz]) s = s + p[c - sz];
                        if (k < D - 1 && !occ[c + sz]) s = s + p[c + sz];
                        R gs = (s - div[c]) / cnt[c];
                        p[c] = om1 * p[c] + omega * gs;
                    }
        }
    }
    /* gradient subtraction */
    const R zero = R(0);
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= D; k++)
        for (int j = 0; j <= H; j++)
            for (int i = 0; i <= W; i++) {
                if (j < H && k < D && u_live(d, occ, i, j, k, open)) {
                    R& f = u[d.uix(i, j, k)];
                    if (i == 0) f = f - (p[d.cell(0, j, k)] - zero);
                    else if (i == W) f = f - (zero - p[d.cell(W - 1, j, k)]);
                    else f = f - (p[d.cell(i, j, k)] - p[d.cell(i - 1, j, k)]);
                }
                if (i < W && k < D && v_live(d, occ, i, j, k, open)) {
                    R& f = v[d.vix(i, j, k)];
                    if (j == 0) f = f - (p[d.cell(i, 0, k)] - zero);
                    else if (j == H) f = f - (zero - p[d.cell(i, H - 1, k)]);
                    else f = f - (p[d.cell(i, j, k)] - p[d.cell(i, j - 1, k)]);
                }
                if (i < W && j < H && w_live(d, occ, i, j, k, open)) {
                    R& f = w[d.wix(i, j, k)];
                    if (k == 0) f = f - (p[d.cell(i, j, 0)] - zero);
                    else if (k == D) f = f - (zero - p[d.cell(i, j, D - 1)]);
                    else f = f - (p[d.cell(i, j, k)] - p[d.cell(i, j, k - 1)]);
                }
            }
    if (st) {
        double mx = 0.0, r2 = 0.0;
        int64_t nf = 0;
#pragma omp parallel for schedule(static) reduction(max : mx) reduction(+ : r2, nf)
        for (int k = 0; k < D; k++)
            for (int j = 0; j < H; j++)
                for (int i = 0; i < W; i++) {
                    size_t c = d.cell(i, j, k);
                    if (occ[c]) continue;
                    nf++;
                    double dv = std::fabs((double)divergence(i, j, k));
                    if (dv > mx) mx = dv;
                    double s = 0.0;
                    if (i > 0 && !occ[c - 1]) s += (double)p[c - 1];
                    if (i < W - 1 && !occ[c + 1]) s += (double)p[c + 1];
                    if (j > 0 && !occ[c - sy]) s += (double)p[c - sy];
                    if (j < H - 1 && !occ[c + sy]) s += (double)p[c + sy];
                    if (k > 0 && !occ[c - sz]) s += (double)p[c - sz];
                    if (k < D - 1 && !occ[c + sz]) s += (double)p[c + sz];
                    double r = (double)div[c] - (s - (double)cnt[c] * (double)p[c]);
                    r2 += r * r;
                }
        st->max_abs_div = mx;
        st->residual_l2 = std::sqrt(r2);
        st->div_mean_removed = mean_removed;
        st->free_cells = nf;
    }
    (void)nfree_cells;
    if (p_out) std::copy(p.begin(), p.end(), p_out);
    if (div_out) std::copy(div.begin(), div.end(), div_out);
}

/* One timestep in the order of ZQ_SmokeSimulation3D::UpdateOneFrame
 * (ZQ_SmokeSimulation3D.cpp:156-243): force, attenuation, velocity advection
 * (always with the open write-back, Utils3D:2163), projection, scalar
 * advection (in place, Utils3D:3835), reinjection. */
template <class R>
int step(const Dims& d, R* u, R* v, R* w, R* T, R* rho, const uint8_t* occ, const zqs_params& P, R* p_out) {
    add_force(d, u, v, w, occ, T, rho, P);
    attenuate(d, u, v, w, T, rho, occ, P);
    int rc = advect_velocity(d, u, v, w, occ, P, P.adv_vel_mode, true);
    if (rc) return rc;
    project(d, u, v, w, occ, P, p_out, (R*)nullptr, (zqs_stats*)nullptr);
    rc = advect_scalar(d, u, v, w, occ, T, rho, T, rho, P, P.adv_sca_mode);
    if (rc) return rc;
    reinject(d, T, rho, P);
    return ZQS_OK;
}

}  // namespace zqo

/* ---------------------------------------------------------------------- */
/* extern "C" entry points for ctypes (suffix _f32 / _f64)                 */
/* ---------------------------------------------------------------------- */

#define ZQO_API extern "C" __attribute__((visibility("default")))

#define ZQO_DEFINE(SFX, R)                                                                              \
    ZQO_API void zqo_mac_to_regular4_##SFX(int W, int H, int D, const R* u, const R* v, const R* w,     \
                                           R* vel4) {                                                   \
        zqo::mac_to_regular4<R>(zqo::Dims{W, H, D}, u, v, w, vel4);                                     \
    }                                                                                                   \
    ZQO_API void zqo_regular4_to_mac_##SFX(int W, int H, int D, const R* vel4, R* u, R* v, R* w) {      \
        zqo::regular4_to_mac<R>(zqo::Dims{W, H, D}, vel4, u, v, w);                                     \
    }                                                                                                   \
    ZQO_API void zqo_add_force_##SFX(int W, int H, int D, R* u, R* v, R* w, const uint8_t* occ,         \
                                     const R* T, const R* rho, const zqs_params* P) {                   \
        zqo::add_force<R>(zqo::Dims{W, H, D}, u, v, w, occ, T, rho, *P);                                 \
    }                                                                                                   \
    ZQO_API void zqo_vorticity_##SFX(int W, int H, int D, const R* u, const R* v, const R* w, R h, R* vort,     \
                                     R* vs) {                                                           \
        zqo::vorticity<R>(zqo::Dims{W, H, D}, u, v, w, h, vort, vs);                                    \
    }                                                                                                   \
    ZQO_API void zqo_attenuate_##SFX(int W, int H, int D, R* u, R* v, R* w, R* T, R* rho,               \
                                     const uint8_t* occ, const zqs_params* P) {                         \
        zqo::attenuate<R>(zqo::Dims{W, H, D}, u, v, w, T, rho, occ, *P);                                 \
    }                                                                                                   \
    ZQO_API int zqo_advect_velocity_##SFX(int W, int H, int D, R* u, R* v, R* w, const uint8_t* occ,    \
                                          const zqs_params* P, int mode, int is_open) {                 \
        return zqo::advect_velocity<R>(zqo::Dims{W, H, D}, u, v, w, occ, *P, mode, is_open != 0);       \
    }                                                                                                   \
    ZQO_API int zqo_advect_scalar_##SFX(int W, int H, int D, const R* u, const R* v, const R* w,        \
                                        const uint8_t* occ, const R* Tin, const R* Din, R* Tout,        \
                                        R* Dout, const zqs_params* P, int mode) {                       \
        return zqo::advect_scalar<R>(zqo::Dims{W, H, D}, u, v, w, occ, Tin, Din, Tout, Dout, *P, mode); \
    }                                                                                                   \
    ZQO_API void zqo_project_##SFX(int W, int H, int D, R* u, R* v, R* w, const uint8_t* occ,           \
                                   const zqs_params* P, R* p_out, R* div_out, zqs_stats* st) {          \
        zqo::project<R>(zqo::Dims{W, H, D}, u, v, w, occ, *P, p_out, div_out, st);                      \
    }                                                                                                   \
    ZQO_API void zqo_reinject_##SFX(int W, int H, int D, R* T, R* rho, const zqs_params* P) {           \
        zqo::reinject<R>(zqo::Dims{W, H, D}, T, rho, *P);                                               \
    }                                                                                                   \
    ZQO_API void zqo_apply_advect_result_##SFX(int W, int H, int D, const uint8_t* occ, const R* au,    \
                                               const R* av, const R* aw, R* u, R* v, R* w,              \
                                               int is_open) {                                           \
        zqo::apply_advect_result<R>(zqo::Dims{W, H, D}, occ, au, av, aw, u, v, w, is_open != 0);        \
    }                                                                                                   \
    ZQO_API int zqo_step_##SFX(int W, int H, int D, R* u, R* v, R* w, R* T, R* rho,                     \
                               const uint8_t* occ, const zqs_params* P, int nsteps, R* p_out) {         \
        for (int s = 0; s < nsteps; s++) {                                                              \
            int rc = zqo::step<R>(zqo::Dims{W, H, D}, u, v, w, T, rho, occ, *P, p_out);                  \
            if (rc) return rc;                                                                          \
        }                                                                                               \
        return 0;                                                                                       \
    }

ZQO_DEFINE(f32, float)
ZQO_DEFINE(f64, double)

ZQO_API int zqo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
