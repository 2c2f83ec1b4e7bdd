/*
 * zqs_oracle.cpp -- CPU ORACLE for the 3D smoke step.  TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C++ templated on the arithmetic type R
 * (float or double), the per-timestep path of ZQ_SmokeSimulation3D as the
 * reference computes it.  It checks the results of the CUDA library: only the
 * tests, the smoke check and bench.py's CPU-baseline / reference arm may load
 * it.  Nothing in the product links or calls it.
 *
 * Parity status: pinned to the reference's own kernels for the forces,
 * attenuation, MAC<->regular conversion, velocity and scalar advection and
 * the write-backs.  The reference ships no tests or golden outputs and cannot
 * be built as a program here (Windows/VS2015, missing ZQlib/ZQlibCuda), but
 * its kernel files ZQ_CUDA_MACtoRegular.cu, ZQ_CUDA_Attenuation3D.cu,
 * ZQ_CUDA_AddForce3D.cu and ZQ_CUDA_Advection3D.cu compile unmodified as
 * device modules (oracle/build_ref.py, texture references served by
 * oracle/ref_shim/texref_shim.cuh), and tests/test_ref_pin_gpu.py runs them
 * against this file: bit for bit where the arithmetic is theirs, within 1e-5
 * where their normalised MAC texture coordinates round.  The red-black SOR
 * stays a restatement: its source lives in the un-vendored ZQlibCuda.  See
 * the per-function citations for the in-tree evidence each rule is restated
 * from.  Independent plain-Python / numpy restatements of the reference loops
 * check it in the tests too (SOR, the advection modes and BFECC, the
 * write-backs, forces, object stamping, the coarse stages and block step, the
 * viewer's shader).
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
 * [0, n-1] (fmax/fmin return the non-NaN operand, so NaN becomes 0): outside
 * that range clamp-to-edge filtering returns the edge texel, which the
 * clamped coordinate gives with t = 0 or i0 == i1.  Then floor and fraction.
 * Mirrors cudaAddressModeClamp + cudaFilterModeLinear of the reference's
 * textures (ZQ_CUDA_Advection3D.cu:654-993). */
template <class R> struct Axis {
    int i0, i1;
    R t;
};
template <class R> static inline Axis<R> axis(R g, int n) {
    g = std::fmin(std::fmax(g, R(0)), R(n - 1));
    R f = std::floor(g);
    Axis<R> a;
    a.t = g - f;
    a.i0 = (int)f;
    a.i1 = a.i0 + 1 < n ? a.i0 + 1 : n - 1;
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
 *     the alpha term is not in the reference, alpha = 0 reproduces it)
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

/* F (optional): an external per-cell force added to f after the buoyancy
 * terms, component-major dense (F[q*ncell + cell], q = x, y, z); the control
 * of the adjoint problem (no counterpart in the reference). */
template <class R>
void add_force(const Dims& d, R* u, R* v, R* w, const uint8_t* occ, const R* T, const R* rho,
               const zqs_params& P, const R* F = nullptr) {
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
        if (F) {
            fx = fx + F[c];
            fy = fy + F[n + c];
            fz = fz + F[2 * n + c];
        }
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
 * Regular: the float4 centre field sits at (i+.5, j+.5, k+.5).
 * sg = -1 samples the negated field (the BFECC backward pass negates the
 * velocity arrays in place, Adv3D:1284, and negation is exact). */
template <class R> struct MacSampler {
    Dims d;
    const R *u, *v, *w;
    R sg = R(1);
    void operator()(R px, R py, R pz, R& vx, R& vy, R& vz) const {
        const R hf = R(0.5);
        vx = trilinear<R>(u, d.W + 1, d.H, d.D, 1, 0, px, py - hf, pz - hf);
        vy = trilinear<R>(v, d.W, d.H + 1, d.D, 1, 0, px - hf, py, pz - hf);
        vz = trilinear<R>(w, d.W, d.H, d.D + 1, 1, 0, px - hf, py - hf, pz);
        if (sg < R(0)) {
            vx = -vx;
            vy = -vy;
            vz = -vz;
        }
    }
};
template <class R> struct RegSampler {
    Dims d;
    const R* vel4;
    R sg = R(1);
    void operator()(R px, R py, R pz, R& vx, R& vy, R& vz) const {
        const R hf = R(0.5);
        R gx = px - hf, gy = py - hf, gz = pz - hf;
        vx = trilinear<R>(vel4, d.W, d.H, d.D, 4, 0, gx, gy, gz);
        vy = trilinear<R>(vel4, d.W, d.H, d.D, 4, 1, gx, gy, gz);
        vz = trilinear<R>(vel4, d.W, d.H, d.D, 4, 2, gx, gy, gz);
        if (sg < R(0)) {
            vx = -vx;
            vy = -vy;
            vz = -vz;
        }
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

/* One pass of Advect_Velocity_inMAC_outMAC_{u,v,w}_Kernel (Adv3D:232-377):
 * every face backtraces through the MAC velocity `vel` and samples the MAC
 * input (iu, iv, iw) at the end point; no write-back. */
template <class R>
void mac_pass(const Dims& d, const uint8_t* occ, const AdvCtx<R>& a, const MacSampler<R>& s, const R* iu,
              const R* iv, const R* iw, R* ou, R* ov, R* ow) {
    const R hf = R(0.5);
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k <= d.D; k++)
        for (int j = 0; j <= d.H; j++)
            for (int i = 0; i <= d.W; i++) {
                if (j < d.H && k < d.D) {
                    R px = (R)i, py = (R)j + hf, pz = (R)k + hf;
                    backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                    ou[d.uix(i, j, k)] = trilinear<R>(iu, d.W + 1, d.H, d.D, 1, 0, px, py - hf, pz - hf);
                }
                if (i < d.W && k < d.D) {
                    R px = (R)i + hf, py = (R)j, pz = (R)k + hf;
                    backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                    ov[d.vix(i, j, k)] = trilinear<R>(iv, d.W, d.H + 1, d.D, 1, 0, px - hf, py, pz - hf);
                }
                if (i < d.W && j < d.H) {
                    R px = (R)i + hf, py = (R)j + hf, pz = (R)k;
                    backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                    ow[d.wix(i, j, k)] = trilinear<R>(iw, d.W, d.H, d.D + 1, 1, 0, px - hf, py - hf, pz);
                }
            }
}

/* One pass of Advect_Velocity_inRegular_outMAC_{u,v,w}_Kernel (Adv3D:115-230):
 * faces backtrace through the regular velocity and sample channel q of the
 * regular input in4 at the end point. */
template <class R>
void regmac_pass(const Dims& d, const uint8_t* occ, const AdvCtx<R>& a, const RegSampler<R>& s, const R* in4,
                 R* ou, R* ov, R* ow) {
    const R hf = R(0.5);
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k <= d.D; k++)
        for (int j = 0; j <= d.H; j++)
            for (int i = 0; i <= d.W; i++) {
                if (j < d.H && k < d.D) {
                    R px = (R)i, py = (R)j + hf, pz = (R)k + hf;
                    backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                    ou[d.uix(i, j, k)] = trilinear<R>(in4, d.W, d.H, d.D, 4, 0, px - hf, py - hf, pz - hf);
                }
                if (i < d.W && k < d.D) {
                    R px = (R)i + hf, py = (R)j, pz = (R)k + hf;
                    backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                    ov[d.vix(i, j, k)] = trilinear<R>(in4, d.W, d.H, d.D, 4, 1, px - hf, py - hf, pz - hf);
                }
                if (i < d.W && j < d.H) {
                    R px = (R)i + hf, py = (R)j + hf, pz = (R)k;
                    backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                    ow[d.wix(i, j, k)] = trilinear<R>(in4, d.W, d.H, d.D, 4, 2, px - hf, py - hf, pz - hf);
                }
            }
}

/* One pass of Advect_Velocity_inRegular_outRegular_Kernel (Adv3D:76-113):
 * cell centres backtrace through the regular velocity and sample the regular
 * input in4 (channels 0-2; channel 3 is written 0). */
template <class R>
void regreg_pass(const Dims& d, const uint8_t* occ, const AdvCtx<R>& a, const RegSampler<R>& s, const R* in4,
                 R* out4) {
    const R hf = R(0.5);
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < d.D; k++)
        for (int j = 0; j < d.H; j++)
            for (int i = 0; i < d.W; i++) {
                R px = (R)i + hf, py = (R)j + hf, pz = (R)k + hf;
                backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                size_t c = d.cell(i, j, k);
                for (int q = 0; q < 3; q++)
                    out4[c * 4 + q] = trilinear<R>(in4, d.W, d.H, d.D, 4, q, px - hf, py - hf, pz - hf);
                out4[c * 4 + 3] = R(0);
            }
}

/* The BFECC corrections (Adv3D:56-74).  Input_Increment_Kernel works on float
 * arrays with double constants, so the expression is evaluated in double and
 * rounded once to float; the float4 form multiplies by float constants and
 * rounds each operation.  In FP64 both are the plain expression. */
template <class R> static inline R bfecc_inc(R in, R star) {
    if (sizeof(R) == 4) return (R)((double)in * 1.5 - (double)star * 0.5);
    return in * R(1.5) - star * R(0.5);
}
template <class R> static inline R bfecc_inc4(R in, R star) {
    const R a = in * R(1.5);
    const R b = star * R(0.5);
    return a - b;
}

/* Advect_Velocity (ZQ_CUDA_Advection3D.cu:1686-1749); the write-back follows
 * cu_Apply_Advect_Velocity_Result_{Open,Closed}.  BFECC (Adv3D:1108-1182,
 * 1240-1336, 1389-1474): a forward pass, a pass through the negated velocity
 * from its result, the correction in = 1.5 in - 0.5 in** and a forward pass
 * from the corrected field (the velocity of the passes is the original one
 * throughout).  In the MAC form the correction is written into u, v, w in
 * place, so faces the write-back leaves alone end with the corrected value. */
template <class R>
int advect_velocity(const Dims& d, R* u, R* v, R* w, const uint8_t* occ, const zqs_params& P, int mode,
                    bool open) {
    AdvCtx<R> a = adv_ctx<R>(P);
    std::vector<R> ou(d.nu(), R(0)), ov(d.nv(), R(0)), ow(d.nw(), R(0));
    if (mode == ZQS_ADV_VEL_INMAC_OUTMAC) {
        MacSampler<R> s{d, u, v, w};
        mac_pass(d, occ, a, s, u, v, w, ou.data(), ov.data(), ow.data());
    } else if (mode == ZQS_ADV_VEL_INMAC_OUTMAC_BFECC) {
        std::vector<R> u0(u, u + d.nu()), v0(v, v + d.nv()), w0(w, w + d.nw());
        std::vector<R> su(d.nu(), R(0)), sv(d.nv(), R(0)), sw(d.nw(), R(0));
        MacSampler<R> fwd{d, u0.data(), v0.data(), w0.data()};
        MacSampler<R> bwd = fwd;
        bwd.sg = R(-1);
        mac_pass(d, occ, a, fwd, u0.data(), v0.data(), w0.data(), ou.data(), ov.data(), ow.data());
        mac_pass(d, occ, a, bwd, ou.data(), ov.data(), ow.data(), su.data(), sv.data(), sw.data());
        for (size_t x = 0; x < d.nu(); x++) u[x] = bfecc_inc(u[x], su[x]);
        for (size_t x = 0; x < d.nv(); x++) v[x] = bfecc_inc(v[x], sv[x]);
        for (size_t x = 0; x < d.nw(); x++) w[x] = bfecc_inc(w[x], sw[x]);
        mac_pass(d, occ, a, fwd, u, v, w, ou.data(), ov.data(), ow.data());
    } else if (mode == ZQS_ADV_VEL_INREG_OUTMAC || mode == ZQS_ADV_VEL_INREG_OUTMAC_BFECC) {
        std::vector<R> vel4(d.ncell() * 4);
        mac_to_regular4(d, u, v, w, vel4.data());
        RegSampler<R> fwd{d, vel4.data()};
        if (mode == ZQS_ADV_VEL_INREG_OUTMAC) {
            regmac_pass(d, occ, a, fwd, vel4.data(), ou.data(), ov.data(), ow.data());
        } else {
            RegSampler<R> bwd = fwd;
            bwd.sg = R(-1);
            std::vector<R> t4(d.ncell() * 4);
            regmac_pass(d, occ, a, fwd, vel4.data(), ou.data(), ov.data(), ow.data());
            mac_to_regular4(d, ou.data(), ov.data(), ow.data(), t4.data());
            regmac_pass(d, occ, a, bwd, t4.data(), ou.data(), ov.data(), ow.data());
            mac_to_regular4(d, ou.data(), ov.data(), ow.data(), t4.data());
            for (size_t x = 0; x < t4.size(); x++) t4[x] = bfecc_inc4(vel4[x], t4[x]);
            regmac_pass(d, occ, a, fwd, t4.data(), ou.data(), ov.data(), ow.data());
        }
    } else if (mode == ZQS_ADV_VEL_INREG_OUTREG || mode == ZQS_ADV_VEL_INREG_OUTREG_BFECC) {
        /* then Regular4_to_MAC and the write-back (Adv3D:1061-1106) */
        std::vector<R> vel4(d.ncell() * 4), out4(d.ncell() * 4);
        mac_to_regular4(d, u, v, w, vel4.data());
        RegSampler<R> fwd{d, vel4.data()};
        if (mode == ZQS_ADV_VEL_INREG_OUTREG) {
            regreg_pass(d, occ, a, fwd, vel4.data(), out4.data());
        } else {
            RegSampler<R> bwd = fwd;
            bwd.sg = R(-1);
            std::vector<R> s4(d.ncell() * 4);
            regreg_pass(d, occ, a, fwd, vel4.data(), out4.data());
            regreg_pass(d, occ, a, bwd, out4.data(), s4.data());
            for (size_t x = 0; x < s4.size(); x++) s4[x] = bfecc_inc4(vel4[x], s4[x]);
            regreg_pass(d, occ, a, fwd, s4.data(), out4.data());
        }
        regular4_to_mac(d, out4.data(), ou.data(), ov.data(), ow.data());
    } else {
        return ZQS_EUNSUPPORTED;
    }
    apply_advect_result(d, occ, ou.data(), ov.data(), ow.data(), u, v, w, open);
    return ZQS_OK;
}

/* One pass of Advect_Scalar_{MAC,Regular}_Velocity_Kernel (Adv3D:379-469):
 * backtrace from cell centres, sample T and rho at the final point; every
 * cell is written, occupied ones included. */
template <class R, class VelF>
void scalar_pass(const Dims& d, const uint8_t* occ, const AdvCtx<R>& a, const VelF& s, const R* Tin, const R* Din,
                 R* Tout, R* Dout) {
    const R hf = R(0.5);
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < d.D; k++)
        for (int j = 0; j < d.H; j++)
            for (int i = 0; i < d.W; i++) {
                R px = (R)i + hf, py = (R)j + hf, pz = (R)k + hf;
                backtrace(d, occ, s, a.steps, a.dt, a.h, a.full, px, py, pz);
                size_t c = d.cell(i, j, k);
                Tout[c] = trilinear<R>(Tin, d.W, d.H, d.D, 1, 0, px - hf, py - hf, pz - hf);
                Dout[c] = trilinear<R>(Din, d.W, d.H, d.D, 1, 0, px - hf, py - hf, pz - hf);
            }
}

/* Advect_Scalar (Adv3D:1751-1821) through MAC or regular velocity.  BFECC
 * follows cu_Advect_Scalar_{MAC,Regular}_Velocity_BFECC (Adv3D:1507-1554,
 * 1586-1648): forward pass, negated-velocity pass from its result, the
 * correction of the inputs (double expression, written into Tin/Din as the
 * reference does), forward pass from the corrected fields.  (The reference's
 * Advect_Scalar entry point never calls these and returns zeros for the BFECC
 * types, Adv3D:1786-1794; this restates the intended three passes.) */
template <class R>
int advect_scalar(const Dims& d, const R* u, const R* v, const R* w, const uint8_t* occ, const R* Tin,
                  const R* Din, R* Tout, R* Dout, const zqs_params& P, int mode) {
    AdvCtx<R> a = adv_ctx<R>(P);
    std::vector<R> tt(d.ncell()), dd(d.ncell());
    const bool reg = mode == ZQS_ADV_SCA_REG || mode == ZQS_ADV_SCA_REG_BFECC;
    const bool bfecc = mode == ZQS_ADV_SCA_MAC_BFECC || mode == ZQS_ADV_SCA_REG_BFECC;
    if (mode < ZQS_ADV_SCA_MAC || mode > ZQS_ADV_SCA_REG_BFECC) return ZQS_EUNSUPPORTED;
    std::vector<R> vel4;
    if (reg) {
        vel4.resize(d.ncell() * 4);
        mac_to_regular4(d, u, v, w, vel4.data());
    }
    MacSampler<R> ms{d, u, v, w};
    RegSampler<R> rs{d, vel4.data()};
    auto pass = [&](R sg, const R* ti, const R* di, R* to, R* dout) {
        if (reg) {
            RegSampler<R> s = rs;
            s.sg = sg;
            scalar_pass(d, occ, a, s, ti, di, to, dout);
        } else {
            MacSampler<R> s = ms;
            s.sg = sg;
            scalar_pass(d, occ, a, s, ti, di, to, dout);
        }
    };
    if (!bfecc) {
        pass(R(1), Tin, Din, tt.data(), dd.data());
    } else {
        std::vector<R> t1(d.ncell()), d1(d.ncell()), ti(Tin, Tin + d.ncell()), di(Din, Din + d.ncell());
        pass(R(1), ti.data(), di.data(), t1.data(), d1.data());
        pass(R(-1), t1.data(), d1.data(), tt.data(), dd.data());
        for (size_t x = 0; x < d.ncell(); x++) {
            ti[x] = bfecc_inc(ti[x], tt[x]);
            di[x] = bfecc_inc(di[x], dd[x]);
        }
        pass(R(1), ti.data(), di.data(), tt.data(), dd.data());
    }
    std::copy(tt.begin(), tt.end(), Tout);
    std::copy(dd.begin(), dd.end(), Dout);
    return ZQS_OK;
}

/* ZQ_ReinjectTemperatureDensity3D (Utils3D:3842-3882): cells inside a source
 * get density and temperature overwritten; sources in order, the last wins.
 * Box test |i+.5-cx| <= hx (per axis); sphere test (not in the reference)
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
 * Added: over-relaxation p <- (1-omega)*p + omega*GS, evaluated as
 * fma(omega/cnt, s - div, (1-omega)*p) with omega/cnt rounded once (a
 * per-cell constant); cold start p=0; neighbours summed as the tree
 * ((x- + x+) + (y- + y+)) + (z- + z+), +0 for excluded neighbours.  (The reference's SOR source is not in its tree, so the
 * rounding of the update is this restatement's choice.)
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
                        const R xm = (i > 0 && !occ[c - 1]) ? p[c - 1] : R(0);
                        const R xp = (i < W - 1 && !occ[c + 1]) ? p[c + 1] : R(0);
                        const R ym = (j > 0 && !occ[c - sy]) ? p[c - sy] : R(0);
                        const R yp = (j < H - 1 && !occ[c + sy]) ? p[c + sy] : R(0);
                        const R zm = (k > 0 && !occ[c - sz]) ? p[c - sz] : R(0);
                        const R zp = (k < D - 1 && !occ[c + sz]) ? p[c + sz] : R(0);
                        const R s = ((xm + xp) + (ym + yp)) + (zm + zp);
                        const R wc = omega / cnt[c];
                        p[c] = std::fma(wc, s - div[c], om1 * p[c]);
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

/* ---------------------------------------------------------------------- */
/* Coarse-grid projection (COARSE_{OPEN,CLOSED}_POISSON_SOR)               */
/* ---------------------------------------------------------------------- */
/* ZQ_TotalProjection3D (Utils3D:3688-3794) for the coarse SOR solvers (the
 * reference calls the open coarse solver for both, :3732-3746):
 *   1. face un-occupancy ratios of the grid coarsened by s (ZQ_InitCoarseGrid3D,
 *      Utils3D:1666-1888); a coarse cell with all six ratios 0 is occupied;
 *   2. coarse velocity = mean of the fine faces on each coarse face
 *      (ZQ_MapFine2Coarse3D, Utils3D:2170-2258);
 *   3. red-black SOR on the face-ratio Poisson system of ZQ_InitMatOpenPoisson3D
 *      (Utils3D:476-601: weight = ratio of the face to a free in-domain
 *      neighbour, 1 with p = 0 for a domain face, diagonal = their sum in the
 *      order out-of-domain count, z-, z+, y-, y+, x-, x+), then the velocity
 *      correction of ZQ_AdjustOpenVelocity3D (Utils3D:2794-2866: u -= p_R - p_L
 *      on faces with ratio > 0); the delta is (u - g) - u as the reference forms
 *      it (Utils3D:2611-2642).  The solver itself (SolveOpenPoissonRedBlack-
 *      withFaceRatio3D_MAC) is not in the reference tree; the update is the one
 *      of the fine SOR: p <- fma(omega/diag, s - div, (1-omega) p);
 *   4. the delta added to the fine faces of each coarse face whose fine cells
 *      are free (ZQ_MapCoarse2Fine3D, Utils3D:3172-3296; the x = W face tests
 *      the inside cell x = W-1, where the reference reads one past the row);
 *   5. with s > 1, an exact projection inside every s^3 block
 *      (ZQ_SubProjection3D, Utils3D:3298-3685): blocks without an occupied fine
 *      cell apply the dense matrix of ZQ_InitSubMatPoisson3D (Utils3D:1151-
 *      1391) to the block's faces (products accumulated with fused
 *      multiply-adds in column order, as a GPU matrix product compiled with
 *      contraction accumulates); the others solve their closed Poisson
 *      problem (ratio 1 between free cells, first free cell pinned) in the
 *      least-squares sense (ZQ_SolveSubGrid3D, Utils3D:1393-1521), here by CG
 *      on the normal equations in double, and correct the interior faces. */

template <class R>
struct CoarseGrid {
    Dims c;                         // coarse dims
    std::vector<R> ru, rv, rw;      // face un-occupancy ratios (coarse MAC layout)
    std::vector<uint8_t> occ;       // coarse occupancy
};

template <class R>
void coarse_init(const Dims& f, int s, const uint8_t* occ, CoarseGrid<R>& g) {
    Dims c{f.W / s, f.H / s, f.D / s};
    g.c = c;
    g.ru.assign(c.nu(), R(0));
    g.rv.assign(c.nv(), R(0));
    g.rw.assign(c.nw(), R(0));
    g.occ.assign(c.ncell(), 0);
    const R area = (R)(s * s);
    auto ratio = [&](int n) -> R { return R(1) - (R)n / area; };
    for (int k = 0; k < c.D; k++)
        for (int j = 0; j < c.H; j++)
            for (int i = 0; i <= c.W; i++) {
                int n = 0;
                for (int sk = 0; sk < s; sk++)
                    for (int sj = 0; sj < s; sj++) {
                        const int y = j * s + sj, z = k * s + sk;
                        if (i == 0) n += occ[f.cell(0, y, z)] ? 1 : 0;
                        else if (i == c.W) n += occ[f.cell(f.W - 1, y, z)] ? 1 : 0;
                        else n += (occ[f.cell(i * s, y, z)] || occ[f.cell(i * s - 1, y, z)]) ? 1 : 0;
                    }
                g.ru[c.uix(i, j, k)] = ratio(n);
            }
    for (int k = 0; k < c.D; k++)
        for (int j = 0; j <= c.H; j++)
            for (int i = 0; i < c.W; i++) {
                int n = 0;
                for (int sk = 0; sk < s; sk++)
                    for (int si = 0; si < s; si++) {
                        const int x = i * s + si, z = k * s + sk;
                        if (j == 0) n += occ[f.cell(x, 0, z)] ? 1 : 0;
                        else if (j == c.H) n += occ[f.cell(x, f.H - 1, z)] ? 1 : 0;
                        else n += (occ[f.cell(x, j * s, z)] || occ[f.cell(x, j * s - 1, z)]) ? 1 : 0;
                    }
                g.rv[c.vix(i, j, k)] = ratio(n);
            }
    for (int k = 0; k <= c.D; k++)
        for (int j = 0; j < c.H; j++)
            for (int i = 0; i < c.W; i++) {
                int n = 0;
                for (int sj = 0; sj < s; sj++)
                    for (int si = 0; si < s; si++) {
                        const int x = i * s + si, y = j * s + sj;
                        if (k == 0) n += occ[f.cell(x, y, 0)] ? 1 : 0;
                        else if (k == c.D) n += occ[f.cell(x, y, f.D - 1)] ? 1 : 0;
                        else n += (occ[f.cell(x, y, k * s)] || occ[f.cell(x, y, k * s - 1)]) ? 1 : 0;
                    }
                g.rw[c.wix(i, j, k)] = ratio(n);
            }
    for (int k = 0; k < c.D; k++)
        for (int j = 0; j < c.H; j++)
            for (int i = 0; i < c.W; i++)
                g.occ[c.cell(i, j, k)] = (g.ru[c.uix(i, j, k)] == R(0) && g.ru[c.uix(i + 1, j, k)] == R(0) &&
                                          g.rv[c.vix(i, j, k)] == R(0) && g.rv[c.vix(i, j + 1, k)] == R(0) &&
                                          g.rw[c.wix(i, j, k)] == R(0) && g.rw[c.wix(i, j, k + 1)] == R(0))
                                             ? 1
                                             : 0;
}

/* Steps 2-4: the coarse correction added to the fine faces. */
template <class R>
void coarse_correct(const Dims& f, int s, const uint8_t* occ, const CoarseGrid<R>& g, R* u, R* v, R* w,
                    const zqs_params& P) {
    const Dims& c = g.c;
    const R area = (R)(s * s);
    std::vector<R> cu(c.nu()), cv(c.nv()), cw(c.nw());
    for (int k = 0; k < c.D; k++)
        for (int j = 0; j < c.H; j++)
            for (int i = 0; i <= c.W; i++) {
                R sum = R(0);
                for (int sk = 0; sk < s; sk++)
                    for (int sj = 0; sj < s; sj++) sum += u[f.uix(i * s, j * s + sj, k * s + sk)];
                cu[c.uix(i, j, k)] = sum / area;
            }
    for (int k = 0; k < c.D; k++)
        for (int j = 0; j <= c.H; j++)
            for (int i = 0; i < c.W; i++) {
                R sum = R(0);
                for (int sk = 0; sk < s; sk++)
                    for (int si = 0; si < s; si++) sum += v[f.vix(i * s + si, j * s, k * s + sk)];
                cv[c.vix(i, j, k)] = sum / area;
            }
    for (int k = 0; k <= c.D; k++)
        for (int j = 0; j < c.H; j++)
            for (int i = 0; i < c.W; i++) {
                R sum = R(0);
                for (int sj = 0; sj < s; sj++)
                    for (int si = 0; si < s; si++) sum += w[f.wix(i * s + si, j * s + sj, k * s)];
                cw[c.wix(i, j, k)] = sum / area;
            }
    /* the face-ratio system */
    const int W = c.W, H = c.H, D = c.D;
    const size_t n = c.ncell();
    std::vector<R> div(n, R(0)), diag(n, R(0)), p(n, R(0));
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                const size_t cc = c.cell(i, j, k);
                if (g.occ[cc]) continue;
                div[cc] = ((((cu[c.uix(i + 1, j, k)] - cu[c.uix(i, j, k)]) + cv[c.vix(i, j + 1, k)]) -
                            cv[c.vix(i, j, k)]) + cw[c.wix(i, j, k + 1)]) - cw[c.wix(i, j, k)];
                const int nin = (k > 0) + (k < D - 1) + (j > 0) + (j < H - 1) + (i > 0) + (i < W - 1);
                R cnt = (R)(6 - nin);
                if (k > 0 && !g.occ[cc - (size_t)W * H]) cnt += g.rw[c.wix(i, j, k)];
                if (k < D - 1 && !g.occ[cc + (size_t)W * H]) cnt += g.rw[c.wix(i, j, k + 1)];
                if (j > 0 && !g.occ[cc - W]) cnt += g.rv[c.vix(i, j, k)];
                if (j < H - 1 && !g.occ[cc + W]) cnt += g.rv[c.vix(i, j + 1, k)];
                if (i > 0 && !g.occ[cc - 1]) cnt += g.ru[c.uix(i, j, k)];
                if (i < W - 1 && !g.occ[cc + 1]) cnt += g.ru[c.uix(i + 1, j, k)];
                diag[cc] = cnt;
            }
    const R omega = (R)P.omega;
    const R om1 = R(1) - omega;
    const size_t sy = (size_t)W, sz = (size_t)W * H;
    auto term = [&](bool in, size_t nb, R r) -> R { return (in && !g.occ[nb]) ? r * p[nb] : R(0); };
    for (int it = 0; it < P.sor_iters; it++)
        for (int colour = 0; colour < 2; colour++)
            for (int k = 0; k < D; k++)
                for (int j = 0; j < H; j++)
                    for (int i = (j + k + colour) & 1; i < W; i += 2) {
                        const size_t cc = c.cell(i, j, k);
                        if (g.occ[cc] || diag[cc] == R(0)) continue;
                        const R xm = term(i > 0, cc - 1, g.ru[c.uix(i, j, k)]);
                        const R xp = term(i < W - 1, cc + 1, g.ru[c.uix(i + 1, j, k)]);
                        const R ym = term(j > 0, cc - sy, g.rv[c.vix(i, j, k)]);
                        const R yp = term(j < H - 1, cc + sy, g.rv[c.vix(i, j + 1, k)]);
                        const R zm = term(k > 0, cc - sz, g.rw[c.wix(i, j, k)]);
                        const R zp = term(k < D - 1, cc + sz, g.rw[c.wix(i, j, k + 1)]);
                        const R sum = ((xm + xp) + (ym + yp)) + (zm + zp);
                        const R wc = omega / diag[cc];
                        p[cc] = std::fma(wc, sum - div[cc], om1 * p[cc]);
                    }
    /* delta = (u - (p_R - p_L)) - u on faces with ratio > 0, p = 0 outside */
    const R zero = R(0);
    auto pc = [&](int i, int j, int k) -> R { return p[c.cell(i, j, k)]; };
    std::vector<R> du(c.nu(), R(0)), dv(c.nv(), R(0)), dw(c.nw(), R(0));
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i <= W; i++) {
                const size_t x = c.uix(i, j, k);
                if (!(g.ru[x] > R(0))) continue;
                const R gr = i == 0 ? pc(0, j, k) - zero : (i == W ? zero - pc(W - 1, j, k) : pc(i, j, k) - pc(i - 1, j, k));
                du[x] = (cu[x] - gr) - cu[x];
            }
    for (int k = 0; k < D; k++)
        for (int j = 0; j <= H; j++)
            for (int i = 0; i < W; i++) {
                const size_t x = c.vix(i, j, k);
                if (!(g.rv[x] > R(0))) continue;
                const R gr = j == 0 ? pc(i, 0, k) - zero : (j == H ? zero - pc(i, H - 1, k) : pc(i, j, k) - pc(i, j - 1, k));
                dv[x] = (cv[x] - gr) - cv[x];
            }
    for (int k = 0; k <= D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                const size_t x = c.wix(i, j, k);
                if (!(g.rw[x] > R(0))) continue;
                const R gr = k == 0 ? pc(i, j, 0) - zero : (k == D ? zero - pc(i, j, D - 1) : pc(i, j, k) - pc(i, j, k - 1));
                dw[x] = (cw[x] - gr) - cw[x];
            }
    /* back to the fine faces whose fine cells are free */
    for (int k = 0; k < c.D; k++)
        for (int j = 0; j < c.H; j++)
            for (int i = 0; i <= c.W; i++)
                for (int sk = 0; sk < s; sk++)
                    for (int sj = 0; sj < s; sj++) {
                        const int x = i * s, y = j * s + sj, z = k * s + sk;
                        bool ok;
                        if (i == 0) ok = !occ[f.cell(0, y, z)];
                        else if (i == c.W) ok = !occ[f.cell(f.W - 1, y, z)];
                        else ok = !occ[f.cell(x, y, z)] && !occ[f.cell(x - 1, y, z)];
                        if (ok) u[f.uix(x, y, z)] += du[c.uix(i, j, k)];
                    }
    for (int k = 0; k < c.D; k++)
        for (int j = 0; j <= c.H; j++)
            for (int i = 0; i < c.W; i++)
                for (int sk = 0; sk < s; sk++)
                    for (int si = 0; si < s; si++) {
                        const int x = i * s + si, y = j * s, z = k * s + sk;
                        bool ok;
                        if (j == 0) ok = !occ[f.cell(x, 0, z)];
                        else if (j == c.H) ok = !occ[f.cell(x, f.H - 1, z)];
                        else ok = !occ[f.cell(x, y, z)] && !occ[f.cell(x, y - 1, z)];
                        if (ok) v[f.vix(x, y, z)] += dv[c.vix(i, j, k)];
                    }
    for (int k = 0; k <= c.D; k++)
        for (int j = 0; j < c.H; j++)
            for (int i = 0; i < c.W; i++)
                for (int sj = 0; sj < s; sj++)
                    for (int si = 0; si < s; si++) {
                        const int x = i * s + si, y = j * s + sj, z = k * s;
                        bool ok;
                        if (k == 0) ok = !occ[f.cell(x, y, 0)];
                        else if (k == c.D) ok = !occ[f.cell(x, y, f.D - 1)];
                        else ok = !occ[f.cell(x, y, z)] && !occ[f.cell(x, y, z - 1)];
                        if (ok) w[f.wix(x, y, z)] += dw[c.wix(i, j, k)];
                    }
}

/* Block face order of the sub-projection (Utils3D:3356-3385): u faces
 * (k, j, i = 0..s), then v (k, j = 0..s, i), then w (k = 0..s, j, i); the
 * interior faces (rows of the matrix, Utils3D:1348-1387) in the same order
 * with i, j or k in 1..s-1. */
struct BlockFaces {
    int s, nf, ni;
    int uix(int i, int j, int k) const { return (k * s + j) * (s + 1) + i; }
    int vix(int i, int j, int k) const { return s * s * (s + 1) + (k * (s + 1) + j) * s + i; }
    int wix(int i, int j, int k) const { return 2 * s * s * (s + 1) + (k * s + j) * s + i; }
    explicit BlockFaces(int s_) : s(s_), nf(3 * s_ * s_ * (s_ + 1)), ni(3 * s_ * s_ * (s_ - 1)) {}
    /* interior face r -> block face index */
    std::vector<int> interior() const {
        std::vector<int> r;
        for (int k = 0; k < s; k++)
            for (int j = 0; j < s; j++)
                for (int i = 1; i < s; i++) r.push_back(uix(i, j, k));
        for (int k = 0; k < s; k++)
            for (int j = 1; j < s; j++)
                for (int i = 0; i < s; i++) r.push_back(vix(i, j, k));
        for (int k = 1; k < s; k++)
            for (int j = 0; j < s; j++)
                for (int i = 0; i < s; i++) r.push_back(wix(i, j, k));
        return r;
    }
};

/* ZQ_InitSubMatPoisson3D (Utils3D:1151-1391): the matrix I - D [0; P+ V]
 * restricted to the interior faces, P the block's Neumann Laplacian without
 * the column of cell 0, V the divergence, D the gradient on interior faces;
 * P+ = (P^T P)^-1 P^T (P has full column rank; the reference forms P+ by SVD),
 * with P^T P = (L^2) without row and column 0 and P^T V = L V without row 0
 * (L symmetric).  Built in double, stored as float rows of nf columns. */
static std::vector<float> submatrix(int s) {
    const int n = s * s * s;
    BlockFaces bf(s);
    const int nf = bf.nf;
    std::vector<double> L((size_t)n * n, 0.0);
    auto cell = [&](int i, int j, int k) { return (k * s + j) * s + i; };
    for (int k = 0; k < s; k++)
        for (int j = 0; j < s; j++)
            for (int i = 0; i < s; i++) {
                const int c0 = cell(i, j, k);
                int cnt = 0;
                const int di[6] = {-1, 1, 0, 0, 0, 0}, dj[6] = {0, 0, -1, 1, 0, 0}, dk[6] = {0, 0, 0, 0, -1, 1};
                for (int q = 0; q < 6; q++) {
                    const int a = i + di[q], b = j + dj[q], e = k + dk[q];
                    if (a < 0 || a >= s || b < 0 || b >= s || e < 0 || e >= s) continue;
                    L[(size_t)c0 * n + cell(a, b, e)] = 1.0;
                    cnt++;
                }
                L[(size_t)c0 * n + c0] = -(double)cnt;
            }
    /* V: divergence of cell c over the block faces */
    std::vector<double> V((size_t)n * nf, 0.0);
    for (int k = 0; k < s; k++)
        for (int j = 0; j < s; j++)
            for (int i = 0; i < s; i++) {
                double* r = &V[(size_t)cell(i, j, k) * nf];
                r[bf.uix(i, j, k)] -= 1.0;
                r[bf.uix(i + 1, j, k)] += 1.0;
                r[bf.vix(i, j, k)] -= 1.0;
                r[bf.vix(i, j + 1, k)] += 1.0;
                r[bf.wix(i, j, k)] -= 1.0;
                r[bf.wix(i, j, k + 1)] += 1.0;
            }
    const int m = n - 1;
    /* G = (L^2)[1:,1:], B = (L V)[1:, :] */
    std::vector<double> G((size_t)m * m, 0.0), B((size_t)m * nf, 0.0);
    for (int a = 1; a < n; a++) {
        for (int b = 1; b < n; b++) {
            double acc = 0.0;
            for (int t = 0; t < n; t++) acc += L[(size_t)a * n + t] * L[(size_t)t * n + b];
            G[(size_t)(a - 1) * m + (b - 1)] = acc;
        }
        for (int t = 0; t < n; t++) {
            const double l = L[(size_t)a * n + t];
            if (l == 0.0) continue;
            const double* vr = &V[(size_t)t * nf];
            double* br = &B[(size_t)(a - 1) * nf];
            for (int q = 0; q < nf; q++) br[q] += l * vr[q];
        }
    }
    /* Cholesky G = C C^T, then X = G^-1 B */
    for (int a = 0; a < m; a++) {
        for (int b = 0; b <= a; b++) {
            double acc = G[(size_t)a * m + b];
            for (int t = 0; t < b; t++) acc -= G[(size_t)a * m + t] * G[(size_t)b * m + t];
            if (a == b) G[(size_t)a * m + a] = std::sqrt(acc);
            else G[(size_t)a * m + b] = acc / G[(size_t)b * m + b];
        }
    }
    for (int q = 0; q < nf; q++) {
        for (int a = 0; a < m; a++) {
            double acc = B[(size_t)a * nf + q];
            for (int t = 0; t < a; t++) acc -= G[(size_t)a * m + t] * B[(size_t)t * nf + q];
            B[(size_t)a * nf + q] = acc / G[(size_t)a * m + a];
        }
        for (int a = m - 1; a >= 0; a--) {
            double acc = B[(size_t)a * nf + q];
            for (int t = a + 1; t < m; t++) acc -= G[(size_t)t * m + a] * B[(size_t)t * nf + q];
            B[(size_t)a * nf + q] = acc / G[(size_t)a * m + a];
        }
    }
    /* rows: interior faces; row r of I - D [0; X] */
    const std::vector<int> rows = bf.interior();
    std::vector<float> M((size_t)rows.size() * nf);
    auto pres = [&](int c0, int q) -> double { return c0 == 0 ? 0.0 : B[(size_t)(c0 - 1) * nf + q]; };
    for (size_t r = 0; r < rows.size(); r++) {
        const int fidx = rows[r];
        int ca, cb;  // gradient p(cb) - p(ca)
        if (fidx < s * s * (s + 1)) {
            const int i = fidx % (s + 1), j = (fidx / (s + 1)) % s, k = fidx / (s * (s + 1));
            ca = cell(i - 1, j, k);
            cb = cell(i, j, k);
        } else if (fidx < 2 * s * s * (s + 1)) {
            const int x = fidx - s * s * (s + 1);
            const int i = x % s, j = (x / s) % (s + 1), k = x / (s * (s + 1));
            ca = cell(i, j - 1, k);
            cb = cell(i, j, k);
        } else {
            const int x = fidx - 2 * s * s * (s + 1);
            const int i = x % s, j = (x / s) % s, k = x / (s * s);
            ca = cell(i, j, k - 1);
            cb = cell(i, j, k);
        }
        for (int q = 0; q < nf; q++) {
            const double v = (q == fidx ? 1.0 : 0.0) - (pres(cb, q) - pres(ca, q));
            M[r * nf + q] = (float)v;
        }
    }
    return M;
}

/* The closed least-squares projection of one block with occupied cells
 * (ZQ_SolveSubGrid3D, Utils3D:1393-1521): A = Laplacian of the free cells
 * (weight 1 between free neighbours inside the block), the first free cell
 * (scan order) pinned; min |A p - div| over the other free cells by CG on the
 * normal equations (double; the reference uses PCG to 1e-12), pressures rounded
 * to float, interior faces between two free cells corrected by -(p_b - p_a). */
template <class R>
void block_solve(int s, const uint8_t* bocc, const std::vector<R>& in, std::vector<R>& out) {
    const int n = s * s * s;
    BlockFaces bf(s);
    auto cell = [&](int i, int j, int k) { return (k * s + j) * s + i; };
    int first = -1;
    for (int c0 = 0; c0 < n; c0++)
        if (!bocc[c0]) {
            first = c0;
            break;
        }
    out = in;
    if (first < 0) return;
    std::vector<double> b(n, 0.0);
    for (int k = 0; k < s; k++)
        for (int j = 0; j < s; j++)
            for (int i = 0; i < s; i++) {
                const int c0 = cell(i, j, k);
                if (bocc[c0]) continue;
                const R dv = ((((in[bf.uix(i + 1, j, k)] - in[bf.uix(i, j, k)]) + in[bf.vix(i, j + 1, k)]) -
                               in[bf.vix(i, j, k)]) + in[bf.wix(i, j, k + 1)]) - in[bf.wix(i, j, k)];
                b[c0] = (double)dv;
            }
    auto applyA = [&](const std::vector<double>& x, std::vector<double>& y) {
        for (int k = 0; k < s; k++)
            for (int j = 0; j < s; j++)
                for (int i = 0; i < s; i++) {
                    const int c0 = cell(i, j, k);
                    if (bocc[c0]) {
                        y[c0] = 0.0;
                        continue;
                    }
                    double acc = 0.0;
                    int cnt = 0;
                    const int di[6] = {0, 0, 0, 0, -1, 1}, dj[6] = {0, 0, -1, 1, 0, 0}, dk[6] = {-1, 1, 0, 0, 0, 0};
                    for (int q = 0; q < 6; q++) {
                        const int a = i + di[q], bb = j + dj[q], e = k + dk[q];
                        if (a < 0 || a >= s || bb < 0 || bb >= s || e < 0 || e >= s) continue;
                        const int nb = cell(a, bb, e);
                        if (bocc[nb]) continue;
                        acc += x[nb];
                        cnt++;
                    }
                    y[c0] = acc - (double)cnt * x[c0];
                }
    };
    /* normal equations in p with p[first] = 0: N p = A (A p), b' = A b, both
     * with the pinned and occupied entries zeroed */
    auto mask = [&](std::vector<double>& x) {
        for (int c0 = 0; c0 < n; c0++)
            if (bocc[c0] || c0 == first) x[c0] = 0.0;
    };
    std::vector<double> x(n, 0.0), r(n), pdir(n), t(n), q(n);
    applyA(b, r);
    mask(r);
    pdir = r;
    double rr = 0.0;
    for (int c0 = 0; c0 < n; c0++) rr += r[c0] * r[c0];
    const double rr0 = rr;
    const int maxit = 2 * (n + bf.nf + 1);
    for (int it = 0; it < maxit && rr > 1e-24 * rr0 && rr > 0.0; it++) {
        applyA(pdir, t);
        applyA(t, q);
        mask(q);
        double pq = 0.0;
        for (int c0 = 0; c0 < n; c0++) pq += pdir[c0] * q[c0];
        if (!(pq > 0.0)) break;
        const double alpha = rr / pq;
        double rn = 0.0;
        for (int c0 = 0; c0 < n; c0++) {
            x[c0] += alpha * pdir[c0];
            r[c0] -= alpha * q[c0];
            rn += r[c0] * r[c0];
        }
        const double beta = rn / rr;
        rr = rn;
        for (int c0 = 0; c0 < n; c0++) pdir[c0] = r[c0] + beta * pdir[c0];
    }
    std::vector<R> p(n);
    for (int c0 = 0; c0 < n; c0++) p[c0] = (R)x[c0];
    for (int k = 0; k < s; k++)
        for (int j = 0; j < s; j++)
            for (int i = 1; i < s; i++)
                if (!bocc[cell(i, j, k)] && !bocc[cell(i - 1, j, k)]) {
                    const R d = -(p[cell(i, j, k)] - p[cell(i - 1, j, k)]);
                    out[bf.uix(i, j, k)] = in[bf.uix(i, j, k)] + d;
                }
    for (int k = 0; k < s; k++)
        for (int j = 1; j < s; j++)
            for (int i = 0; i < s; i++)
                if (!bocc[cell(i, j, k)] && !bocc[cell(i, j - 1, k)]) {
                    const R d = -(p[cell(i, j, k)] - p[cell(i, j - 1, k)]);
                    out[bf.vix(i, j, k)] = in[bf.vix(i, j, k)] + d;
                }
    for (int k = 1; k < s; k++)
        for (int j = 0; j < s; j++)
            for (int i = 0; i < s; i++)
                if (!bocc[cell(i, j, k)] && !bocc[cell(i, j, k - 1)]) {
                    const R d = -(p[cell(i, j, k)] - p[cell(i, j, k - 1)]);
                    out[bf.wix(i, j, k)] = in[bf.wix(i, j, k)] + d;
                }
}

template <class R>
void sub_projection(const Dims& f, int s, const uint8_t* occ, const std::vector<float>& M, R* u, R* v, R* w) {
    BlockFaces bf(s);
    const std::vector<int> rows = bf.interior();
    const int cW = f.W / s, cH = f.H / s, cD = f.D / s;
#pragma omp parallel for schedule(dynamic, 1)
    for (int K = 0; K < cD; K++)
        for (int J = 0; J < cH; J++)
            for (int I = 0; I < cW; I++) {
                const int x0 = I * s, y0 = J * s, z0 = K * s;
                std::vector<R> in(bf.nf), out;
                std::vector<uint8_t> bocc(s * s * s);
                bool any = false;
                for (int k = 0; k < s; k++)
                    for (int j = 0; j < s; j++)
                        for (int i = 0; i < s; i++) {
                            const uint8_t o = occ[f.cell(x0 + i, y0 + j, z0 + k)] ? 1 : 0;
                            bocc[(k * s + j) * s + i] = o;
                            any = any || o;
                        }
                for (int k = 0; k < s; k++)
                    for (int j = 0; j < s; j++)
                        for (int i = 0; i <= s; i++) in[bf.uix(i, j, k)] = u[f.uix(x0 + i, y0 + j, z0 + k)];
                for (int k = 0; k < s; k++)
                    for (int j = 0; j <= s; j++)
                        for (int i = 0; i < s; i++) in[bf.vix(i, j, k)] = v[f.vix(x0 + i, y0 + j, z0 + k)];
                for (int k = 0; k <= s; k++)
                    for (int j = 0; j < s; j++)
                        for (int i = 0; i < s; i++) in[bf.wix(i, j, k)] = w[f.wix(x0 + i, y0 + j, z0 + k)];
                if (!any) {
                    out = in;
                    for (size_t r = 0; r < rows.size(); r++) {
                        R acc = R(0);
                        const float* mr = &M[r * bf.nf];
                        for (int q = 0; q < bf.nf; q++) acc = std::fma((R)mr[q], in[q], acc);
                        out[rows[r]] = acc;
                    }
                } else {
                    block_solve(s, bocc.data(), in, out);
                }
                for (int k = 0; k < s; k++)
                    for (int j = 0; j < s; j++)
                        for (int i = 1; i < s; i++) u[f.uix(x0 + i, y0 + j, z0 + k)] = out[bf.uix(i, j, k)];
                for (int k = 0; k < s; k++)
                    for (int j = 1; j < s; j++)
                        for (int i = 0; i < s; i++) v[f.vix(x0 + i, y0 + j, z0 + k)] = out[bf.vix(i, j, k)];
                for (int k = 1; k < s; k++)
                    for (int j = 0; j < s; j++)
                        for (int i = 0; i < s; i++) w[f.wix(x0 + i, y0 + j, z0 + k)] = out[bf.wix(i, j, k)];
            }
}

template <class R>
int project_coarse(const Dims& d, R* u, R* v, R* w, const uint8_t* occ, const zqs_params& P) {
    const int s = P.sub_size;
    if (s < 1 || d.W % s || d.H % s || d.D % s) return ZQS_EINVAL;
    CoarseGrid<R> g;
    coarse_init(d, s, occ, g);
    coarse_correct(d, s, occ, g, u, v, w, P);
    if (s > 1) {
        const std::vector<float> M = submatrix(s);
        sub_projection(d, s, occ, M, u, v, w);
    }
    return ZQS_OK;
}

/* ZQ_ApplyMovingObject3D (Utils3D:1933-2046): the occupancy becomes the
 * objects' voxels (plus the six domain walls for the closed solvers, :1994-
 * 2044); each in-domain voxel of each object, in order, is occupied and its
 * six faces take the object's velocity, an int scaled by h/dt (float
 * division, widened) and truncated to int (:1958-1962). */
template <class R>
void stamp_objects(const Dims& d, uint8_t* occ, R* u, R* v, R* w, const zqs_object* objs, int n, int closed,
                   const zqs_params& P) {
    const int W = d.W, H = d.H, D = d.D;
    // closed: 0 no walls, 1 the six walls of the closed solvers, 2 all but y = H-1
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++)
                occ[d.cell(i, j, k)] = (closed && (i == 0 || i == W - 1 || j == 0 || (j == H - 1 && closed == 1) ||
                                                   k == 0 || k == D - 1))
                                           ? 1
                                           : 0;
    const double scale = (double)(P.voxel_size / P.step_time);
    for (int q = 0; q < n; q++) {
        const zqs_object& o = objs[q];
        int cu = o.vel[0], cv = o.vel[1], cw = o.vel[2];
        cu = (int)(cu * scale);
        cv = (int)(cv * scale);
        cw = (int)(cw * scale);
        for (int sk = 0; sk < o.size[2]; sk++)
            for (int sj = 0; sj < o.size[1]; sj++)
                for (int si = 0; si < o.size[0]; si++) {
                    if (!o.mask[((size_t)sk * o.size[1] + sj) * o.size[0] + si]) continue;
                    const int ix = si + o.pos[0] - o.center[0];
                    const int iy = sj + o.pos[1] - o.center[1];
                    const int iz = sk + o.pos[2] - o.center[2];
                    if (ix < 0 || ix >= W || iy < 0 || iy >= H || iz < 0 || iz >= D) continue;
                    occ[d.cell(ix, iy, iz)] = 1;
                    u[d.uix(ix, iy, iz)] = (R)cu;
                    u[d.uix(ix + 1, iy, iz)] = (R)cu;
                    v[d.vix(ix, iy, iz)] = (R)cv;
                    v[d.vix(ix, iy + 1, iz)] = (R)cv;
                    w[d.wix(ix, iy, iz)] = (R)cw;
                    w[d.wix(ix, iy, iz + 1)] = (R)cw;
                }
    }
}

/* One timestep in the order of ZQ_SmokeSimulation3D::UpdateOneFrame
 * (ZQ_SmokeSimulation3D.cpp:156-243): force, attenuation, velocity advection
 * (always with the open write-back, Utils3D:2163), projection, scalar
 * advection (in place, Utils3D:3835), reinjection. */
template <class R>
int step(const Dims& d, R* u, R* v, R* w, R* T, R* rho, const uint8_t* occ, const zqs_params& P, R* p_out,
         const R* F = nullptr) {
    add_force(d, u, v, w, occ, T, rho, P, F);
    attenuate(d, u, v, w, T, rho, occ, P);
    int rc = advect_velocity(d, u, v, w, occ, P, P.adv_vel_mode, true);
    if (rc) return rc;
    if (P.solver == ZQS_SOLVER_COARSE_OPEN) {
        rc = project_coarse(d, u, v, w, occ, P);
        if (rc) return rc;
    } else {
        project(d, u, v, w, occ, P, p_out, (R*)nullptr, (zqs_stats*)nullptr);
    }
    rc = advect_scalar(d, u, v, w, occ, T, rho, T, rho, P, P.adv_sca_mode);
    if (rc) return rc;
    reinject(d, T, rho, P);
    return ZQS_OK;
}

/* ====================================================================== */
/* Reverse mode (adjoint) of the step, for the force-field control problem */
/* ====================================================================== */
/* No counterpart in the reference: the differentiable path is new.  The
 * forward map is step() with the control F; its adjoint is written stage by
 * stage in reverse order, in the arithmetic type R (double for the FP64
 * gradient).  Discrete decisions (the backtrace's occupancy/domain break,
 * clamping, floor cells, the zero-length normal of the confinement force) are
 * held at their forward values: this is the derivative almost everywhere.
 * Stage rules (each the transpose of the forward rule restated above):
 *   reinjection       adjoint zeroed on source cells (values overwritten)
 *   advection         the final trilinear sample scattered back to its 8
 *                     corners (transposed trilinear), and the position chain
 *                     x_{s+1} = x_s - (dt/h) vel(x_s) reversed substep by
 *                     substep: g_vel(x_s) = -(dt/h) g_x is scattered into the
 *                     MAC velocity, g_x += J_vel(x_s)^T g_vel(x_s)
 *   projection        G^T, then the 2K half-sweeps transposed in reverse
 *                     order (black then red), then div^T (closed: minus the
 *                     free-cell mean first)
 *   attenuation       the same factors on the same live faces / cells
 *   force             face averaging transposed into cell forces; buoyancy
 *                     into T and rho; confinement through N = g/|g|, the
 *                     one-sided/central gradient of |w|, the curl stencil and
 *                     the MAC-to-centre average. */

template <class R> static inline bool bt_ok(const Dims& d, const uint8_t* occ, R x, R y, R z) {
    if (!(x >= R(0) && x <= (R)d.W && y >= R(0) && y <= (R)d.H && z >= R(0) && z <= (R)d.D)) return false;
    int i = clampi((int)std::floor(x), 0, d.W - 1);
    int j = clampi((int)std::floor(y), 0, d.H - 1);
    int k = clampi((int)std::floor(z), 0, d.D - 1);
    return occ[d.cell(i, j, k)] == 0;
}

/* backtrace() with every position kept: xs[3s..3s+2] = x_s; returns m, the
 * index of the point backtrace() returns. */
template <class R, class VelF>
static inline int backtrace_record(const Dims& d, const uint8_t* occ, const VelF& vel, int steps, R dt, R h,
                                   bool full, R px, R py, R pz, R* xs) {
    R vx, vy, vz;
    vel(px, py, pz, vx, vy, vz);
    xs[0] = px;
    xs[1] = py;
    xs[2] = pz;
    int m = 0, istep = 0;
    bool broke = false;
    do {
        if (!bt_ok(d, occ, px, py, pz)) {
            broke = true;
            break;
        }
        m = istep;
        px = px - (vx * dt) / h;
        py = py - (vy * dt) / h;
        pz = pz - (vz * dt) / h;
        vel(px, py, pz, vx, vy, vz);
        istep++;
        xs[3 * istep + 0] = px;
        xs[3 * istep + 1] = py;
        xs[3 * istep + 2] = pz;
    } while (istep < steps);
    if (full && !broke && bt_ok(d, occ, px, py, pz)) m = istep;
    return m;
}

/* Trilinear value and its gradient with respect to (gx, gy, gz); clamped
 * axes have equal corners and so a zero derivative. */
template <class R, class S>
static inline R trilinear_grad(const S* base, int nx, int ny, int nz, R gx, R gy, R gz, R g[3]) {
    Axis<R> ax = axis(gx, nx), ay = axis(gy, ny), az = axis(gz, nz);
    auto at = [&](int i, int j, int k) -> R { return (R)base[(((size_t)k * ny) + j) * nx + i]; };
    R c000 = at(ax.i0, ay.i0, az.i0), c100 = at(ax.i1, ay.i0, az.i0);
    R c010 = at(ax.i0, ay.i1, az.i0), c110 = at(ax.i1, ay.i1, az.i0);
    R c001 = at(ax.i0, ay.i0, az.i1), c101 = at(ax.i1, ay.i0, az.i1);
    R c011 = at(ax.i0, ay.i1, az.i1), c111 = at(ax.i1, ay.i1, az.i1);
    R c00 = lerp(c000, c100, ax.t), c10 = lerp(c010, c110, ax.t);
    R c01 = lerp(c001, c101, ax.t), c11 = lerp(c011, c111, ax.t);
    R c0 = lerp(c00, c10, ay.t), c1 = lerp(c01, c11, ay.t);
    g[0] = lerp(lerp(c100 - c000, c110 - c010, ay.t), lerp(c101 - c001, c111 - c011, ay.t), az.t);
    g[1] = lerp(c10 - c00, c11 - c01, az.t);
    g[2] = c1 - c0;
    return lerp(c0, c1, az.t);
}

template <class R> static inline void atomic_add(R* p, R v) {
#pragma omp atomic
    *p += v;
}

/* Transposed trilinear: val times each corner weight added to the corners. */
template <class R>
static inline void trilinear_scatter(R* base, int nx, int ny, int nz, R gx, R gy, R gz, R val) {
    if (val == R(0)) return;
    Axis<R> ax = axis(gx, nx), ay = axis(gy, ny), az = axis(gz, nz);
    const R wx[2] = {R(1) - ax.t, ax.t}, wy[2] = {R(1) - ay.t, ay.t}, wz[2] = {R(1) - az.t, az.t};
    const int ix[2] = {ax.i0, ax.i1}, iy[2] = {ay.i0, ay.i1}, iz[2] = {az.i0, az.i1};
    for (int c = 0; c < 2; c++)
        for (int b = 0; b < 2; b++)
            for (int a = 0; a < 2; a++)
                atomic_add(base + ((((size_t)iz[c] * ny) + iy[b]) * nx + ix[a]), ((wx[a] * wy[b]) * wz[c]) * val);
}

/* MAC velocity: Jacobian rows J[a] = grad vel_a, and the transposed sample. */
template <class R> struct MacAdj {
    Dims d;
    const R *u, *v, *w;
    void jac(R px, R py, R pz, R J[3][3]) const {
        const R hf = R(0.5);
        trilinear_grad<R>(u, d.W + 1, d.H, d.D, px, py - hf, pz - hf, J[0]);
        trilinear_grad<R>(v, d.W, d.H + 1, d.D, px - hf, py, pz - hf, J[1]);
        trilinear_grad<R>(w, d.W, d.H, d.D + 1, px - hf, py - hf, pz, J[2]);
    }
    void scatter(R* gu, R* gv, R* gw, R px, R py, R pz, const R g[3]) const {
        const R hf = R(0.5);
        trilinear_scatter<R>(gu, d.W + 1, d.H, d.D, px, py - hf, pz - hf, g[0]);
        trilinear_scatter<R>(gv, d.W, d.H + 1, d.D, px - hf, py, pz - hf, g[1]);
        trilinear_scatter<R>(gw, d.W, d.H, d.D + 1, px - hf, py - hf, pz, g[2]);
    }
};

/* Reverse the position chain of a recorded backtrace: gx (adjoint of x_m) in,
 * velocity adjoint scattered into (gu, gv, gw). */
template <class R>
static inline void backtrace_adjoint(const MacAdj<R>& V, R* gu, R* gv, R* gw, const R* xs, int m, R dt, R h,
                                     R gx[3]) {
    const R c = dt / h;
    for (int s = m - 1; s >= 0; s--) {
        const R* x = xs + 3 * s;
        R gvel[3] = {-c * gx[0], -c * gx[1], -c * gx[2]};
        V.scatter(gu, gv, gw, x[0], x[1], x[2], gvel);
        R J[3][3];
        V.jac(x[0], x[1], x[2], J);
        for (int b = 0; b < 3; b++) gx[b] += (J[0][b] * gvel[0] + J[1][b] * gvel[1]) + J[2][b] * gvel[2];
    }
}

/* Adjoint of advect_scalar (MAC velocity): (gTout, gDout) in; adjoints of the
 * advected fields added to (gTin, gDin) and of the velocity to (gu, gv, gw). */
template <class R>
void advect_scalar_adjoint(const Dims& d, const R* u, const R* v, const R* w, const uint8_t* occ, const R* Tin,
                           const R* Din, const R* gTout, const R* gDout, R* gTin, R* gDin, R* gu, R* gv, R* gw,
                           const zqs_params& P) {
    AdvCtx<R> a = adv_ctx<R>(P);
    const R hf = R(0.5);
    MacSampler<R> ms{d, u, v, w};
    MacAdj<R> V{d, u, v, w};
#pragma omp parallel
    {
        std::vector<R> xs(3 * (a.steps + 1));
#pragma omp for schedule(dynamic, 1)
        for (int k = 0; k < d.D; k++)
            for (int j = 0; j < d.H; j++)
                for (int i = 0; i < d.W; i++) {
                    size_t c = d.cell(i, j, k);
                    R gT = gTout[c], gD = gDout[c];
                    if (gT == R(0) && gD == R(0)) continue;
                    int m = backtrace_record(d, occ, ms, a.steps, a.dt, a.h, a.full, (R)i + hf, (R)j + hf,
                                             (R)k + hf, xs.data());
                    R* x = xs.data() + 3 * m;
                    trilinear_scatter<R>(gTin, d.W, d.H, d.D, x[0] - hf, x[1] - hf, x[2] - hf, gT);
                    trilinear_scatter<R>(gDin, d.W, d.H, d.D, x[0] - hf, x[1] - hf, x[2] - hf, gD);
                    R g1[3], g2[3];
                    trilinear_grad<R>(Tin, d.W, d.H, d.D, x[0] - hf, x[1] - hf, x[2] - hf, g1);
                    trilinear_grad<R>(Din, d.W, d.H, d.D, x[0] - hf, x[1] - hf, x[2] - hf, g2);
                    R gx[3] = {gT * g1[0] + gD * g2[0], gT * g1[1] + gD * g2[1], gT * g1[2] + gD * g2[2]};
                    backtrace_adjoint(V, gu, gv, gw, xs.data(), m, a.dt, a.h, gx);
                }
    }
}

/* Adjoint of advect_velocity (inMAC_outMAC, open write-back): the adjoint of
 * the output (gu3..) in, the adjoint of the input velocity (gu2..) ASSIGNED. */
template <class R>
void advect_velocity_adjoint(const Dims& d, const R* u, const R* v, const R* w, const uint8_t* occ,
                             const zqs_params& P, const R* gu3, const R* gv3, const R* gw3, R* gu2, R* gv2, R* gw2) {
    AdvCtx<R> a = adv_ctx<R>(P);
    const R hf = R(0.5);
    std::fill(gu2, gu2 + d.nu(), R(0));
    std::fill(gv2, gv2 + d.nv(), R(0));
    std::fill(gw2, gw2 + d.nw(), R(0));
    MacSampler<R> ms{d, u, v, w};
    MacAdj<R> V{d, u, v, w};
#pragma omp parallel
    {
        std::vector<R> xs(3 * (a.steps + 1));
#pragma omp for schedule(dynamic, 1)
        for (int k = 0; k <= d.D; k++)
            for (int j = 0; j <= d.H; j++)
                for (int i = 0; i <= d.W; i++) {
                    for (int q = 0; q < 3; q++) {
                        bool in, live;
                        R px = (R)i + hf, py = (R)j + hf, pz = (R)k + hf;
                        size_t f;
                        const R* gin;
                        R* gout;
                        if (q == 0) {
                            in = j < d.H && k < d.D;
                            if (!in) continue;
                            live = u_live(d, occ, i, j, k, true);
                            px = (R)i;
                            f = d.uix(i, j, k);
                            gin = gu3;
                            gout = gu2;
                        } else if (q == 1) {
                            in = i < d.W && k < d.D;
                            if (!in) continue;
                            live = v_live(d, occ, i, j, k, true);
                            py = (R)j;
                            f = d.vix(i, j, k);
                            gin = gv3;
                            gout = gv2;
                        } else {
                            in = i < d.W && j < d.H;
                            if (!in) continue;
                            live = w_live(d, occ, i, j, k, true);
                            pz = (R)k;
                            f = d.wix(i, j, k);
                            gin = gw3;
                            gout = gw2;
                        }
                        const R g = gin[f];
                        if (g == R(0)) continue;
                        if (!live) {
                            atomic_add(gout + f, g);
                            continue;
                        }
                        int m = backtrace_record(d, occ, ms, a.steps, a.dt, a.h, a.full, px, py, pz, xs.data());
                        R* x = xs.data() + 3 * m;
                        R gx[3];
                        if (q == 0) {
                            trilinear_scatter<R>(gu2, d.W + 1, d.H, d.D, x[0], x[1] - hf, x[2] - hf, g);
                            trilinear_grad<R>(u, d.W + 1, d.H, d.D, x[0], x[1] - hf, x[2] - hf, gx);
                        } else if (q == 1) {
                            trilinear_scatter<R>(gv2, d.W, d.H + 1, d.D, x[0] - hf, x[1], x[2] - hf, g);
                            trilinear_grad<R>(v, d.W, d.H + 1, d.D, x[0] - hf, x[1], x[2] - hf, gx);
                        } else {
                            trilinear_scatter<R>(gw2, d.W, d.H, d.D + 1, x[0] - hf, x[1] - hf, x[2], g);
                            trilinear_grad<R>(w, d.W, d.H, d.D + 1, x[0] - hf, x[1] - hf, x[2], gx);
                        }
                        for (int b = 0; b < 3; b++) gx[b] = gx[b] * g;
                        backtrace_adjoint(V, gu2, gv2, gw2, xs.data(), m, a.dt, a.h, gx);
                    }
                }
    }
}

/* SOR stencil weight of each cell (0 for occupied cells), as project(). */
template <class R> static void sor_counts(const Dims& d, const uint8_t* occ, bool open, std::vector<R>& cnt) {
    cnt.assign(d.ncell(), R(0));
    for (int k = 0; k < d.D; k++)
        for (int j = 0; j < d.H; j++)
            for (int i = 0; i < d.W; i++) {
                size_t c = d.cell(i, j, k);
                if (occ[c]) continue;
                int nin = 0, nfree = 0;
                const int di[6] = {-1, 1, 0, 0, 0, 0}, dj[6] = {0, 0, -1, 1, 0, 0}, dk[6] = {0, 0, 0, 0, -1, 1};
                for (int q = 0; q < 6; q++) {
                    int a = i + di[q], b = j + dj[q], e = k + dk[q];
                    if (a < 0 || a >= d.W || b < 0 || b >= d.H || e < 0 || e >= d.D) continue;
                    nin++;
                    if (!occ[d.cell(a, b, e)]) nfree++;
                }
                cnt[c] = open ? (R)(6 - (nin - nfree)) : (R)nfree;
            }
}

/* Adjoint of project(): (gu, gv, gw) = adjoint of the projected velocity in,
 * adjoint of the velocity before projection out (in place). */
template <class R>
void project_adjoint(const Dims& d, R* gu, R* gv, R* gw, const uint8_t* occ, const zqs_params& P) {
    const int W = d.W, H = d.H, D = d.D;
    const size_t n = d.ncell();
    const bool open = P.solver == ZQS_SOLVER_OPEN;
    std::vector<R> cnt;
    sor_counts(d, occ, open, cnt);
    std::vector<R> gp(n, R(0)), gd(n, R(0));
    /* G^T: u_f -= p_R - p_L  =>  gp_R -= g_f, gp_L += g_f */
    for (int k = 0; k <= D; k++)
        for (int j = 0; j <= H; j++)
            for (int i = 0; i <= W; i++) {
                if (j < H && k < D && u_live(d, occ, i, j, k, open)) {
                    R g = gu[d.uix(i, j, k)];
                    if (i < W) gp[d.cell(i, j, k)] -= g;
                    if (i > 0) gp[d.cell(i - 1, j, k)] += g;
                }
                if (i < W && k < D && v_live(d, occ, i, j, k, open)) {
                    R g = gv[d.vix(i, j, k)];
                    if (j < H) gp[d.cell(i, j, k)] -= g;
                    if (j > 0) gp[d.cell(i, j - 1, k)] += g;
                }
                if (i < W && j < H && w_live(d, occ, i, j, k, open)) {
                    R g = gw[d.wix(i, j, k)];
                    if (k < D) gp[d.cell(i, j, k)] -= g;
                    if (k > 0) gp[d.cell(i, j, k - 1)] += g;
                }
            }
    /* SOR^T: half-sweeps in reverse order; for the half-sweep of colour c,
     * z_c = (omega/cnt_c) gp_c goes to every free in-domain neighbour and
     * (negated) to gd_c, then gp_c *= (1-omega). */
    const R omega = (R)P.omega, om1 = R(1) - omega;
    const size_t sy = (size_t)W, sz = (size_t)W * H;
    auto upd = [&](size_t c) { return !occ[c] && cnt[c] != R(0); };
    for (int it = P.sor_iters - 1; it >= 0; it--) {
        for (int colour = 1; colour >= 0; colour--) {
            /* gather into the other colour from this colour's cells */
#pragma omp parallel for schedule(static)
            for (int k = 0; k < D; k++)
                for (int j = 0; j < H; j++)
                    for (int i = (j + k + colour + 1) & 1; i < W; i += 2) {
                        size_t c = d.cell(i, j, k);
                        if (occ[c]) continue;
                        R s = R(0);
                        if (i > 0 && upd(c - 1)) s += (omega / cnt[c - 1]) * gp[c - 1];
                        if (i < W - 1 && upd(c + 1)) s += (omega / cnt[c + 1]) * gp[c + 1];
                        if (j > 0 && upd(c - sy)) s += (omega / cnt[c - sy]) * gp[c - sy];
                        if (j < H - 1 && upd(c + sy)) s += (omega / cnt[c + sy]) * gp[c + sy];
                        if (k > 0 && upd(c - sz)) s += (omega / cnt[c - sz]) * gp[c - sz];
                        if (k < D - 1 && upd(c + sz)) s += (omega / cnt[c + sz]) * gp[c + sz];
                        gp[c] += s;
                    }
#pragma omp parallel for schedule(static)
            for (int k = 0; k < D; k++)
                for (int j = 0; j < H; j++)
                    for (int i = (j + k + colour) & 1; i < W; i += 2) {
                        size_t c = d.cell(i, j, k);
                        if (!upd(c)) continue;
                        gd[c] -= (omega / cnt[c]) * gp[c];
                        gp[c] = om1 * gp[c];
                    }
        }
    }
    if (!open) {
        /* d -= mean_free(d) is its own transpose (an orthogonal projection) */
        double s = 0.0;
        int64_t nf = 0;
        for (size_t c = 0; c < n; c++)
            if (!occ[c]) {
                s += (double)gd[c];
                nf++;
            }
        if (nf > 0) {
            R mean = (R)(s / (double)nf);
            for (size_t c = 0; c < n; c++)
                if (!occ[c]) gd[c] -= mean;
        }
    }
    /* div^T: d_c = u[i+1]-u[i] + v[j+1]-v[j] + w[k+1]-w[k] on free cells */
    auto gdc = [&](int i, int j, int k) -> R {
        if (i < 0 || i >= W || j < 0 || j >= H || k < 0 || k >= D) return R(0);
        size_t c = d.cell(i, j, k);
        return occ[c] ? R(0) : gd[c];
    };
#pragma omp parallel for schedule(static)
    for (int k = 0; k <= D; k++)
        for (int j = 0; j <= H; j++)
            for (int i = 0; i <= W; i++) {
                if (j < H && k < D) gu[d.uix(i, j, k)] += gdc(i - 1, j, k) - gdc(i, j, k);
                if (i < W && k < D) gv[d.vix(i, j, k)] += gdc(i, j - 1, k) - gdc(i, j, k);
                if (i < W && j < H) gw[d.wix(i, j, k)] += gdc(i, j, k - 1) - gdc(i, j, k);
            }
}

/* Adjoint of add_force (F included): (gu, gv, gw) = adjoint of the velocity
 * after the face update in, adjoint of the velocity before it out (in place);
 * adjoints of T, rho and F are ADDED (gF may be null). */
template <class R>
void add_force_adjoint(const Dims& d, const R* u, const R* v, const R* w, const uint8_t* occ, const zqs_params& P,
                       R* gu, R* gv, R* gw, R* gT, R* grho, R* gF) {
    const size_t n = d.ncell();
    const int W = d.W, H = d.H, D = d.D;
    const size_t sy = (size_t)W, sz = (size_t)W * H;
    const R h = (R)P.voxel_size;
    std::vector<R> vort(n * 3, R(0)), vs(n, R(0)), gf(n * 3, R(0));
    vorticity(d, u, v, w, h, vort.data(), vs.data());
    const R dt = (R)P.step_time, hdt = dt * R(0.5);
    /* face averaging transposed */
    for (int k = 0; k <= D; k++)
        for (int j = 0; j <= H; j++)
            for (int i = 0; i <= W; i++) {
                if (j < H && k < D && u_live(d, occ, i, j, k, true)) {
                    R g = gu[d.uix(i, j, k)];
                    if (i == 0) gf[d.cell(0, j, k) * 3 + 0] += dt * g;
                    else if (i == W) gf[d.cell(W - 1, j, k) * 3 + 0] += dt * g;
                    else {
                        gf[d.cell(i, j, k) * 3 + 0] += hdt * g;
                        gf[d.cell(i - 1, j, k) * 3 + 0] += hdt * g;
                    }
                }
                if (i < W && k < D && v_live(d, occ, i, j, k, true)) {
                    R g = gv[d.vix(i, j, k)];
                    if (j == 0) gf[d.cell(i, 0, k) * 3 + 1] += dt * g;
                    else if (j == H) gf[d.cell(i, H - 1, k) * 3 + 1] += dt * g;
                    else {
                        gf[d.cell(i, j, k) * 3 + 1] += hdt * g;
                        gf[d.cell(i, j - 1, k) * 3 + 1] += hdt * g;
                    }
                }
                if (i < W && j < H && w_live(d, occ, i, j, k, true)) {
                    R g = gw[d.wix(i, j, k)];
                    if (k == 0) gf[d.cell(i, j, 0) * 3 + 2] += dt * g;
                    else if (k == D) gf[d.cell(i, j, D - 1) * 3 + 2] += dt * g;
                    else {
                        gf[d.cell(i, j, k) * 3 + 2] += hdt * g;
                        gf[d.cell(i, j, k - 1) * 3 + 2] += hdt * g;
                    }
                }
            }
    const R cc = (R)P.confine * h;
    const R beta = (R)P.buoyancy, alpha = (R)P.gravity;
    std::vector<R> gvs(n, R(0)), gom(n * 3, R(0)), gg(n * 3, R(0));
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                size_t c = d.cell(i, j, k);
                R fx = gf[c * 3 + 0], fy = gf[c * 3 + 1], fz = gf[c * 3 + 2];
                if (gF) {
                    gF[c] += fx;
                    gF[n + c] += fy;
                    gF[2 * n + c] += fz;
                }
                gT[c] += beta * fy;
                grho[c] -= alpha * fy;
                /* recompute the normal of this cell as add_force() does */
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
                R Nx = gx, Ny = gy, Nz = gz;
                if (len != R(0)) {
                    Nx = gx / len;
                    Ny = gy / len;
                    Nz = gz / len;
                }
                const R ox = vort[c * 3 + 0], oy = vort[c * 3 + 1], oz = vort[c * 3 + 2];
                /* f = cc * (N x w) */
                R gNx = cc * (oy * fz - oz * fy), gNy = cc * (oz * fx - ox * fz), gNz = cc * (ox * fy - oy * fx);
                gom[c * 3 + 0] = cc * (Nz * fy - Ny * fz);
                gom[c * 3 + 1] = cc * (Nx * fz - Nz * fx);
                gom[c * 3 + 2] = cc * (Ny * fx - Nx * fy);
                if (len != R(0)) {
                    R dot = (Nx * gNx + Ny * gNy) + Nz * gNz;
                    gg[c * 3 + 0] = (gNx - Nx * dot) / len;
                    gg[c * 3 + 1] = (gNy - Ny * dot) / len;
                    gg[c * 3 + 2] = (gNz - Nz * dot) / len;
                }
            }
    /* gradient of |w| transposed (central x0.5 inside, one-sided at the boundary) */
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                size_t c = d.cell(i, j, k);
                R g = gg[c * 3 + 0];
                if (i == 0) { gvs[c + 1] += g; gvs[c] -= g; }
                else if (i == W - 1) { gvs[c] += g; gvs[c - 1] -= g; }
                else { gvs[c + 1] += R(0.5) * g; gvs[c - 1] -= R(0.5) * g; }
                g = gg[c * 3 + 1];
                if (j == 0) { gvs[c + sy] += g; gvs[c] -= g; }
                else if (j == H - 1) { gvs[c] += g; gvs[c - sy] -= g; }
                else { gvs[c + sy] += R(0.5) * g; gvs[c - sy] -= R(0.5) * g; }
                g = gg[c * 3 + 2];
                if (k == 0) { gvs[c + sz] += g; gvs[c] -= g; }
                else if (k == D - 1) { gvs[c] += g; gvs[c - sz] -= g; }
                else { gvs[c + sz] += R(0.5) * g; gvs[c - sz] -= R(0.5) * g; }
            }
    /* |w| and the curl stencil, interior cells only */
    std::vector<R> gU(n, R(0)), gV(n, R(0)), gW(n, R(0));
    const R twoh = R(2) * h;
    for (int k = 1; k < D - 1; k++)
        for (int j = 1; j < H - 1; j++)
            for (int i = 1; i < W - 1; i++) {
                size_t c = d.cell(i, j, k);
                R ox = vort[c * 3 + 0], oy = vort[c * 3 + 1], oz = vort[c * 3 + 2];
                R gox = gom[c * 3 + 0], goy = gom[c * 3 + 1], goz = gom[c * 3 + 2];
                if (vs[c] != R(0)) {
                    gox += ox / vs[c] * gvs[c];
                    goy += oy / vs[c] * gvs[c];
                    goz += oz / vs[c] * gvs[c];
                }
                gox = gox / twoh;
                goy = goy / twoh;
                goz = goz / twoh;
                gW[c + sy] += gox; gW[c - sy] -= gox; gV[c + sz] -= gox; gV[c - sz] += gox;
                gU[c + sz] += goy; gU[c - sz] -= goy; gW[c + 1] -= goy; gW[c - 1] += goy;
                gV[c + 1] += goz; gV[c - 1] -= goz; gU[c + sy] -= goz; gU[c - sy] += goz;
            }
    /* centre = 0.5*(lo + hi) transposed */
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                size_t c = d.cell(i, j, k);
                gu[d.uix(i, j, k)] += R(0.5) * gU[c];
                gu[d.uix(i + 1, j, k)] += R(0.5) * gU[c];
                gv[d.vix(i, j, k)] += R(0.5) * gV[c];
                gv[d.vix(i, j + 1, k)] += R(0.5) * gV[c];
                gw[d.wix(i, j, k)] += R(0.5) * gW[c];
                gw[d.wix(i, j, k + 1)] += R(0.5) * gW[c];
            }
}

/* Cells a source overwrites (reinject()'s test). */
template <class R> static void source_mask(const Dims& d, const zqs_params& P, std::vector<uint8_t>& m) {
    m.assign(d.ncell(), 0);
    std::vector<R> T(d.ncell(), R(0)), rho(d.ncell(), R(0));
    zqs_params Q = P;
    for (int s = 0; s < Q.n_sources; s++) Q.sources[s].density = 1.0f;
    reinject(d, T.data(), rho.data(), Q);
    for (size_t c = 0; c < d.ncell(); c++) m[c] = rho[c] != R(0);
}

/* Adjoint of one step(F) from the state s0 at its start.  (gu..grho) = the
 * adjoint of the state after the step in, of s0 out; gF (nullable) += the
 * adjoint of F. */
template <class R>
int step_adjoint(const Dims& d, const R* u0, const R* v0, const R* w0, const R* T0, const R* rho0,
                 const uint8_t* occ, const zqs_params& P, const R* F, R* gu, R* gv, R* gw, R* gT, R* grho, R* gF) {
    if (P.adv_vel_mode != ZQS_ADV_VEL_INMAC_OUTMAC || P.adv_sca_mode != ZQS_ADV_SCA_MAC) return ZQS_EUNSUPPORTED;
    const size_t n = d.ncell();
    /* forward intermediates */
    std::vector<R> u2(u0, u0 + d.nu()), v2(v0, v0 + d.nv()), w2(w0, w0 + d.nw());
    std::vector<R> T1(T0, T0 + n), D1(rho0, rho0 + n);
    add_force(d, u2.data(), v2.data(), w2.data(), occ, T0, rho0, P, F);
    attenuate(d, u2.data(), v2.data(), w2.data(), T1.data(), D1.data(), occ, P);
    std::vector<R> u4(u2), v4(v2), w4(w2);
    int rc = advect_velocity(d, u4.data(), v4.data(), w4.data(), occ, P, P.adv_vel_mode, true);
    if (rc) return rc;
    project(d, u4.data(), v4.data(), w4.data(), occ, P, (R*)nullptr, (R*)nullptr, (zqs_stats*)nullptr);
    /* reinjection */
    std::vector<uint8_t> src;
    source_mask<R>(d, P, src);
    for (size_t c = 0; c < n; c++)
        if (src[c]) {
            gT[c] = R(0);
            grho[c] = R(0);
        }
    /* scalar advection: velocity u4, fields T1, D1 */
    std::vector<R> gT1(n, R(0)), gD1(n, R(0));
    advect_scalar_adjoint(d, u4.data(), v4.data(), w4.data(), occ, T1.data(), D1.data(), gT, grho, gT1.data(),
                          gD1.data(), gu, gv, gw, P);
    /* projection */
    project_adjoint(d, gu, gv, gw, occ, P);
    /* velocity advection */
    std::vector<R> gu2(d.nu()), gv2(d.nv()), gw2(d.nw());
    advect_velocity_adjoint(d, u2.data(), v2.data(), w2.data(), occ, P, gu, gv, gw, gu2.data(), gv2.data(),
                            gw2.data());
    /* attenuation */
    const R av = (R)P.vel_atten, at = (R)P.temp_atten, ad = (R)P.dens_atten;
    for (int k = 0; k <= d.D; k++)
        for (int j = 0; j <= d.H; j++)
            for (int i = 0; i <= d.W; i++) {
                if (j < d.H && k < d.D) {
                    size_t f = d.uix(i, j, k);
                    gu[f] = u_live(d, occ, i, j, k, true) ? av * gu2[f] : gu2[f];
                }
                if (i < d.W && k < d.D) {
                    size_t f = d.vix(i, j, k);
                    gv[f] = v_live(d, occ, i, j, k, true) ? av * gv2[f] : gv2[f];
                }
                if (i < d.W && j < d.H) {
                    size_t f = d.wix(i, j, k);
                    gw[f] = w_live(d, occ, i, j, k, true) ? av * gw2[f] : gw2[f];
                }
            }
    for (size_t c = 0; c < n; c++) {
        gT[c] = at * gT1[c];
        grho[c] = ad * gD1[c];
    }
    /* forces */
    add_force_adjoint(d, u0, v0, w0, occ, P, gu, gv, gw, gT, grho, gF);
    return ZQS_OK;
}

/* The control problem: L(F) = sum_c (rho_n[c] - target[c])^2 after nsteps
 * steps of step(F) from the given state.  With gF non-null, the gradient
 * dL/dF is stored there (every step state is kept; test sizes only) and,
 * when g0 is non-null, the adjoint of the initial state (u,v,w,T,rho packed
 * in that order) too. */
template <class R>
int control_loss(const Dims& d, const R* u, const R* v, const R* w, const R* T, const R* rho, const uint8_t* occ,
                 const zqs_params& P, int nsteps, const R* F, const R* target, double* loss, R* gF, R* g0) {
    const size_t n = d.ncell(), nu = d.nu(), nv = d.nv(), nw = d.nw();
    const size_t ns = nu + nv + nw + 2 * n;
    std::vector<R> s(u, u + nu);
    s.insert(s.end(), v, v + nv);
    s.insert(s.end(), w, w + nw);
    s.insert(s.end(), T, T + n);
    s.insert(s.end(), rho, rho + n);
    std::vector<R> hist;
    if (gF) hist.resize(ns * (size_t)nsteps);
    for (int t = 0; t < nsteps; t++) {
        if (gF) std::copy(s.begin(), s.end(), hist.begin() + ns * (size_t)t);
        R* p = s.data();
        int rc = step(d, p, p + nu, p + nu + nv, p + nu + nv + nw, p + nu + nv + nw + n, occ, P, (R*)nullptr, F);
        if (rc) return rc;
    }
    const R* rn = s.data() + nu + nv + nw + n;
    double L = 0.0;
    for (size_t c = 0; c < n; c++) {
        double e = (double)rn[c] - (double)target[c];
        L += e * e;
    }
    *loss = L;
    if (!gF) return ZQS_OK;
    std::fill(gF, gF + 3 * n, R(0));
    std::vector<R> g(ns, R(0));
    for (size_t c = 0; c < n; c++) g[nu + nv + nw + n + c] = R(2) * (rn[c] - target[c]);
    for (int t = nsteps - 1; t >= 0; t--) {
        const R* p = hist.data() + ns * (size_t)t;
        R* q = g.data();
        int rc = step_adjoint(d, p, p + nu, p + nu + nv, p + nu + nv + nw, p + nu + nv + nw + n, occ, P, F, q,
                              q + nu, q + nu + nv, q + nu + nv + nw, q + nu + nv + nw + n, gF);
        if (rc) return rc;
    }
    if (g0) std::copy(g.begin(), g.end(), g0);
    return ZQS_OK;
}

/* Headless ray march of a dense density volume: the viewer's fragment shader
 * (SampleSmokeGUI/raycastingshader.h:10-70) per pixel, py from the bottom
 * row, (0, 0, 0, 1) where the ray misses the box.  The 3D texture is read as
 * GL_LINEAR with GL_CLAMP: coordinates clamped to [0, 1], texel centres at
 * (i + 0.5) / n, zero outside, exact trilinear weights a + t (b - a) in x,
 * then y, then z.  Every expression keeps the shader's order of operations. */
template <class R>
void render(const R* vol, int W, int H, int D, const zqs_camera& c, R* out) {
    auto at = [&](int i, int j, int k) -> R {
        if (i < 0 || i >= W || j < 0 || j >= H || k < 0 || k >= D) return R(0);
        return vol[((size_t)k * H + j) * W + i];
    };
    auto lerp = [](R a, R b, R t) { return a + t * (b - a); };
    auto sample = [&](R s, R t, R r) -> R {
        s = std::fmin(std::fmax(s, R(0)), R(1));  // fmax/fmin: a NaN coordinate clamps to 0
        t = std::fmin(std::fmax(t, R(0)), R(1));
        r = std::fmin(std::fmax(r, R(0)), R(1));
        const R fx = s * (R)W - R(0.5), fy = t * (R)H - R(0.5), fz = r * (R)D - R(0.5);
        const R x0 = std::floor(fx), y0 = std::floor(fy), z0 = std::floor(fz);
        const R ax = fx - x0, ay = fy - y0, az = fz - z0;
        const int i = (int)x0, j = (int)y0, k = (int)z0;
        const R e00 = lerp(at(i, j, k), at(i + 1, j, k), ax), e10 = lerp(at(i, j + 1, k), at(i + 1, j + 1, k), ax);
        const R e01 = lerp(at(i, j, k + 1), at(i + 1, j, k + 1), ax);
        const R e11 = lerp(at(i, j + 1, k + 1), at(i + 1, j + 1, k + 1), ax);
        return lerp(lerp(e00, e10, ay), lerp(e01, e11, ay), az);
    };
    const R hw = ((R)c.width - R(1)) / R(2), hh = ((R)c.height - R(1)) / R(2);
    R m[9], eye[3], bmin[3], bmax[3], bsize[3];
    for (int q = 0; q < 9; q++) m[q] = (R)c.inv_view[q];
    for (int q = 0; q < 3; q++) {
        eye[q] = (R)c.eye[q];
        bmin[q] = (R)c.box_min[q];
        bmax[q] = (R)c.box_max[q];
        bsize[q] = (R)c.box_size[q];
    }
#pragma omp parallel for schedule(dynamic, 4)
    for (int py = 0; py < c.height; py++)
        for (int px = 0; px < c.width; px++) {
            R dx = ((R)px + R(0.5)) - hw, dy = ((R)py + R(0.5)) - hh, dz = -(R)c.focal;
            R len = std::sqrt((dx * dx + dy * dy) + dz * dz);
            dx = dx / len, dy = dy / len, dz = dz / len;
            R rx = (m[0] * dx + m[1] * dy) + m[2] * dz;
            R ry = (m[3] * dx + m[4] * dy) + m[5] * dz;
            R rz = (m[6] * dx + m[7] * dy) + m[8] * dz;
            len = std::sqrt((rx * rx + ry * ry) + rz * rz);
            rx = rx / len, ry = ry / len, rz = rz / len;
            const R ix = R(1) / rx, iy = R(1) / ry, iz = R(1) / rz;
            const R bx0 = ix * (bmin[0] - eye[0]), bx1 = ix * (bmax[0] - eye[0]);
            const R by0 = iy * (bmin[1] - eye[1]), by1 = iy * (bmax[1] - eye[1]);
            const R bz0 = iz * (bmin[2] - eye[2]), bz1 = iz * (bmax[2] - eye[2]);
            using std::fmax;
            using std::fmin;
            const R tminx = fmin(bx1, bx0), tminy = fmin(by1, by0), tminz = fmin(bz1, bz0);
            const R tmaxx = fmax(bx1, bx0), tmaxy = fmax(by1, by0), tmaxz = fmax(bz1, bz0);
            const R tnear = fmax(fmax(tminx, tminy), fmax(tminx, tminz));
            const R tfar = fmin(fmin(tmaxx, tmaxy), fmin(tmaxx, tmaxz));
            R* o = out + ((size_t)py * c.width + px) * 4;
            if (!(tfar > tnear)) {
                o[0] = o[1] = o[2] = R(0);
                o[3] = R(1);
                continue;
            }
            R sx = ((eye[0] + rx * tnear) - bmin[0]) / bsize[0];
            R sy = ((eye[1] + ry * tnear) - bmin[1]) / bsize[1];
            R sz = ((eye[2] + rz * tnear) - bmin[2]) / bsize[2];
            R steplen = (tfar - tnear) / (R)c.steps;
            const R qx = (steplen * rx) / bsize[0], qy = (steplen * ry) / bsize[1], qz = (steplen * rz) / bsize[2];
            steplen = steplen / bsize[0];
            R acc = R(0);
            for (int n = 0; n < c.steps; n++) {
                acc = acc + steplen * sample(sx, sy, sz);
                sx = sx + qx, sy = sy + qy, sz = sz + qz;
            }
            const R v = acc * (R)c.density_scale;
            o[0] = o[1] = o[2] = v;
            o[3] = std::exp(-v);
        }
}

}  // namespace zqo

/* ---------------------------------------------------------------------- */
/* extern "C" entry points for ctypes (suffix _f32 / _f64)                 */
/* ---------------------------------------------------------------------- */

#define ZQO_API extern "C" __attribute__((visibility("default")))

/* The sub-projection matrix of block edge s: rows (3 s^2 (s-1)) x cols (3 s^2 (s+1)) floats. */
ZQO_API int zqo_submatrix(int s, float* out, int cap) {
    if (s < 2) return -1;
    const std::vector<float> M = zqo::submatrix(s);
    if ((int)M.size() > cap) return -(int)M.size();
    std::copy(M.begin(), M.end(), out);
    return (int)M.size();
}

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
    ZQO_API int zqo_project_coarse_##SFX(int W, int H, int D, R* u, R* v, R* w, const uint8_t* occ,     \
                                         const zqs_params* P) {                                         \
        return zqo::project_coarse<R>(zqo::Dims{W, H, D}, u, v, w, occ, *P);                            \
    }                                                                                                   \
    ZQO_API void zqo_stamp_objects_##SFX(int W, int H, int D, uint8_t* occ, R* u, R* v, R* w,            \
                                         const zqs_object* objs, int n, int closed, const zqs_params* P) { \
        zqo::stamp_objects<R>(zqo::Dims{W, H, D}, occ, u, v, w, objs, n, closed, *P);              \
    }                                                                                                   \
    ZQO_API void zqo_render_##SFX(const R* vol, int W, int H, int D, const zqs_camera* cam, R* rgba) {    \
        zqo::render<R>(vol, W, H, D, *cam, rgba);                                                       \
    }                                                                                                   \
    ZQO_API void zqo_reinject_##SFX(int W, int H, int D, R* T, R* rho, const zqs_params* P) {           \
        zqo::reinject<R>(zqo::Dims{W, H, D}, T, rho, *P);                                               \
    }                                                                                                   \
    ZQO_API void zqo_apply_advect_result_##SFX(int W, int H, int D, const uint8_t* occ, const R* au,    \
                                               const R* av, const R* aw, R* u, R* v, R* w,              \
                                               int is_open) {                                           \
        zqo::apply_advect_result<R>(zqo::Dims{W, H, D}, occ, au, av, aw, u, v, w, is_open != 0);        \
    }                                                                                                   \
    ZQO_API int zqo_step_ctrl_##SFX(int W, int H, int D, R* u, R* v, R* w, R* T, R* rho,                \
                                    const uint8_t* occ, const zqs_params* P, int nsteps, const R* F) {  \
        for (int s = 0; s < nsteps; s++) {                                                              \
            int rc = zqo::step<R>(zqo::Dims{W, H, D}, u, v, w, T, rho, occ, *P, (R*)nullptr, F);         \
            if (rc) return rc;                                                                          \
        }                                                                                               \
        return 0;                                                                                       \
    }                                                                                                   \
    ZQO_API void zqo_project_adjoint_##SFX(int W, int H, int D, R* gu, R* gv, R* gw, const uint8_t* occ, \
                                           const zqs_params* P) {                                       \
        zqo::project_adjoint<R>(zqo::Dims{W, H, D}, gu, gv, gw, occ, *P);                               \
    }                                                                                                   \
    ZQO_API void zqo_advect_scalar_adjoint_##SFX(int W, int H, int D, const R* u, const R* v, const R* w, \
                                                 const uint8_t* occ, const R* Tin, const R* Din,        \
                                                 const R* gTout, const R* gDout, R* gTin, R* gDin,      \
                                                 R* gu, R* gv, R* gw, const zqs_params* P) {            \
        zqo::advect_scalar_adjoint<R>(zqo::Dims{W, H, D}, u, v, w, occ, Tin, Din, gTout, gDout, gTin,   \
                                      gDin, gu, gv, gw, *P);                                            \
    }                                                                                                   \
    ZQO_API void zqo_advect_velocity_adjoint_##SFX(int W, int H, int D, const R* u, const R* v,          \
                                                   const R* w, const uint8_t* occ, const zqs_params* P, \
                                                   const R* gu3, const R* gv3, const R* gw3, R* gu2,    \
                                                   R* gv2, R* gw2) {                                    \
        zqo::advect_velocity_adjoint<R>(zqo::Dims{W, H, D}, u, v, w, occ, *P, gu3, gv3, gw3, gu2, gv2,  \
                                        gw2);                                                           \
    }                                                                                                   \
    ZQO_API void zqo_add_force_ctrl_##SFX(int W, int H, int D, R* u, R* v, R* w, const uint8_t* occ,     \
                                          const R* T, const R* rho, const zqs_params* P, const R* F) {  \
        zqo::add_force<R>(zqo::Dims{W, H, D}, u, v, w, occ, T, rho, *P, F);                              \
    }                                                                                                   \
    ZQO_API void zqo_add_force_adjoint_##SFX(int W, int H, int D, const R* u, const R* v, const R* w,    \
                                             const uint8_t* occ, const zqs_params* P, R* gu, R* gv,     \
                                             R* gw, R* gT, R* grho, R* gF) {                            \
        zqo::add_force_adjoint<R>(zqo::Dims{W, H, D}, u, v, w, occ, *P, gu, gv, gw, gT, grho, gF);      \
    }                                                                                                   \
    ZQO_API int zqo_step_adjoint_##SFX(int W, int H, int D, const R* u, const R* v, const R* w,          \
                                       const R* T, const R* rho, const uint8_t* occ, const zqs_params* P, \
                                       const R* F, R* gu, R* gv, R* gw, R* gT, R* grho, R* gF) {        \
        return zqo::step_adjoint<R>(zqo::Dims{W, H, D}, u, v, w, T, rho, occ, *P, F, gu, gv, gw, gT,    \
                                    grho, gF);                                                          \
    }                                                                                                   \
    ZQO_API int zqo_control_loss_##SFX(int W, int H, int D, const R* u, const R* v, const R* w,          \
                                       const R* T, const R* rho, const uint8_t* occ, const zqs_params* P, \
                                       int nsteps, const R* F, const R* target, double* loss, R* gF,    \
                                       R* g0) {                                                         \
        return zqo::control_loss<R>(zqo::Dims{W, H, D}, u, v, w, T, rho, occ, *P, nsteps, F, target,    \
                                    loss, gF, g0);                                                      \
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
