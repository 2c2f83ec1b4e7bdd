// Headless ray march of the density: the volume fragment shader of the
// reference's viewer (SampleSmokeGUI/raycastingshader.h:10-70, uniforms from
// ZQ_SmokeGUI.cpp:711-752) as one CUDA thread per pixel writing RGBA floats
// into device memory.  No graphics API is involved.
//
// Per pixel (px, py), py counted from the bottom row as gl_FragCoord is:
//   d  = normalize(px + 0.5 - (w-1)/2, py + 0.5 - (h-1)/2, -focal)
//   d1 = normalize(invView * d)
//   slab test of the ray eye + t d1 against [boxMin, boxMax]
//   hit: `steps` samples from the entry point, intensity += steplen * rho(pos),
//        steplen = (tfar - tnear) / steps / boxSize.x; out = (v, v, v, exp(-v)),
//        v = intensity * densityScale
//   miss: (0, 0, 0, 1), the value that leaves the viewer's blend unchanged.
// The density is sampled as the viewer's 3D texture (GL_LINEAR, GL_CLAMP):
// texture coordinates clamped to [0, 1], texel centres at (i + 0.5) / n, texels
// outside the volume read 0 (the border colour).  The filter is exact
// trilinear interpolation a + t (b - a) in x, then y, then z, in FP32; the
// hardware filter's 8-bit weights are not reproduced.
#include <cmath>
#include <cstdint>
#include <string>

#include "zqs_capi.h"
#include "zqs_grid.h"

namespace zqs {

namespace {

constexpr int kMaxRaySteps = 1 << 16;

struct RayCam {
    int width, height, steps;
    float focal, hw, hh, dscale;
    float m[9], eye[3], bmin[3], bmax[3], bsize[3];
};

__device__ __forceinline__ float lerpf(float a, float b, float t) { return __fadd_rn(a, __fmul_rn(t, __fsub_rn(b, a))); }

// The density with a one-texel zero border, (W+2) x (H+2) x (D+2) floats, so
// that every texel a clamped sample touches (x in [-1, W]) is a plain load.
struct Volume {
    const float* __restrict__ f;  // texel (0, 0, 0) of the bordered copy
    int W, H, D;
    int sy, sz;  // row and plane strides of the bordered copy

    // GL_LINEAR with GL_CLAMP: s in [0, 1], u = s n - 0.5, border texels 0
    __device__ __forceinline__ float sample(float s, float t, float r) const {
        s = fminf(fmaxf(s, 0.0f), 1.0f);
        t = fminf(fmaxf(t, 0.0f), 1.0f);
        r = fminf(fmaxf(r, 0.0f), 1.0f);
        const float fx = __fsub_rn(__fmul_rn(s, (float)W), 0.5f);
        const float fy = __fsub_rn(__fmul_rn(t, (float)H), 0.5f);
        const float fz = __fsub_rn(__fmul_rn(r, (float)D), 0.5f);
        const float x0 = floorf(fx), y0 = floorf(fy), z0 = floorf(fz);
        const float ax = __fsub_rn(fx, x0), ay = __fsub_rn(fy, y0), az = __fsub_rn(fz, z0);
        const float* p = f + ((int)z0 * sz + (int)y0 * sy + (int)x0);
        const float c000 = __ldg(p), c100 = __ldg(p + 1);
        const float c010 = __ldg(p + sy), c110 = __ldg(p + sy + 1);
        const float c001 = __ldg(p + sz), c101 = __ldg(p + sz + 1);
        const float c011 = __ldg(p + sz + sy), c111 = __ldg(p + sz + sy + 1);
        const float e00 = lerpf(c000, c100, ax), e10 = lerpf(c010, c110, ax);
        const float e01 = lerpf(c001, c101, ax), e11 = lerpf(c011, c111, ax);
        return lerpf(lerpf(e00, e10, ay), lerpf(e01, e11, ay), az);
    }
};

__global__ void __launch_bounds__(256) k_raymarch(Volume V, RayCam C, float4* __restrict__ out) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    const int py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= C.width || py >= C.height) return;
    // eye-space direction through the pixel centre, normalised
    float dx = __fsub_rn(__fadd_rn((float)px, 0.5f), C.hw);
    float dy = __fsub_rn(__fadd_rn((float)py, 0.5f), C.hh);
    float dz = -C.focal;
    float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
    dx = __fdiv_rn(dx, len);
    dy = __fdiv_rn(dy, len);
    dz = __fdiv_rn(dz, len);
    // world direction
    const float* m = C.m;
    float rx = __fadd_rn(__fadd_rn(__fmul_rn(m[0], dx), __fmul_rn(m[1], dy)), __fmul_rn(m[2], dz));
    float ry = __fadd_rn(__fadd_rn(__fmul_rn(m[3], dx), __fmul_rn(m[4], dy)), __fmul_rn(m[5], dz));
    float rz = __fadd_rn(__fadd_rn(__fmul_rn(m[6], dx), __fmul_rn(m[7], dy)), __fmul_rn(m[8], dz));
    len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(rx, rx), __fmul_rn(ry, ry)), __fmul_rn(rz, rz)));
    rx = __fdiv_rn(rx, len);
    ry = __fdiv_rn(ry, len);
    rz = __fdiv_rn(rz, len);
    // slab test (intersectBox)
    const float ix = __fdiv_rn(1.0f, rx), iy = __fdiv_rn(1.0f, ry), iz = __fdiv_rn(1.0f, rz);
    const float bx0 = __fmul_rn(ix, __fsub_rn(C.bmin[0], C.eye[0])), bx1 = __fmul_rn(ix, __fsub_rn(C.bmax[0], C.eye[0]));
    const float by0 = __fmul_rn(iy, __fsub_rn(C.bmin[1], C.eye[1])), by1 = __fmul_rn(iy, __fsub_rn(C.bmax[1], C.eye[1]));
    const float bz0 = __fmul_rn(iz, __fsub_rn(C.bmin[2], C.eye[2])), bz1 = __fmul_rn(iz, __fsub_rn(C.bmax[2], C.eye[2]));
    const float tminx = fminf(bx1, bx0), tminy = fminf(by1, by0), tminz = fminf(bz1, bz0);
    const float tmaxx = fmaxf(bx1, bx0), tmaxy = fmaxf(by1, by0), tmaxz = fmaxf(bz1, bz0);
    const float tnear = fmaxf(fmaxf(tminx, tminy), fmaxf(tminx, tminz));
    const float tfar = fminf(fminf(tmaxx, tmaxy), fminf(tmaxx, tmaxz));
    float4 o = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    if (tfar > tnear) {
        float sx = __fdiv_rn(__fsub_rn(__fadd_rn(C.eye[0], __fmul_rn(rx, tnear)), C.bmin[0]), C.bsize[0]);
        float sy = __fdiv_rn(__fsub_rn(__fadd_rn(C.eye[1], __fmul_rn(ry, tnear)), C.bmin[1]), C.bsize[1]);
        float sz = __fdiv_rn(__fsub_rn(__fadd_rn(C.eye[2], __fmul_rn(rz, tnear)), C.bmin[2]), C.bsize[2]);
        float steplen = __fdiv_rn(__fsub_rn(tfar, tnear), (float)C.steps);
        const float qx = __fdiv_rn(__fmul_rn(steplen, rx), C.bsize[0]);
        const float qy = __fdiv_rn(__fmul_rn(steplen, ry), C.bsize[1]);
        const float qz = __fdiv_rn(__fmul_rn(steplen, rz), C.bsize[2]);
        steplen = __fdiv_rn(steplen, C.bsize[0]);
        float acc = 0.0f;
        for (int n = 0; n < C.steps; n++) {
            acc = __fadd_rn(acc, __fmul_rn(steplen, V.sample(sx, sy, sz)));
            sx = __fadd_rn(sx, qx);
            sy = __fadd_rn(sy, qy);
            sz = __fadd_rn(sz, qz);
        }
        const float v = __fmul_rn(acc, C.dscale);
        o = make_float4(v, v, v, expf(-v));
    }
    out[(size_t)py * C.width + px] = o;
}

// Bordered copy: out has (W+2) x (H+2) x (D+2) texels, 0 on the border.
__global__ void k_border_volume(const float* __restrict__ in, long long in_sy, long long in_sz, int W, int H, int D,
                                float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // bordered coordinates
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= W + 2 || j >= H + 2) return;
    const bool inside = i >= 1 && i <= W && j >= 1 && j <= H && k >= 1 && k <= D;
    out[((size_t)k * (H + 2) + j) * (W + 2) + i] =
        inside ? __ldg(in + (k - 1) * in_sz + (j - 1) * in_sy + (i - 1)) : 0.0f;
}

int check_camera(const zqs_camera* c, const char* fn) {
    if (!c || c->width <= 0 || c->height <= 0 || c->steps < 0 || c->steps > kMaxRaySteps ||
        (long long)c->width * c->height > (1LL << 31)) {
        set_error(std::string(fn) + ": bad camera (image size > 0, 0 <= steps <= 65536)");
        return ZQS_EINVAL;
    }
    return ZQS_OK;
}

// Density (strides in floats) -> bordered copy in stream-ordered scratch ->
// ray march -> scratch released on the stream.
int launch_raymarch(const float* dens, long long sy, long long sz, int W, int H, int D, const zqs_camera* c,
                    float* rgba, cudaStream_t s) {
    if ((reinterpret_cast<uintptr_t>(rgba) & 15) != 0) {
        set_error("render: the image must be 16-byte aligned (RGBA float4 stores)");
        return ZQS_EINVAL;
    }
    const long long texels = (long long)(W + 2) * (H + 2) * (D + 2);
    if (texels >= (1LL << 31)) {
        set_error("render: the volume is too large (over 2^31 texels with its border)");
        return ZQS_EINVAL;
    }
    float* vol = nullptr;
    ZQS_CUDA_TRY(cudaMallocAsync((void**)&vol, (size_t)texels * sizeof(float), s));
    {
        const dim3 b(32, 8, 1), g((W + 2 + 31) / 32, (H + 2 + 7) / 8, D + 2);
        k_border_volume<<<g, b, 0, s>>>(dens, sy, sz, W, H, D, vol);
    }
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) {
        cudaFreeAsync(vol, s);
        return cuda_fail(le, "k_border_volume");
    }
    // texel (-1, -1, -1) of the volume is element 0 of the copy
    Volume V{vol + (W + 2) * (H + 2) + (W + 2) + 1, W, H, D, W + 2, (W + 2) * (H + 2)};
    RayCam C;
    C.width = c->width;
    C.height = c->height;
    C.steps = c->steps;
    C.focal = c->focal;
    C.hw = ((float)c->width - 1.0f) / 2.0f;
    C.hh = ((float)c->height - 1.0f) / 2.0f;
    C.dscale = c->density_scale;
    for (int q = 0; q < 9; q++) C.m[q] = c->inv_view[q];
    for (int q = 0; q < 3; q++) {
        C.eye[q] = c->eye[q];
        C.bmin[q] = c->box_min[q];
        C.bmax[q] = c->box_max[q];
        C.bsize[q] = c->box_size[q];
    }
    const dim3 b(16, 16, 1), g((c->width + 15) / 16, (c->height + 15) / 16, 1);
    k_raymarch<<<g, b, 0, s>>>(V, C, reinterpret_cast<float4*>(rgba));
    le = cudaGetLastError();
    cudaFreeAsync(vol, s);
    if (le != cudaSuccess) return cuda_fail(le, "k_raymarch");
    return ZQS_OK;
}

}  // namespace

}  // namespace zqs

using namespace zqs;

extern "C" ZQS_API void zqs_camera_default(zqs_camera* c, int image_width, int image_height, int W, int H, int D) {
    if (!c) return;
    // the viewer's start-up view (ZQ_SmokeGUI.cpp:10-17, 34, 49, 250-253, 536-537,
    // 711-752): fovy 40, gluLookAt from (0, 0, 2) to the origin with y up and no
    // scene rotation, a box of height 1 with the volume's aspect, 300 samples
    const float fovy = 40.0f;
    c->width = image_width;
    c->height = image_height;
    c->focal = (float)(image_height / 2.0 / std::atan(fovy / 360.0f * M_PI));
    const float m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int q = 0; q < 9; q++) c->inv_view[q] = m[q];
    c->eye[0] = 0.0f;
    c->eye[1] = 0.0f;
    c->eye[2] = 2.0f;
    const float ylen = 1.0f;
    const float xlen = H > 0 ? (float)W / H * ylen : 1.0f;
    const float zlen = H > 0 ? (float)D / H * ylen : 1.0f;
    const float len[3] = {xlen, ylen, zlen};
    for (int q = 0; q < 3; q++) {
        c->box_min[q] = (float)(-0.5 * len[q]);
        c->box_max[q] = (float)(0.5 * len[q]);
        c->box_size[q] = len[q];
    }
    c->steps = 300;
    c->density_scale = 1.0f;
}

extern "C" ZQS_API int zqs_render_density(const float* density, int W, int H, int D, const zqs_camera* cam,
                                          float* rgba, void* stream) {
    if (!density || !rgba || W <= 0 || H <= 0 || D <= 0) {
        set_error("zqs_render_density: bad arguments");
        return ZQS_EINVAL;
    }
    int rc = check_camera(cam, "zqs_render_density");
    if (rc) return rc;
    return launch_raymarch(density, W, (long long)W * H, W, H, D, cam, rgba, (cudaStream_t)stream);
}

extern "C" ZQS_API int zqs_grid_render(zqs_grid* g, const zqs_camera* cam, float* rgba, void* stream) {
    if (!g || !rgba) {
        set_error("zqs_grid_render: bad arguments");
        return ZQS_EINVAL;
    }
    int rc = check_camera(cam, "zqs_grid_render");
    if (rc) return rc;
    const Layout& L = g->g.L;
    return launch_raymarch(g->g.rho, L.px, (long long)L.plane, L.W, L.H, L.D, cam, rgba, g->pick(stream));
}
