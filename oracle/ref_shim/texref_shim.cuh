// Software stand-in for the legacy texture references of ZQ_CUDA_Advection3D.cu.
// TEST INFRASTRUCTURE ONLY: force-included (nvcc -include) by oracle/build_ref.py
// when it compiles the reference's unmodified advection file into a device-only
// module, so that the reference's own advection kernels run on this GPU.
//
// Texture references (texture<T,3,mode>, cudaBindTextureToArray, tex3D on a
// reference) were removed in CUDA 12; the reference declares eleven of them at
// namespace scope (ZQ_CUDA_Advection3D.cu:10-20).  The macro below turns every
// such declaration into a __device__ variable of zq_texref<T,3,mode>, a plain
// struct the test harness fills through the module's global symbols: a pointer
// to a dense x-fastest copy of the bound data (the harness snapshots the data
// at bind time, as cudaMemcpy3D into a cudaArray does in the reference's
// cu_Copy_to_tex_* helpers, ZQ_CUDA_Advection3D.cu:654-993), its extents, and
// the filter and normalisation flags those helpers set.
//
// tex3D on a zq_texref follows the texture-fetch rules of the CUDA programming
// guide for the modes the reference uses:
//   * normalised coordinates: the texel-space coordinate is u * n;
//   * linear filtering: x_B = x - 0.5, i = floor(x_B), t = frac(x_B), the two
//     texels of each axis clamped to [0, n-1] (cudaAddressModeClamp);
//   * point filtering: i = floor(x) clamped to [0, n-1].
// The hardware computes the weights in 9-bit fixed point, which cannot be
// reproduced bit for bit; this stand-in computes them exactly in FP32, in the
// same form as the CPU oracle (coordinate clamped to [0, n-1] before the floor,
// lerp a + t*(b - a), x then y then z).  All shim arithmetic uses
// round-to-nearest intrinsics, so it is the same whatever contraction flags the
// reference's own code is compiled with.
//
// The float4 operators below stand in for the vector helper header the
// reference's ZQlibCuda build pulls in (component-wise float arithmetic).
#pragma once
#include <cuda_runtime.h>

template <class T, int dim, enum cudaTextureReadMode mode>
struct zq_texref {
    int normalized;                            // written by the reference's host code
    enum cudaTextureFilterMode filterMode;
    enum cudaTextureAddressMode addressMode[3];
    int linear;                                // harness: 1 linear filtering, 0 point
    const T* data;                             // harness: dense x-fastest nx*ny*nz
    int nx, ny, nz;
    int pad;
};

// Every `texture<...> name;` of the reference becomes a device variable.
#define texture __device__ zq_texref

// The host wrappers of the reference bind and unbind through these; they are
// declared only so the file parses (no host code of the module is compiled).
template <class T, int d, enum cudaTextureReadMode m>
cudaError_t cudaBindTextureToArray(const zq_texref<T, d, m>&, cudaArray_const_t, const cudaChannelFormatDesc&);
template <class T, int d, enum cudaTextureReadMode m>
cudaError_t cudaUnbindTexture(const zq_texref<T, d, m>&);

namespace zq_texref_impl {

struct Ax {
    int i0, i1;
    float t;
};

__device__ __forceinline__ float texel_coord(float u, int n, int normalized) {
    return normalized ? __fmul_rn(u, (float)n) : u;
}

__device__ __forceinline__ Ax lin_axis(float u, int n, int normalized) {
    float g = __fsub_rn(texel_coord(u, n, normalized), 0.5f);
    g = fminf(fmaxf(g, 0.0f), (float)(n - 1));
    const float f = floorf(g);
    Ax a;
    a.t = __fsub_rn(g, f);
    a.i0 = (int)f;
    a.i1 = a.i0 + 1 < n ? a.i0 + 1 : n - 1;
    return a;
}

__device__ __forceinline__ int pt_axis(float u, int n, int normalized) {
    const float g = floorf(texel_coord(u, n, normalized));
    int i = (g != g) ? 0 : (g < 0.0f ? 0 : (g > (float)(n - 1) ? n - 1 : (int)g));
    return i;
}

__device__ __forceinline__ float lerp(float a, float b, float t) { return __fadd_rn(a, __fmul_rn(t, __fsub_rn(b, a))); }
__device__ __forceinline__ float4 lerp(float4 a, float4 b, float t) {
    return make_float4(lerp(a.x, b.x, t), lerp(a.y, b.y, t), lerp(a.z, b.z, t), lerp(a.w, b.w, t));
}

template <class T>
__device__ __forceinline__ T at(const T* p, int i, int j, int k, int nx, int ny) {
    return p[((size_t)k * ny + j) * nx + i];
}

}  // namespace zq_texref_impl

template <class T, enum cudaTextureReadMode M>
__device__ T tex3D(const zq_texref<T, 3, M>& t, float x, float y, float z) {
    using namespace zq_texref_impl;
    const int nx = t.nx, ny = t.ny, nz = t.nz;
    if (!t.linear) return at(t.data, pt_axis(x, nx, t.normalized), pt_axis(y, ny, t.normalized),
                             pt_axis(z, nz, t.normalized), nx, ny);
    const Ax ax = lin_axis(x, nx, t.normalized), ay = lin_axis(y, ny, t.normalized), az = lin_axis(z, nz, t.normalized);
    const T* p = t.data;
    const T c00 = lerp(at(p, ax.i0, ay.i0, az.i0, nx, ny), at(p, ax.i1, ay.i0, az.i0, nx, ny), ax.t);
    const T c10 = lerp(at(p, ax.i0, ay.i1, az.i0, nx, ny), at(p, ax.i1, ay.i1, az.i0, nx, ny), ax.t);
    const T c01 = lerp(at(p, ax.i0, ay.i0, az.i1, nx, ny), at(p, ax.i1, ay.i0, az.i1, nx, ny), ax.t);
    const T c11 = lerp(at(p, ax.i0, ay.i1, az.i1, nx, ny), at(p, ax.i1, ay.i1, az.i1, nx, ny), ax.t);
    return lerp(lerp(c00, c10, ay.t), lerp(c01, c11, ay.t), az.t);
}

// unsigned char textures are only point-sampled by the reference (tex_occupy)
template <enum cudaTextureReadMode M>
__device__ unsigned char tex3D(const zq_texref<unsigned char, 3, M>& t, float x, float y, float z) {
    using namespace zq_texref_impl;
    return at(t.data, pt_axis(x, t.nx, t.normalized), pt_axis(y, t.ny, t.normalized), pt_axis(z, t.nz, t.normalized),
              t.nx, t.ny);
}

// component-wise float4 arithmetic used by the reference's kernels
__host__ __device__ __forceinline__ float4 operator*(float4 a, float b) {
    return make_float4(a.x * b, a.y * b, a.z * b, a.w * b);
}
__host__ __device__ __forceinline__ float4 operator/(float4 a, float b) {
    return make_float4(a.x / b, a.y / b, a.z / b, a.w / b);
}
__host__ __device__ __forceinline__ float4 operator-(float4 a, float4 b) {
    return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
__host__ __device__ __forceinline__ float4 operator-(float4 a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }
__host__ __device__ __forceinline__ void operator-=(float4& a, float4 b) {
    a.x -= b.x;
    a.y -= b.y;
    a.z -= b.z;
    a.w -= b.w;
}
