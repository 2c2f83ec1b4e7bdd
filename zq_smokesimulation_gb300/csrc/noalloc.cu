// Allocation-free projection entry point (zqs_project_sor_noalloc).
//
// Who needs it: callers that cannot ask the driver for memory at the moment
// they project -- a framework that has already reserved the whole GPU for its
// own pool, code running while a CUDA graph is being captured, or a runtime
// with no allocator of its own.  They already hold the velocity and the
// occupancy in device memory; this entry point projects them in place using a
// fixed working area that is part of the library image instead of cudaMalloc.
//
// The working area is one file-scope __device__ array.  In host code its name
// is only a stand-in, so its device address is looked up with
// cudaGetSymbolAddress, once per device, with that device current; kernels get
// the looked-up pointer.  Every call reuses the same array: the fields that
// must start at zero are cleared at the start of each call, and two calls
// that run at the same time on the GPU would overwrite each other's data.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/zqs_legacy.h"
#include "zqs_internal.h"

namespace zqs {

namespace {

constexpr long long kMaxElems = ZQS_NOALLOC_MAX_ELEMS;  // per padded field
constexpr size_t kFieldBytes = ((size_t)kMaxElems * 4 + 255) / 256 * 256;
constexpr size_t kFlagBytes = ((size_t)kMaxElems + 255) / 256 * 256;
constexpr long long kRedDoubles = 65536;                // FP64 reduction scratch
constexpr int kFloatFields = 6;                         // u, v, w, p, p2, div
constexpr size_t kScratchBytes = kFloatFields * kFieldBytes + kFlagBytes + (size_t)kRedDoubles * 8;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_zqs_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the fixed working area on the current device (looked up
// on the first call per device).
int scratch_address(void** out) {
    int dev = 0;
    ZQS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("zqs_project_sor_noalloc: device ordinal out of range");
        return ZQS_EINVAL;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_zqs_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "zqs_project_sor_noalloc: cudaGetSymbolAddress");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return ZQS_OK;
}

int dense_to_padded(float* dst, const float* src, const Layout& L, int nx, int ny, int nz, cudaStream_t s) {
    cudaMemcpy3DParms m = {};
    m.srcPtr = make_cudaPitchedPtr(const_cast<float*>(src), (size_t)nx * 4, (size_t)nx, (size_t)ny);
    m.dstPtr = make_cudaPitchedPtr(dst, (size_t)L.px * 4, (size_t)nx, (size_t)L.py);
    m.extent = make_cudaExtent((size_t)nx * 4, (size_t)ny, (size_t)nz);
    m.kind = cudaMemcpyDeviceToDevice;
    ZQS_CUDA_TRY(cudaMemcpy3DAsync(&m, s));
    return ZQS_OK;
}

int padded_to_dense(float* dst, const float* src, const Layout& L, int nx, int ny, int nz, cudaStream_t s) {
    cudaMemcpy3DParms m = {};
    m.srcPtr = make_cudaPitchedPtr(const_cast<float*>(src), (size_t)L.px * 4, (size_t)nx, (size_t)L.py);
    m.dstPtr = make_cudaPitchedPtr(dst, (size_t)nx * 4, (size_t)nx, (size_t)ny);
    m.extent = make_cudaExtent((size_t)nx * 4, (size_t)ny, (size_t)nz);
    m.kind = cudaMemcpyDeviceToDevice;
    ZQS_CUDA_TRY(cudaMemcpy3DAsync(&m, s));
    return ZQS_OK;
}

}  // namespace

}  // namespace zqs

using namespace zqs;

extern "C" ZQS_API int zqs_project_sor_noalloc(float* d_u, float* d_v, float* d_w, const uint8_t* d_occupy,
                                               int width, int height, int depth, int solver, int maxIter,
                                               float omega, void* stream) {
    if (!d_u || !d_v || !d_w || !d_occupy) {
        set_error("zqs_project_sor_noalloc: NULL pointer");
        return ZQS_EINVAL;
    }
    if (width < 2 || height < 2 || depth < 2 || maxIter < 0 ||
        (solver != ZQS_SOLVER_OPEN && solver != ZQS_SOLVER_CLOSED)) {
        set_error("zqs_project_sor_noalloc: dimensions must be >= 2, maxIter >= 0, solver open or closed");
        return ZQS_EINVAL;
    }
    Layout L;
    L.W = width;
    L.H = height;
    L.D = depth;
    L.px = ((width + 1) + 3) / 4 * 4;
    L.py = height + 1;
    L.pz = depth + 1;
    L.plane = (long long)L.px * L.py;
    L.elems = L.plane * (L.pz + 2);
    if (L.elems > kMaxElems) {
        set_error("zqs_project_sor_noalloc: grid needs " + std::to_string(L.elems) +
                  " padded elements per field; the fixed working area holds " + std::to_string(kMaxElems) +
                  " ((W+1 rounded up to 4)*(H+1)*(D+3); 64x64x64 fits)");
        return ZQS_EINVAL;
    }
    const long long nblocks = (long long)((width + 31) / 32) * ((height + 7) / 8) * depth;
    if (2 * nblocks + 2 > kRedDoubles) {
        set_error("zqs_project_sor_noalloc: grid too tall for the fixed reduction area");
        return ZQS_EINVAL;
    }
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;

    // carve the fields out of the fixed area (each field pointer skips its guard plane)
    unsigned char* b = (unsigned char*)base;
    DevGrid g = {};
    g.L = L;
    float* fields[kFloatFields];
    for (int f = 0; f < kFloatFields; f++) fields[f] = (float*)(b + (size_t)f * kFieldBytes);
    g.u = fields[0] + L.plane;
    g.v = fields[1] + L.plane;
    g.w = fields[2] + L.plane;
    g.p = fields[3] + L.plane;
    g.p2 = fields[4] + L.plane;
    g.div = fields[5] + L.plane;
    g.flags = (uint8_t*)(b + (size_t)kFloatFields * kFieldBytes) + L.plane;
    g.red = (double*)(b + (size_t)kFloatFields * kFieldBytes + kFlagBytes);
    g.red_len = kRedDoubles;

    cudaStream_t s = (cudaStream_t)stream;
    // The previous call's contents are still there: clear every field whose
    // out-of-extent entries are read as zeros.
    for (int f = 0; f < kFloatFields; f++) ZQS_CUDA_TRY(cudaMemsetAsync(fields[f], 0, (size_t)L.elems * 4, s));
    if ((rc = dense_to_padded(g.u, d_u, L, width + 1, height, depth, s))) return rc;
    if ((rc = dense_to_padded(g.v, d_v, L, width, height + 1, depth, s))) return rc;
    if ((rc = dense_to_padded(g.w, d_w, L, width, height, depth + 1, s))) return rc;
    LaunchCounter lc;
    if ((rc = launch_build_flags(g, d_occupy, solver, s, lc))) return rc;

    zqs_params p;
    zqs_params_default(&p, width, height, depth);
    p.solver = solver;
    p.omega = omega;
    KParams kp;
    make_kparams(p, kp);
    SorConfig cfg;
    float* pfinal = nullptr;
    if ((rc = launch_project(g, kp, maxIter, cfg, s, lc, &pfinal))) return rc;
    if ((rc = padded_to_dense(d_u, g.u, L, width + 1, height, depth, s))) return rc;
    if ((rc = padded_to_dense(d_v, g.v, L, width, height + 1, depth, s))) return rc;
    if ((rc = padded_to_dense(d_w, g.w, L, width, height, depth + 1, s))) return rc;
    return ZQS_OK;
}
