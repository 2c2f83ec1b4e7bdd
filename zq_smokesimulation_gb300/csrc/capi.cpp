// Host implementation of the handle-based C ABI (include/zqs_capi.h).
//
// A zqs_grid owns one device allocation holding every field in the padded
// layout (zqs_internal.h), its own non-blocking stream, the per-step CUDA
// graphs and the parameters.  The step replays a captured graph: one graph per
// (velocity buffer, scalar buffer) parity, rebuilt when parameters or the SOR
// configuration change.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>

#include "zqs_coarse.h"
#include "zqs_grid.h"

namespace zqs {

static thread_local std::string g_last_error;

// zqs_debug_fail_alloc: the allocation that is due to fail counts down to 0
// (-1: none).
static std::atomic<long long> g_alloc_fail_in{-1};

cudaError_t dev_alloc_raw(void** p, size_t bytes) {
    long long n = g_alloc_fail_in.load(std::memory_order_relaxed);
    while (n >= 0) {
        if (g_alloc_fail_in.compare_exchange_weak(n, n - 1, std::memory_order_relaxed)) {
            if (n == 0) {
                *p = nullptr;
                return cudaErrorMemoryAllocation;
            }
            break;
        }
    }
    return cudaMalloc(p, bytes);
}

void set_error(const std::string& msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char* what) {
    set_error(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
    return e == cudaErrorMemoryAllocation ? ZQS_ENOMEM : ZQS_ECUDA;
}

static bool is_pow2(float h) {
    if (!(h > 0.0f) || !std::isfinite(h)) return false;
    int e;
    float m = std::frexp(h, &e);
    return m == 0.5f;
}

int make_kparams(const zqs_params& p, KParams& kp) {
    kp.h = p.voxel_size;
    kp.dt = p.step_time;
    kp.dt_sub = (float)p.step_time / (float)p.substeps;  // Utils3D:2155
    kp.inv_h = is_pow2(p.voxel_size) ? 1.0f / p.voxel_size : 0.0f;
    kp.substeps = p.substeps;
    kp.full = p.backtrace_full ? 1 : 0;
    kp.cc = p.confine * p.voxel_size;
    kp.twoh = 2.0f * p.voxel_size;
    kp.beta = p.buoyancy;
    kp.alpha = p.gravity;
    kp.tamb = p.tamb;
    kp.vel_atten = p.vel_atten;
    kp.temp_atten = p.temp_atten;
    kp.dens_atten = p.dens_atten;
    kp.omega = p.omega;
    kp.om1 = 1.0f - p.omega;
    kp.solver = p.solver;
    kp.mean_override = 0;
    kp.mean_value = 0.0f;
    kp.fext = nullptr;
    return ZQS_OK;
}

int validate_params(const zqs_params& p) {
    if (!(p.voxel_size > 0.0f) || !std::isfinite(p.voxel_size)) {
        set_error("voxel_size must be a positive finite number");
        return ZQS_EINVAL;
    }
    if (!std::isfinite(p.step_time)) {
        set_error("step_time must be finite");
        return ZQS_EINVAL;
    }
    if (p.substeps < 1) {
        set_error("substeps must be >= 1");
        return ZQS_EINVAL;
    }
    if (p.sor_iters < 0) {
        set_error("sor_iters must be >= 0");
        return ZQS_EINVAL;
    }
    if (p.solver != ZQS_SOLVER_OPEN && p.solver != ZQS_SOLVER_CLOSED && p.solver != ZQS_SOLVER_COARSE_OPEN) {
        set_error("solver must be ZQS_SOLVER_OPEN, ZQS_SOLVER_CLOSED or ZQS_SOLVER_COARSE_OPEN");
        return ZQS_EINVAL;
    }
    if (p.adv_vel_mode < 0 || p.adv_vel_mode > 5 || p.adv_sca_mode < 0 || p.adv_sca_mode > 3) {
        set_error("advection mode out of range");
        return ZQS_EINVAL;
    }
    if (p.n_sources < 0 || p.n_sources > ZQS_MAX_SOURCES) {
        set_error("n_sources must be in [0, 16]");
        return ZQS_EINVAL;
    }
    for (int s = 0; s < p.n_sources; s++)
        if (p.sources[s].shape != ZQS_SOURCE_BOX && p.sources[s].shape != ZQS_SOURCE_SPHERE) {
            set_error("source shape must be ZQS_SOURCE_BOX or ZQS_SOURCE_SPHERE");
            return ZQS_EINVAL;
        }
    return ZQS_OK;
}

}  // namespace zqs

using namespace zqs;

namespace zqs {
// Internal hooks for the legacy shims (same library).
DevGrid& grid_dev(zqs_grid* g) { return g->g; }
KParams& grid_kparams(zqs_grid* g) { return g->kp; }
cudaStream_t grid_stream(zqs_grid* g) { return g->own; }
void grid_swap_velocity(zqs_grid* g) { g->swap_velocity(); }
void grid_swap_scalars(zqs_grid* g) { g->swap_scalars(); }
float*& grid_p_last(zqs_grid* g) { return g->p_last; }
SorConfig& grid_sor(zqs_grid* g) { return g->sor; }
}  // namespace zqs

namespace {

Layout make_layout(int W, int H, int D) {
    Layout L;
    L.W = W;
    L.H = H;
    L.D = D;
    L.px = ((W + 1) + 3) / 4 * 4;
    L.py = H + 1;
    L.pz = D + 1;
    L.plane = (long long)L.px * L.py;
    L.elems = L.plane * (L.pz + 2);
    return L;
}

// (rows, row elements, planes) of a field in the reference layout.
bool field_shape(const Layout& L, int field, int& nx, int& ny, int& nz, size_t& esize) {
    nx = L.W;
    ny = L.H;
    nz = L.D;
    esize = 4;
    switch (field) {
        case ZQS_FIELD_U: nx = L.W + 1; return true;
        case ZQS_FIELD_V: ny = L.H + 1; return true;
        case ZQS_FIELD_W: nz = L.D + 1; return true;
        case ZQS_FIELD_TEMPERATURE:
        case ZQS_FIELD_DENSITY:
        case ZQS_FIELD_PRESSURE:
        case ZQS_FIELD_DIVERGENCE: return true;
        case ZQS_FIELD_OCCUPANCY: esize = 1; return true;
        default: return false;
    }
}

float* field_ptr(zqs_grid* g, int field) {
    switch (field) {
        case ZQS_FIELD_U: return g->g.u;
        case ZQS_FIELD_V: return g->g.v;
        case ZQS_FIELD_W: return g->g.w;
        case ZQS_FIELD_TEMPERATURE: return g->g.T;
        case ZQS_FIELD_DENSITY: return g->g.rho;
        case ZQS_FIELD_PRESSURE: return g->p_last ? g->p_last : g->g.p;
        case ZQS_FIELD_DIVERGENCE: return g->g.div;
        default: return nullptr;
    }
}

int copy3d(void* dst, size_t dpitch, size_t dysize, const void* src, size_t spitch, size_t sysize, size_t rowbytes,
           size_t rows, size_t planes, cudaMemcpyKind kind, cudaStream_t s) {
    cudaMemcpy3DParms m;
    memset(&m, 0, sizeof(m));
    m.srcPtr = make_cudaPitchedPtr(const_cast<void*>(src), spitch, rowbytes, sysize);
    m.dstPtr = make_cudaPitchedPtr(dst, dpitch, rowbytes, dysize);
    m.extent = make_cudaExtent(rowbytes, rows, planes);
    m.kind = kind;
    ZQS_CUDA_TRY(cudaMemcpy3DAsync(&m, s));
    return ZQS_OK;
}

// Dense device buffer of at least n floats for host transfers (grown on
// demand).  Transfers on different streams share it: each use waits for the
// previous one (stage_ev, recorded by stage_done) on the device.
int host_stage(zqs_grid* g, size_t n, cudaStream_t s, float** out) {
    if (!g->stage_ev) ZQS_CUDA_TRY(cudaEventCreateWithFlags(&g->stage_ev, cudaEventDisableTiming));
    if (n > g->stage_cap) {
        ZQS_CUDA_TRY(cudaEventSynchronize(g->stage_ev));
        if (g->stage) cudaFree(g->stage);
        g->stage = nullptr;
        g->stage_cap = 0;
        ZQS_CUDA_TRY(dev_alloc(&g->stage, n * sizeof(float)));
        g->stage_cap = n;
    }
    ZQS_CUDA_TRY(cudaStreamWaitEvent(s, g->stage_ev, 0));
    *out = g->stage;
    return ZQS_OK;
}

int stage_done(zqs_grid* g, cudaStream_t s) {
    ZQS_CUDA_TRY(cudaEventRecord(g->stage_ev, s));
    return ZQS_OK;
}

}  // namespace

extern "C" {

ZQS_API int zqs_version(void) { return ZQS_VERSION; }

ZQS_API const char* zqs_last_error(void) { return zqs::g_last_error.c_str(); }

ZQS_API void zqs_params_default(zqs_params* p, int W, int H, int D) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->voxel_size = (float)(1.0 / (double)W);  // Utils3D:323
    p->step_time = 0.01f;
    p->substeps = 20;
    p->confine = 0.0f;
    p->buoyancy = 1.0f;
    p->gravity = 0.0f;
    p->tamb = 10.0f;
    p->vel_atten = 1.0f;
    p->temp_atten = 1.0f;
    p->dens_atten = 1.0f;
    p->solver = ZQS_SOLVER_OPEN;
    p->sor_iters = 100;
    p->omega = 1.0f;
    p->adv_vel_mode = ZQS_ADV_VEL_INMAC_OUTMAC;
    p->adv_sca_mode = ZQS_ADV_SCA_MAC;
    p->backtrace_full = 0;
    p->sub_size = 4;  // Utils3D:18 (subSize)
    p->n_sources = 1;
    zqs_source& s = p->sources[0];  // Utils3D:31-40, unit coordinates times W/H/D in float
    s.shape = ZQS_SOURCE_BOX;
    s.cx = 0.5f * (float)W;
    s.cy = 0.1f * (float)H;
    s.cz = 0.5f * (float)D;
    s.hx = 0.1f * (float)W;
    s.hy = 0.05f * (float)H;
    s.hz = 0.1f * (float)D;
    s.density = 1.0f;
    s.temperature = 10.0f * 20.0f;
}

ZQS_API int zqs_grid_create(zqs_grid** out, int W, int H, int D) {
    if (!out) {
        set_error("zqs_grid_create: out is NULL");
        return ZQS_EINVAL;
    }
    *out = nullptr;
    if (W < 2 || H < 2 || D < 2) {
        set_error("zqs_grid_create: every dimension must be >= 2");
        return ZQS_EINVAL;
    }
    Layout L = make_layout(W, H, D);
    if (L.elems >= (1LL << 31) - 1) {
        set_error("zqs_grid_create: grid too large for 32-bit indexing");
        return ZQS_EINVAL;
    }
    zqs_grid* g = new zqs_grid();
    g->g.L = L;
    // 13 float fields + 5 float4 fields (2 temporaries, 3 velocity quads) + flags + FP64 scratch
    const size_t fbytes = (size_t)L.elems * 4;
    const size_t nflt = 13;
    const long long nblocks = (long long)((W + 31) / 32) * ((H + 7) / 8) * D;
    g->g.red_len = 3 * nblocks + 16;
    size_t total = nflt * fbytes + 5 * (size_t)L.elems * 16 + (((size_t)L.elems + 255) / 256) * 256 +
                   (size_t)g->g.red_len * 8 + 256;
    cudaError_t e = dev_alloc(&g->base, total);
    if (e != cudaSuccess) {
        delete g;
        return cuda_fail(e, "zqs_grid_create: cudaMalloc");
    }
    e = dev_alloc(&g->occ_dense, (size_t)W * H * D);
    if (e != cudaSuccess) {
        cudaFree(g->base);
        delete g;
        return cuda_fail(e, "zqs_grid_create: cudaMalloc(occupancy)");
    }
    e = cudaStreamCreateWithFlags(&g->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaFree(g->occ_dense);
        cudaFree(g->base);
        delete g;
        return cuda_fail(e, "zqs_grid_create: cudaStreamCreate");
    }
    e = cudaMemsetAsync(g->base, 0, total, g->own);
    if (e == cudaSuccess) e = cudaMemsetAsync(g->occ_dense, 0, (size_t)W * H * D, g->own);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->own);
    if (e != cudaSuccess) {
        int rc = cuda_fail(e, "zqs_grid_create: clear");
        cudaStreamDestroy(g->own);
        cudaFree(g->occ_dense);
        cudaFree(g->base);
        delete g;
        return rc;
    }
    int prc = sor_prepare();
    if (prc) {
        cudaStreamDestroy(g->own);
        cudaFree(g->occ_dense);
        cudaFree(g->base);
        delete g;
        return prc;
    }
    char* b = (char*)g->base;
    auto take_f = [&](void) -> float* {
        float* p = (float*)b + L.plane;  // skip the leading guard plane
        b += fbytes;
        return p;
    };
    g->g.u = take_f();
    g->g.v = take_f();
    g->g.w = take_f();
    g->g.u2 = take_f();
    g->g.v2 = take_f();
    g->g.w2 = take_f();
    g->g.T = take_f();
    g->g.rho = take_f();
    g->g.T2 = take_f();
    g->g.rho2 = take_f();
    g->g.p = take_f();
    g->g.p2 = take_f();
    g->g.div = take_f();
    g->g.t4a = (float4*)b + L.plane;
    b += (size_t)L.elems * 16;
    g->g.t4b = (float4*)b + L.plane;
    b += (size_t)L.elems * 16;
    g->g.qu = (float4*)b + L.plane;
    b += (size_t)L.elems * 16;
    g->g.qv = (float4*)b + L.plane;
    b += (size_t)L.elems * 16;
    g->g.qw = (float4*)b + L.plane;
    b += (size_t)L.elems * 16;
    g->g.flags = (uint8_t*)b + L.plane;
    b += (((size_t)L.elems + 255) / 256) * 256;
    g->g.red = (double*)b;
    *out = g;
    return ZQS_OK;
}

ZQS_API int zqs_grid_destroy(zqs_grid* g) {
    if (!g) return ZQS_OK;
    g->drop_graphs();
    if (g->own) cudaStreamSynchronize(g->own);
    cudaStreamDestroy(g->own);
    cudaFree(g->occ_dense);
    cudaFree(g->base);
    coarse_free(g->g.coarse);
    if (g->obj_mask) cudaFree(g->obj_mask);
    if (g->stage) cudaFree(g->stage);
    if (g->stage_ev) cudaEventDestroy(g->stage_ev);
    if (g->fext_base) cudaFree(g->fext_base);
    delete g;
    return ZQS_OK;
}

ZQS_API int zqs_grid_get_layout(const zqs_grid* g, zqs_grid_layout* out) {
    if (!g || !out) {
        set_error("zqs_grid_get_layout: NULL argument");
        return ZQS_EINVAL;
    }
    const Layout& L = g->g.L;
    out->W = L.W;
    out->H = L.H;
    out->D = L.D;
    out->pitch_x = L.px;
    out->rows = L.py;
    out->planes = L.pz;
    out->plane_elems = L.plane;
    out->field_elems = L.elems;
    return ZQS_OK;
}

ZQS_API int zqs_grid_set_params(zqs_grid* g, const zqs_params* p) {
    if (!g || !p) {
        set_error("zqs_grid_set_params: NULL argument");
        return ZQS_EINVAL;
    }
    int rc = validate_params(*p);
    if (rc) return rc;
    if (p->solver == ZQS_SOLVER_COARSE_OPEN) {
        rc = coarse_prepare(g->g.coarse, g->g.L, p->sub_size, g->coarse_tc);
        if (rc) return rc;
    } else {
        coarse_free(g->g.coarse);
    }
    bool solver_changed = !g->has_params || g->params.solver != p->solver;
    g->params = *p;
    make_kparams(*p, g->kp);
    if (g->fext_on) g->kp.fext = g->fext_base + g->g.L.plane;
    g->src.n = p->n_sources;
    for (int s = 0; s < p->n_sources; s++) g->src.s[s] = p->sources[s];
    g->has_params = true;
    g->drop_graphs();
    if (solver_changed && g->has_occ) {
        LaunchCounter lc;
        rc = launch_build_flags(g->g, g->occ_dense, p->solver, g->own, lc);
        if (rc) return rc;
        ZQS_CUDA_TRY(cudaStreamSynchronize(g->own));
    }
    return ZQS_OK;
}

ZQS_API int zqs_grid_get_params(const zqs_grid* g, zqs_params* p) {
    if (!g || !p) {
        set_error("zqs_grid_get_params: NULL argument");
        return ZQS_EINVAL;
    }
    if (!g->has_params) {
        set_error("zqs_grid_get_params: no parameters set");
        return ZQS_ENOTREADY;
    }
    *p = g->params;
    return ZQS_OK;
}

ZQS_API int zqs_grid_upload(zqs_grid* g, int field, const void* src, int src_on_device, void* stream) {
    if (!g || !src) {
        set_error("zqs_grid_upload: NULL argument");
        return ZQS_EINVAL;
    }
    const Layout& L = g->g.L;
    cudaStream_t s = g->pick(stream);
    int nx, ny, nz;
    size_t es;
    if (!field_shape(L, field, nx, ny, nz, es) || field == ZQS_FIELD_PRESSURE || field == ZQS_FIELD_DIVERGENCE) {
        set_error("zqs_grid_upload: field cannot be uploaded");
        return ZQS_EINVAL;
    }
    cudaMemcpyKind kind = src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (field == ZQS_FIELD_OCCUPANCY) {
        ZQS_CUDA_TRY(cudaMemcpyAsync(g->occ_dense, src, (size_t)L.W * L.H * L.D, kind, s));
        g->has_occ = true;
        LaunchCounter lc;
        int rc = launch_build_flags(g->g, g->occ_dense, g->has_params ? g->params.solver : ZQS_SOLVER_OPEN, s, lc);
        if (rc) return rc;
        g->drop_graphs();
        return ZQS_OK;
    }
    float* dst = field_ptr(g, field);
    if (!src_on_device) {
        // one contiguous host -> device copy into a dense staging buffer, then
        // the strided placement on the device (row-by-row host copies of the
        // padded layout run far below the link's bandwidth)
        const size_t n = (size_t)nx * ny * nz;
        float* st = nullptr;
        int rc = host_stage(g, n, s, &st);
        if (rc) return rc;
        ZQS_CUDA_TRY(cudaMemcpyAsync(st, src, n * sizeof(float), cudaMemcpyHostToDevice, s));
        rc = copy3d(dst, (size_t)L.px * 4, (size_t)L.py, st, (size_t)nx * 4, (size_t)ny, (size_t)nx * 4, ny, nz,
                    cudaMemcpyDeviceToDevice, s);
        return rc ? rc : stage_done(g, s);
    }
    return copy3d(dst, (size_t)L.px * 4, (size_t)L.py, src, (size_t)nx * 4, (size_t)ny, (size_t)nx * 4, ny, nz, kind,
                  s);
}

ZQS_API int zqs_grid_download(zqs_grid* g, int field, void* dst, int dst_on_device, void* stream) {
    if (!g || !dst) {
        set_error("zqs_grid_download: NULL argument");
        return ZQS_EINVAL;
    }
    const Layout& L = g->g.L;
    cudaStream_t s = g->pick(stream);
    int nx, ny, nz;
    size_t es;
    if (!field_shape(L, field, nx, ny, nz, es)) {
        set_error("zqs_grid_download: unknown field");
        return ZQS_EINVAL;
    }
    cudaMemcpyKind kind = dst_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (field == ZQS_FIELD_OCCUPANCY) {
        ZQS_CUDA_TRY(cudaMemcpyAsync(dst, g->occ_dense, (size_t)L.W * L.H * L.D, kind, s));
        return ZQS_OK;
    }
    const float* src = field_ptr(g, field);
    if (!dst_on_device) {
        // dense gather on the device, then one contiguous device -> host copy
        const size_t n = (size_t)nx * ny * nz;
        float* st = nullptr;
        int rc = host_stage(g, n, s, &st);
        if (rc) return rc;
        rc = copy3d(st, (size_t)nx * 4, (size_t)ny, src, (size_t)L.px * 4, (size_t)L.py, (size_t)nx * 4, ny, nz,
                    cudaMemcpyDeviceToDevice, s);
        if (rc) return rc;
        ZQS_CUDA_TRY(cudaMemcpyAsync(dst, st, n * sizeof(float), cudaMemcpyDeviceToHost, s));
        return stage_done(g, s);
    }
    return copy3d(dst, (size_t)nx * 4, (size_t)ny, src, (size_t)L.px * 4, (size_t)L.py, (size_t)nx * 4, ny, nz, kind,
                  s);
}

ZQS_API int zqs_grid_use_graph(zqs_grid* g, int enable) {
    if (!g) {
        set_error("zqs_grid_use_graph: NULL grid");
        return ZQS_EINVAL;
    }
    g->use_graph = enable != 0;
    if (!g->use_graph) g->drop_graphs();
    return ZQS_OK;
}

ZQS_API int zqs_grid_set_sor_config(zqs_grid* g, int temporal_depth, int split_colours) {
    if (!g || temporal_depth < 0 || temporal_depth > 4) {
        set_error("zqs_grid_set_sor_config: temporal_depth must be in [0, 4]");
        return ZQS_EINVAL;
    }
    g->sor.temporal_depth = temporal_depth;
    g->sor.split = split_colours ? 1 : 0;
    g->sor.variant = -1;
    g->drop_graphs();
    return ZQS_OK;
}

ZQS_API int zqs_grid_get_sor_choice(zqs_grid* g, int* variant, int* zchunk, float* us_per_iter, void* stream) {
    if (!g) return set_error("zqs_grid_get_sor_choice: NULL grid"), ZQS_EINVAL;
    int rc = g->ready();
    if (rc) return rc;
    rc = g->resolve_sor(g->pick(stream));
    if (rc) return rc;
    const SorConfig& e = g->sor_eff;
    if (variant) *variant = e.split ? -1 : (e.variant >= 0 ? e.variant : sor_default_variant(e.temporal_depth));
    if (zchunk) *zchunk = g->sor_eff.zchunk;
    if (us_per_iter) *us_per_iter = (g->sor_eff.variant == g->tuned.variant) ? g->tuned.us_per_iter : 0.0f;
    return ZQS_OK;
}

ZQS_API int zqs_grid_step(zqs_grid* g, int nsteps, void* stream) {
    if (!g || nsteps < 0) {
        set_error("zqs_grid_step: bad arguments");
        return ZQS_EINVAL;
    }
    int rc = g->ready();
    if (rc) return rc;
    cudaStream_t s = g->pick(stream);
    for (int n = 0; n < nsteps; n++) {
        if (!g->use_graph) {
            rc = g->resolve_sor(s);
            if (rc) return rc;
            LaunchCounter lc;
            rc = g->issue_step(s, lc);
            if (rc) return rc;
            g->step_launches = lc.n;
            continue;
        }
        const int key = g->vel_par * 2 + g->sca_par;
        if (!g->graph[key]) {
            rc = g->resolve_sor(s);  // before the capture: the tuner synchronises
            if (rc) return rc;
            // Capture on the grid's own stream: the launches read the current
            // buffer pointers, so capturing advances the parities; restore them.
            const int vp = g->vel_par, sp = g->sca_par;
            DevGrid saved = g->g;
            float* saved_p = g->p_last;
            LaunchCounter lc;
            ZQS_CUDA_TRY(cudaStreamBeginCapture(g->own, cudaStreamCaptureModeThreadLocal));
            rc = g->issue_step(g->own, lc);
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(g->own, &graph);
            float* captured_p = g->p_last;  // p and p2 never move, so this holds for every replay
            g->g = saved;
            g->vel_par = vp;
            g->sca_par = sp;
            g->p_last = saved_p;
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (e != cudaSuccess) return cuda_fail(e, "zqs_grid_step: cudaStreamEndCapture");
            e = cudaGraphInstantiate(&g->graph[key], graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                g->graph[key] = nullptr;
                return cuda_fail(e, "zqs_grid_step: cudaGraphInstantiate");
            }
            g->graph_launches[key] = lc.n;
            g->graph_p_last[key] = captured_p;
        }
        ZQS_CUDA_TRY(cudaGraphLaunch(g->graph[key], s));
        // advance the buffer roles exactly as issue_step does
        g->swap_velocity();
        g->swap_scalars();
        g->p_last = g->graph_p_last[key];
        g->step_launches = g->graph_launches[key];
    }
    return ZQS_OK;
}

ZQS_API int zqs_stage_add_force(zqs_grid* g, void* stream) {
    if (!g) return set_error("NULL grid"), ZQS_EINVAL;
    int rc = g->ready();
    if (rc) return rc;
    LaunchCounter lc;
    return launch_force(g->g, g->kp, false, g->pick(stream), lc);
}

ZQS_API int zqs_stage_attenuate(zqs_grid* g, void* stream) {
    if (!g) return set_error("NULL grid"), ZQS_EINVAL;
    int rc = g->ready();
    if (rc) return rc;
    LaunchCounter lc;
    return launch_attenuate(g->g, g->kp, g->pick(stream), lc);
}

ZQS_API int zqs_stage_advect_velocity(zqs_grid* g, int mode, int is_open, void* stream) {
    if (!g) return set_error("NULL grid"), ZQS_EINVAL;
    int rc = g->ready();
    if (rc) return rc;
    LaunchCounter lc;
    rc = launch_advect_velocity(g->g, g->kp, mode, is_open != 0, g->pick(stream), lc);
    if (rc) return rc;
    g->swap_velocity();
    return ZQS_OK;
}

ZQS_API int zqs_stage_project(zqs_grid* g, void* stream) {
    if (!g) return set_error("NULL grid"), ZQS_EINVAL;
    int rc = g->ready();
    if (rc) return rc;
    LaunchCounter lc;
    rc = g->resolve_sor(g->pick(stream));
    if (rc) return rc;
    return launch_project(g->g, g->kp, g->params.sor_iters, g->sor_eff, g->pick(stream), lc, &g->p_last);
}

ZQS_API int zqs_stage_advect_scalar(zqs_grid* g, int mode, void* stream) {
    if (!g) return set_error("NULL grid"), ZQS_EINVAL;
    int rc = g->ready();
    if (rc) return rc;
    LaunchCounter lc;
    rc = launch_advect_scalar(g->g, g->kp, mode, false, nullptr, g->pick(stream), lc);
    if (rc) return rc;
    g->swap_scalars();
    return ZQS_OK;
}

ZQS_API int zqs_stage_reinject(zqs_grid* g, void* stream) {
    if (!g) return set_error("NULL grid"), ZQS_EINVAL;
    int rc = g->ready();
    if (rc) return rc;
    LaunchCounter lc;
    return launch_reinject(g->g, g->src, g->pick(stream), lc);
}

ZQS_API int zqs_grid_mac_to_regular4(zqs_grid* g, float* vel4, int dst_on_device, void* stream) {
    if (!g || !vel4) return set_error("NULL argument"), ZQS_EINVAL;
    const Layout& L = g->g.L;
    cudaStream_t s = g->pick(stream);
    LaunchCounter lc;
    size_t bytes = (size_t)L.W * L.H * L.D * 16;
    if (dst_on_device) return launch_reg4_dense(g->g, nullptr, (float4*)vel4, s, lc);
    // stage through t4b's storage (large enough: elems*16 >= W*H*D*16)
    int rc = launch_reg4_dense(g->g, nullptr, g->g.t4b, s, lc);
    if (rc) return rc;
    ZQS_CUDA_TRY(cudaMemcpyAsync(vel4, g->g.t4b, bytes, cudaMemcpyDeviceToHost, s));
    return ZQS_OK;
}

ZQS_API int zqs_grid_stats(zqs_grid* g, zqs_stats* out, void* stream) {
    if (!g || !out) return set_error("NULL argument"), ZQS_EINVAL;
    int rc = g->ready();
    if (rc) return rc;
    cudaStream_t s = g->pick(stream);
    memset(out, 0, sizeof(*out));
    const float* p = g->p_last ? g->p_last : g->g.p;
    rc = launch_stats(g->g, g->kp, p, out, s);
    if (rc) return rc;
    if (g->params.solver == ZQS_SOLVER_CLOSED) {
        double m[2];
        ZQS_CUDA_TRY(cudaMemcpy(m, g->g.red + g->g.red_len - 2, sizeof(m), cudaMemcpyDeviceToHost));
        out->div_mean_removed = (double)(float)m[0];
    }
    return ZQS_OK;
}

ZQS_API int zqs_sor_variant_count(void) { return sor_variant_count(); }

ZQS_API int zqs_sor_variant_info(int index, zqs_sor_variant* out) { return sor_variant_info(index, out); }

ZQS_API int zqs_grid_set_sor_variant(zqs_grid* g, int index, int zchunk) {
    if (!g || index < -1 || index >= sor_variant_count() || zchunk < 0) {
        set_error("zqs_grid_set_sor_variant: bad arguments");
        return ZQS_EINVAL;
    }
    if (index >= 0) {
        zqs_sor_variant v;
        int rc = sor_variant_info(index, &v);
        if (rc) return rc;
        if (v.ctas_per_sm < 1) {
            set_error("zqs_grid_set_sor_variant: variant does not fit on this device");
            return ZQS_EUNSUPPORTED;
        }
    }
    g->sor.variant = index;
    g->sor.zchunk = zchunk;
    g->drop_graphs();
    return ZQS_OK;
}

ZQS_API int zqs_grid_synchronize(zqs_grid* g, void* stream) {
    if (!g) return set_error("NULL grid"), ZQS_EINVAL;
    ZQS_CUDA_TRY(cudaStreamSynchronize(g->pick(stream)));
    int rc = coarse_check(g->g.coarse, g->pick(stream));
    return rc ? rc : sor_sync_check();
}

ZQS_API int zqs_grid_set_coarse_gemm(zqs_grid* g, int mode) {
    if (!g || mode < 0 || mode > 1) {
        set_error("zqs_grid_set_coarse_gemm: mode must be 0 (FP32 SIMT) or 1 (tensor cores, 3xTF32)");
        return ZQS_EINVAL;
    }
    g->coarse_tc = mode;
    if (g->g.coarse) {
        ZQS_CUDA_TRY(cudaStreamSynchronize(g->own));
        int rc = coarse_prepare(g->g.coarse, g->g.L, g->g.coarse->s, mode);
        if (rc) return rc;
    }
    g->drop_graphs();
    return ZQS_OK;
}

ZQS_API int64_t zqs_grid_launch_count(const zqs_grid* g) { return g ? g->step_launches : 0; }

ZQS_API int zqs_debug_fail_alloc(int nth) {
    if (nth < -1) {
        set_error("zqs_debug_fail_alloc: nth must be >= -1");
        return ZQS_EINVAL;
    }
    g_alloc_fail_in.store(nth, std::memory_order_relaxed);
    return ZQS_OK;
}

}  // extern "C"
