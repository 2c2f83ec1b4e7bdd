// The reference's entry points (include/zqs_legacy.h) as shims over the
// library's kernels.  Host-pointer calls copy into a cached device grid of the
// requested size, run the stage, copy back and return the elapsed ms of the
// whole call, like the reference wrappers (e.g. ZQ_CUDA_AddForce3D.cu:606-659),
// but without per-call allocation and without exiting on errors.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/zqs_legacy.h"
#include "zqs_internal.h"

namespace zqs {
DevGrid& grid_dev(zqs_grid* g);
KParams& grid_kparams(zqs_grid* g);
cudaStream_t grid_stream(zqs_grid* g);
void grid_swap_velocity(zqs_grid* g);
void grid_swap_scalars(zqs_grid* g);
float*& grid_p_last(zqs_grid* g);
SorConfig& grid_sor(zqs_grid* g);
}  // namespace zqs

using namespace zqs;

namespace {

std::mutex g_mu;
zqs_grid* g_cache = nullptr;
int g_dims[3] = {0, 0, 0};

// Advection state set by ZQ_Cuda_Prepare_Advection (process-wide, as in the reference).
struct AdvState {
    unsigned W = 0, H = 0, D = 0, steps = 0;
    float h = 0.0f, dt_sub = 0.0f;
    bool set = false;
} g_adv;

int cached_grid(int W, int H, int D, zqs_grid** out) {
    if (g_cache && g_dims[0] == W && g_dims[1] == H && g_dims[2] == D) {
        *out = g_cache;
        return ZQS_OK;
    }
    if (g_cache) {
        zqs_grid_destroy(g_cache);
        g_cache = nullptr;
    }
    int rc = zqs_grid_create(&g_cache, W, H, D);
    if (rc) return rc;
    g_dims[0] = W;
    g_dims[1] = H;
    g_dims[2] = D;
    *out = g_cache;
    return ZQS_OK;
}

KParams base_kparams() {
    zqs_params p;
    zqs_params_default(&p, 2, 2, 2);
    KParams kp;
    make_kparams(p, kp);
    return kp;
}

void set_adv(KParams& kp) {
    kp.h = g_adv.h;
    kp.dt_sub = g_adv.dt_sub;  // deltatt as passed (ZQ_CUDA_Advection3D.cu:1652-1668)
    int e;
    float m = std::frexp(g_adv.h, &e);
    kp.inv_h = (g_adv.h > 0.0f && m == 0.5f) ? 1.0f / g_adv.h : 0.0f;
    kp.substeps = (int)g_adv.steps;
    kp.full = 0;
}

struct Timer {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaStream_t s;
    explicit Timer(cudaStream_t st) : s(st) {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, s);
    }
    float stop() {
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        return ms;
    }
    ~Timer() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

float fail(int rc) { return -(float)rc; }

#define LEG_TRY(expr)              \
    do {                           \
        int _rc = (expr);          \
        if (_rc) return fail(_rc); \
    } while (0)

int set_occ(zqs_grid* g, const bool* occ, int solver) {
    static_assert(sizeof(bool) == 1, "bool must be one byte");
    zqs_params p;
    if (zqs_grid_get_params(g, &p) != ZQS_OK || p.solver != solver) {
        zqs_params_default(&p, 2, 2, 2);
        p.solver = solver;
        int rc = zqs_grid_set_params(g, &p);
        if (rc) return rc;
    }
    return zqs_grid_upload(g, ZQS_FIELD_OCCUPANCY, occ, 0, nullptr);
}

}  // namespace

namespace ZQ_CUDA_Advection3D {

extern "C" ZQS_API void ZQ_Cuda_Prepare_Advection(const unsigned int width, const unsigned int height,
                                                  const unsigned int depth, const float voxelSize,
                                                  const unsigned int steps, const float deltatt) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_adv.W = width;
    g_adv.H = height;
    g_adv.D = depth;
    g_adv.h = voxelSize;
    g_adv.steps = steps;
    g_adv.dt_sub = deltatt;
    g_adv.set = true;
}

extern "C" ZQS_API float Advect_Velocity(float* u, float* v, float* w, const bool* occupy, bool is_open,
                                         enum AdvectVelocityType type) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_adv.set || !u || !v || !w || !occupy || g_adv.steps < 1) {
        set_error("Advect_Velocity: call ZQ_Cuda_Prepare_Advection first with steps >= 1; pointers must be non-NULL");
        return fail(ZQS_EINVAL);
    }
    if ((int)type < (int)ADV_VEL_INREG_OUTREG || (int)type > (int)ADV_VEL_INREG_OUTMAC_BFECC) {
        set_error("Advect_Velocity: unknown advection type; arrays left untouched");
        return fail(ZQS_EINVAL);
    }
    zqs_grid* g;
    LEG_TRY(cached_grid(g_adv.W, g_adv.H, g_adv.D, &g));
    cudaStream_t s = grid_stream(g);
    Timer t(s);
    LEG_TRY(set_occ(g, occupy, ZQS_SOLVER_OPEN));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_U, u, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_V, v, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_W, w, 0, nullptr));
    KParams kp = base_kparams();
    set_adv(kp);
    LaunchCounter lc;
    LEG_TRY(launch_advect_velocity(grid_dev(g), kp, (int)type, is_open, s, lc));
    grid_swap_velocity(g);
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_U, u, 0, nullptr));
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_V, v, 0, nullptr));
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_W, w, 0, nullptr));
    return t.stop();
}

extern "C" ZQS_API float Advect_Scalar(const float* u, const float* v, const float* w, const bool* occupy,
                                       const float* input_temperature, const float* input_density,
                                       float* output_temperature, float* output_density,
                                       enum AdvectScalarType type) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_adv.set || !u || !v || !w || !occupy || !input_temperature || !input_density || !output_temperature ||
        !output_density || g_adv.steps < 1) {
        set_error("Advect_Scalar: call ZQ_Cuda_Prepare_Advection first with steps >= 1; pointers must be non-NULL");
        return fail(ZQS_EINVAL);
    }
    if ((int)type < (int)ADV_SCA_MAC || (int)type > (int)ADV_SCA_REG_BFECC) {
        set_error("Advect_Scalar: unknown advection type; outputs left untouched");
        return fail(ZQS_EINVAL);
    }
    zqs_grid* g;
    LEG_TRY(cached_grid(g_adv.W, g_adv.H, g_adv.D, &g));
    cudaStream_t s = grid_stream(g);
    Timer t(s);
    LEG_TRY(set_occ(g, occupy, ZQS_SOLVER_OPEN));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_U, u, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_V, v, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_W, w, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_TEMPERATURE, input_temperature, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_DENSITY, input_density, 0, nullptr));
    KParams kp = base_kparams();
    set_adv(kp);
    LaunchCounter lc;
    LEG_TRY(launch_advect_scalar(grid_dev(g), kp, (int)type, false, nullptr, s, lc));
    grid_swap_scalars(g);
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_TEMPERATURE, output_temperature, 0, nullptr));
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_DENSITY, output_density, 0, nullptr));
    return t.stop();
}

}  // namespace ZQ_CUDA_Advection3D

namespace ZQ_CUDA_AddForce3D {

extern "C" ZQS_API float AddForce3D(float* mac_u, float* mac_v, float* mac_w, const bool* occupy,
                                    const float* temperature, const float deltah, const float deltat,
                                    const float buoyCoeff, const float confineCoeff, const float Tamb,
                                    const int width, const int height, const int depth, enum AddForceType type) {
    std::lock_guard<std::mutex> lk(g_mu);
    (void)type;
    if (!mac_u || !mac_v || !mac_w || !occupy || !temperature) {
        set_error("AddForce3D: NULL pointer");
        return fail(ZQS_EINVAL);
    }
    zqs_grid* g;
    LEG_TRY(cached_grid(width, height, depth, &g));
    cudaStream_t s = grid_stream(g);
    Timer t(s);
    LEG_TRY(set_occ(g, occupy, ZQS_SOLVER_OPEN));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_U, mac_u, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_V, mac_v, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_W, mac_w, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_TEMPERATURE, temperature, 0, nullptr));
    DevGrid& dg = grid_dev(g);
    // the reference passes no density; alpha = 0 makes the density term vanish
    if (cudaMemsetAsync(dg.rho - dg.L.plane, 0, (size_t)dg.L.elems * 4, s) != cudaSuccess) return fail(ZQS_ECUDA);
    KParams kp = base_kparams();
    kp.h = deltah;
    kp.dt = deltat;
    kp.beta = buoyCoeff;
    kp.cc = confineCoeff * deltah;
    kp.twoh = 2.0f * deltah;
    kp.tamb = Tamb;
    kp.alpha = 0.0f;
    LaunchCounter lc;
    LEG_TRY(launch_force(dg, kp, false, s, lc));
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_U, mac_u, 0, nullptr));
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_V, mac_v, 0, nullptr));
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_W, mac_w, 0, nullptr));
    return t.stop();
}

}  // namespace ZQ_CUDA_AddForce3D

namespace ZQ_CUDA_Attenuation3D {

extern "C" ZQS_API float Attenuation3D(float* mac_u, float* mac_v, float* mac_w, float* temperature,
                                       float* density, const bool* occupy, const float velAtten,
                                       const float tempAtten, const float densityAtten, const int width,
                                       const int height, const int depth) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!mac_u || !mac_v || !mac_w || !occupy || !temperature || !density) {
        set_error("Attenuation3D: NULL pointer");
        return fail(ZQS_EINVAL);
    }
    zqs_grid* g;
    LEG_TRY(cached_grid(width, height, depth, &g));
    cudaStream_t s = grid_stream(g);
    Timer t(s);
    LEG_TRY(set_occ(g, occupy, ZQS_SOLVER_OPEN));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_U, mac_u, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_V, mac_v, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_W, mac_w, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_TEMPERATURE, temperature, 0, nullptr));
    LEG_TRY(zqs_grid_upload(g, ZQS_FIELD_DENSITY, density, 0, nullptr));
    KParams kp = base_kparams();
    kp.vel_atten = velAtten;
    kp.temp_atten = tempAtten;
    kp.dens_atten = densityAtten;
    LaunchCounter lc;
    LEG_TRY(launch_attenuate(grid_dev(g), kp, s, lc));
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_U, mac_u, 0, nullptr));
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_V, mac_v, 0, nullptr));
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_W, mac_w, 0, nullptr));
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_TEMPERATURE, temperature, 0, nullptr));
    LEG_TRY(zqs_grid_download(g, ZQS_FIELD_DENSITY, density, 0, nullptr));
    return t.stop();
}

}  // namespace ZQ_CUDA_Attenuation3D

namespace ZQ_CUDA_MACtoRegular {

ZQS_API void cu_MAC_to_Regular4(const float* mac_u, const float* mac_v, const float* mac_w, float4* vel4, int width,
                                int height, int depth) {
    launch_dense_mac_to_centre(width, height, depth, mac_u, mac_v, mac_w, vel4, nullptr, nullptr, nullptr, 0);
}

ZQS_API void cu_Regular4_to_MAC(const float4* vel4, float* mac_u, float* mac_v, float* mac_w, int width, int height,
                                int depth) {
    launch_dense_reg4_to_mac(width, height, depth, vel4, mac_u, mac_v, mac_w, 0);
}

}  // namespace ZQ_CUDA_MACtoRegular

namespace {

int project_host(float* u, float* v, float* w, const uint8_t* occ, int W, int H, int D, int solver, int maxIter,
                 float omega, bool given_mean, float mean) {
    if (!u || !v || !w || !occ || maxIter < 0) {
        set_error("project: NULL pointer or negative iteration count");
        return ZQS_EINVAL;
    }
    zqs_grid* g;
    int rc = cached_grid(W, H, D, &g);
    if (rc) return rc;
    rc = set_occ(g, (const bool*)occ, solver);
    if (rc) return rc;
    cudaStream_t s = grid_stream(g);
    if ((rc = zqs_grid_upload(g, ZQS_FIELD_U, u, 0, nullptr))) return rc;
    if ((rc = zqs_grid_upload(g, ZQS_FIELD_V, v, 0, nullptr))) return rc;
    if ((rc = zqs_grid_upload(g, ZQS_FIELD_W, w, 0, nullptr))) return rc;
    KParams kp = base_kparams();
    kp.solver = solver;
    kp.omega = omega;
    kp.om1 = 1.0f - omega;
    kp.mean_override = given_mean ? 1 : 0;
    kp.mean_value = mean;
    LaunchCounter lc;
    rc = launch_project(grid_dev(g), kp, maxIter, grid_sor(g), s, lc, &grid_p_last(g));
    if (rc) return rc;
    if ((rc = zqs_grid_download(g, ZQS_FIELD_U, u, 0, nullptr))) return rc;
    if ((rc = zqs_grid_download(g, ZQS_FIELD_V, v, 0, nullptr))) return rc;
    if ((rc = zqs_grid_download(g, ZQS_FIELD_W, w, 0, nullptr))) return rc;
    ZQS_CUDA_TRY(cudaStreamSynchronize(s));
    return ZQS_OK;
}

}  // namespace

namespace ZQ_CUDA_PoissonSolver3D {

ZQS_API void SolveOpenPoissonRedBlackwithOccupy3D_MAC(float* mac_u, float* mac_v, float* mac_w, const bool* occupy,
                                                      int width, int height, int depth, int maxIter) {
    std::lock_guard<std::mutex> lk(g_mu);
    project_host(mac_u, mac_v, mac_w, (const uint8_t*)occupy, width, height, depth, ZQS_SOLVER_OPEN, maxIter, 1.0f,
                 false, 0.0f);
}

ZQS_API void SolveClosedPoissonRedBlackwithOccupy3D_MAC(float* mac_u, float* mac_v, float* mac_w, const bool* occupy,
                                                        float div_per_volume, int width, int height, int depth,
                                                        int maxIter) {
    std::lock_guard<std::mutex> lk(g_mu);
    project_host(mac_u, mac_v, mac_w, (const uint8_t*)occupy, width, height, depth, ZQS_SOLVER_CLOSED, maxIter, 1.0f,
                 true, div_per_volume);
}

ZQS_API void cu_MAC_to_Regular_vel(float* u, float* v, float* w, const float* mac_u, const float* mac_v,
                                   const float* mac_w, int width, int height, int depth) {
    launch_dense_mac_to_centre(width, height, depth, mac_u, mac_v, mac_w, nullptr, u, v, w, 0);
}

}  // namespace ZQ_CUDA_PoissonSolver3D

extern "C" ZQS_API int zqs_project_sor(float* mac_u, float* mac_v, float* mac_w, const uint8_t* occupy, int width,
                                       int height, int depth, int solver, int maxIter, float omega) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (solver != ZQS_SOLVER_OPEN && solver != ZQS_SOLVER_CLOSED) {
        set_error("zqs_project_sor: bad solver");
        return ZQS_EINVAL;
    }
    return project_host(mac_u, mac_v, mac_w, occupy, width, height, depth, solver, maxIter, omega, false, 0.0f);
}
