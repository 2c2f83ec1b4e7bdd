// Moving voxel objects (ZQ_ApplyMovingObject3D, ZQ_SmokeSimulationUtils3D.cpp:
// 1933-2046) on the device: the occupancy is rebuilt from the objects (and the
// domain walls of the closed solvers), the faces of every object voxel take the
// object's velocity, then the cell flags are rebuilt.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "zqs_capi.h"
#include "zqs_grid.h"

namespace zqs {

namespace {

// occupancy = 0, or the six domain walls when closed == 1 (Utils3D:1994-2044),
// or all but the y = H-1 layer when closed == 2
__global__ void k_occ_walls(int W, int H, int D, uint8_t* __restrict__ occ, int closed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= W || j >= H || k >= D) return;
    const bool wall =
        closed && (i == 0 || i == W - 1 || j == 0 || (j == H - 1 && closed == 1) || k == 0 || k == D - 1);
    occ[((size_t)k * H + j) * W + i] = wall ? 1 : 0;
}

// One thread per object voxel (Utils3D:1966-1990): an in-domain solid voxel
// is occupied and its six faces take the object's velocity.
__global__ void k_stamp_object(Layout L, uint8_t* __restrict__ occ, float* __restrict__ u, float* __restrict__ v,
                               float* __restrict__ w, const uint8_t* __restrict__ mask, int sx, int sy, int sz,
                               int ox, int oy, int oz, float cu, float cv, float cw) {
    const int si = blockIdx.x * blockDim.x + threadIdx.x;
    const int sj = blockIdx.y * blockDim.y + threadIdx.y;
    const int sk = blockIdx.z;
    if (si >= sx || sj >= sy || sk >= sz) return;
    if (!mask[((size_t)sk * sy + sj) * sx + si]) return;
    const int ix = si + ox, iy = sj + oy, iz = sk + oz;
    if (ix < 0 || ix >= L.W || iy < 0 || iy >= L.H || iz < 0 || iz >= L.D) return;
    occ[((size_t)iz * L.H + iy) * L.W + ix] = 1;
    const int c = lidx(L, ix, iy, iz);
    u[c] = cu;
    u[c + 1] = cu;
    v[c] = cv;
    v[c + L.px] = cv;
    w[c] = cw;
    w[c + (int)L.plane] = cw;
}

}  // namespace

}  // namespace zqs

using namespace zqs;

extern "C" ZQS_API int zqs_grid_stamp_objects(zqs_grid* g, const zqs_object* objs, int n, int closed_walls,
                                              void* stream) {
    if (!g || n < 0 || (n > 0 && !objs) || closed_walls < 0 || closed_walls > 2) {
        set_error("zqs_grid_stamp_objects: bad arguments");
        return ZQS_EINVAL;
    }
    if (!g->has_params) {
        set_error("zqs_grid_stamp_objects: set the parameters first (h / dt scales the velocities)");
        return ZQS_ENOTREADY;
    }
    // every mask in one host buffer, copied once: the stamping kernels then
    // read their object's slice (no synchronisation between objects)
    std::vector<size_t> off(n + 1, 0);
    for (int q = 0; q < n; q++) {
        const zqs_object& o = objs[q];
        const size_t nb = (o.size[0] < 0 || o.size[1] < 0 || o.size[2] < 0)
                              ? 0
                              : (size_t)o.size[0] * (size_t)o.size[1] * (size_t)o.size[2];
        // z is a launch dimension (at most 65535 planes)
        if (o.size[0] < 0 || o.size[1] < 0 || o.size[2] < 0 || o.size[2] > 65535 || (!o.mask && nb > 0)) {
            set_error("zqs_grid_stamp_objects: object " + std::to_string(q) + " has a bad size or no mask");
            return ZQS_EINVAL;
        }
        off[q + 1] = off[q] + nb;
    }
    const size_t need = off[n];
    cudaStream_t s = g->pick(stream);
    // the previous call's copy and kernels may still read the buffer
    ZQS_CUDA_TRY(cudaStreamSynchronize(s));
    if (need > g->obj_mask_cap) {
        if (g->obj_mask) cudaFree(g->obj_mask);
        g->obj_mask = nullptr;
        g->obj_mask_cap = 0;
        ZQS_CUDA_TRY(dev_alloc(&g->obj_mask, need));
        g->obj_mask_cap = need;
    }
    if (need > 0) {
        std::vector<uint8_t> all(need);
        for (int q = 0; q < n; q++)
            if (off[q + 1] > off[q]) std::memcpy(all.data() + off[q], objs[q].mask, off[q + 1] - off[q]);
        // pageable source: the copy has completed when the call returns
        ZQS_CUDA_TRY(cudaMemcpyAsync(g->obj_mask, all.data(), need, cudaMemcpyHostToDevice, s));
    }
    const Layout& L = g->g.L;
    const dim3 b(32, 8, 1);
    k_occ_walls<<<dim3((L.W + 31) / 32, (L.H + 7) / 8, L.D), b, 0, s>>>(L.W, L.H, L.D, g->occ_dense,
                                                                        closed_walls);
    ZQS_LAUNCH_CHECK("k_occ_walls");
    // deltah / deltat in float, widened to double; int velocity * scale truncated (Utils3D:1958-1962)
    const double scale = (double)(g->params.voxel_size / g->params.step_time);
    for (int q = 0; q < n; q++) {
        const zqs_object& o = objs[q];
        const size_t nb = off[q + 1] - off[q];
        if (nb == 0) continue;
        const int cu = (int)((double)o.vel[0] * scale);
        const int cv = (int)((double)o.vel[1] * scale);
        const int cw = (int)((double)o.vel[2] * scale);
        k_stamp_object<<<dim3((o.size[0] + 31) / 32, (o.size[1] + 7) / 8, o.size[2]), b, 0, s>>>(
            L, g->occ_dense, g->g.u, g->g.v, g->g.w, g->obj_mask + off[q], o.size[0], o.size[1], o.size[2],
            o.pos[0] - o.center[0], o.pos[1] - o.center[1], o.pos[2] - o.center[2], (float)cu, (float)cv, (float)cw);
        ZQS_LAUNCH_CHECK("k_stamp_object");
    }
    LaunchCounter lc;
    int rc = launch_build_flags(g->g, g->occ_dense, g->params.solver, s, lc);
    if (rc) return rc;
    g->has_occ = true;
    return ZQS_OK;
}
