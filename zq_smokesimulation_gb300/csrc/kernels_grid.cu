// Grid set-up kernels: flag construction and MAC -> cell-centre velocity.
#include "zqs_internal.h"

namespace zqs {

namespace {

// One thread per padded index (i,j,k), i < pitch, j < rows, k < planes.
// occ is the reference-layout occupancy (W*H*D bytes, nonzero = occupied).
// Face rules: ZQ_CUDA_Advection3D.cu:471-575 (open write-back), which the
// force (ZQ_CUDA_AddForce3D.cu:211-385) and attenuation
// (ZQ_CUDA_Attenuation3D.cu:8-98) kernels share.  Stencil weight: free
// in-domain neighbours count 1, outside the domain counts 1 for the open
// solver (ZQ_SmokeSimulationUtils3D.cpp:570, count = 6 - #in-domain) and 0 for
// the closed one.
// The SOR sweeps sum all six neighbours and the divergence writes only free
// cells, so pressure and right-hand side must hold 0 in every occupied cell;
// occupancy that changes (moving objects, a new upload) clears them there.
__global__ void k_build_flags(Layout L, const uint8_t* __restrict__ occ, uint8_t* __restrict__ flags, int open,
                              float* __restrict__ p, float* __restrict__ p2, float* __restrict__ div) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i >= L.px || j >= L.py || k >= L.pz) return;
    const int W = L.W, H = L.H, D = L.D;
    auto occupied = [&](int a, int b, int c) -> bool { return occ[((size_t)c * H + b) * W + a] != 0; };
    uint8_t f = 0;
    if (i < W && j < H && k < D && occupied(i, j, k)) {
        const int c = lidx(L, i, j, k);
        p[c] = 0.0f;
        p2[c] = 0.0f;
        div[c] = 0.0f;
    }
    if (i < W && j < H && k < D && !occupied(i, j, k)) {
        f |= F_FREE;
        int nin = 0, nfree = 0;
        const int di[6] = {-1, 1, 0, 0, 0, 0}, dj[6] = {0, 0, -1, 1, 0, 0}, dk[6] = {0, 0, 0, 0, -1, 1};
        for (int q = 0; q < 6; q++) {
            int a = i + di[q], b = j + dj[q], c = k + dk[q];
            if (a < 0 || a >= W || b < 0 || b >= H || c < 0 || c >= D) continue;
            nin++;
            if (!occupied(a, b, c)) nfree++;
        }
        int cnt = open ? 6 - (nin - nfree) : nfree;
        f |= (uint8_t)(cnt << F_CNT_SHIFT);
    }
    if (i <= W && j < H && k < D) {
        bool live;
        if (i == 0) live = !occupied(0, j, k);
        else if (i == W) live = !occupied(W - 1, j, k);
        else live = !occupied(i, j, k) && !occupied(i - 1, j, k);
        if (live) f |= F_UFACE;
    }
    if (i < W && j <= H && k < D) {
        bool live;
        if (j == 0) live = !occupied(i, 0, k);
        else if (j == H) live = !occupied(i, H - 1, k);
        else live = !occupied(i, j, k) && !occupied(i, j - 1, k);
        if (live) f |= F_VFACE;
    }
    if (i < W && j < H && k <= D) {
        bool live;
        if (k == 0) live = !occupied(i, j, 0);
        else if (k == D) live = !occupied(i, j, D - 1);
        else live = !occupied(i, j, k) && !occupied(i, j, k - 1);
        if (live) f |= F_WFACE;
    }
    flags[lidx(L, i, j, k)] = f;
}

// MAC_to_Regular4_Kernel semantics (ZQ_CUDA_MACtoRegular.cu:9-27):
// centre = 0.5f*(lo + hi), fourth channel 0.  DENSE writes the reference's
// W*H*D float4 layout, otherwise the padded index space.
template <bool DENSE>
__global__ void k_mac_to_reg4(Layout L, const float* __restrict__ u, const float* __restrict__ v,
                              const float* __restrict__ w, float4* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    int c = lidx(L, i, j, k);
    float4 r;
    r.x = 0.5f * (__ldg(u + c) + __ldg(u + c + 1));
    r.y = 0.5f * (__ldg(v + c) + __ldg(v + c + L.px));
    r.z = 0.5f * (__ldg(w + c) + __ldg(w + c + (int)L.plane));
    r.w = 0.0f;
    if (DENSE) out[((size_t)k * L.H + j) * L.W + i] = r;
    else out[c] = r;
}

// Dense (unpadded reference layout) forms for the device-pointer entry points
// cu_MAC_to_Regular4 / cu_Regular4_to_MAC (ZQ_CUDA_MACtoRegular.cu:9-99) and
// cu_MAC_to_Regular_vel.  One thread per (i,j,k) of the (W+1)(H+1)(D+1) box.
__global__ void k_dense_mac_to_centre(int W, int H, int D, const float* __restrict__ u, const float* __restrict__ v,
                                      const float* __restrict__ w, float4* __restrict__ vel4, float* __restrict__ uc,
                                      float* __restrict__ vc, float* __restrict__ wc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i >= W || j >= H || k >= D) return;
    size_t c = ((size_t)k * H + j) * W + i;
    size_t cu = ((size_t)k * H + j) * (W + 1) + i;
    size_t cv = ((size_t)k * (H + 1) + j) * W + i;
    float a = 0.5f * (u[cu] + u[cu + 1]);
    float b = 0.5f * (v[cv] + v[cv + W]);
    float d = 0.5f * (w[c] + w[c + (size_t)W * H]);
    if (vel4) vel4[c] = make_float4(a, b, d, 0.0f);
    if (uc) {
        uc[c] = a;
        vc[c] = b;
        wc[c] = d;
    }
}

__global__ void k_dense_reg4_to_mac(int W, int H, int D, const float4* __restrict__ c4, float* __restrict__ u,
                                    float* __restrict__ v, float* __restrict__ w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i > W || j > H || k > D) return;
    auto C = [&](int a, int b, int e) -> float4 { return c4[((size_t)e * H + b) * W + a]; };
    if (j < H && k < D) {
        float o;
        if (i == 0) o = C(0, j, k).x;
        else if (i == W) o = C(W - 1, j, k).x;
        else o = 0.5f * (C(i, j, k).x + C(i - 1, j, k).x);
        u[((size_t)k * H + j) * (W + 1) + i] = o;
    }
    if (i < W && k < D) {
        float o;
        if (j == 0) o = C(i, 0, k).y;
        else if (j == H) o = C(i, H - 1, k).y;
        else o = 0.5f * (C(i, j, k).y + C(i, j - 1, k).y);
        v[((size_t)k * (H + 1) + j) * W + i] = o;
    }
    if (i < W && j < H) {
        float o;
        if (k == 0) o = C(i, j, 0).z;
        else if (k == D) o = C(i, j, D - 1).z;
        else o = 0.5f * (C(i, j, k).z + C(i, j, k - 1).z);
        w[((size_t)k * H + j) * W + i] = o;
    }
}

}  // namespace

int launch_dense_mac_to_centre(int W, int H, int D, const float* u, const float* v, const float* w, float4* vel4,
                               float* uc, float* vc, float* wc, cudaStream_t s) {
    dim3 b(32, 8, 1), gr((W + 31) / 32, (H + 7) / 8, D);
    k_dense_mac_to_centre<<<gr, b, 0, s>>>(W, H, D, u, v, w, vel4, uc, vc, wc);
    ZQS_LAUNCH_CHECK("k_dense_mac_to_centre");
    return ZQS_OK;
}

int launch_dense_reg4_to_mac(int W, int H, int D, const float4* vel4, float* u, float* v, float* w, cudaStream_t s) {
    dim3 b(32, 8, 1), gr((W + 1 + 31) / 32, (H + 1 + 7) / 8, D + 1);
    k_dense_reg4_to_mac<<<gr, b, 0, s>>>(W, H, D, vel4, u, v, w);
    ZQS_LAUNCH_CHECK("k_dense_reg4_to_mac");
    return ZQS_OK;
}

int launch_build_flags(const DevGrid& g, const uint8_t* occ_dense, int solver, cudaStream_t s, LaunchCounter& lc) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1), gr((L.px + 31) / 32, (L.py + 7) / 8, L.pz);
    k_build_flags<<<gr, b, 0, s>>>(L, occ_dense, g.flags, solver != ZQS_SOLVER_CLOSED ? 1 : 0, g.p, g.p2, g.div);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_build_flags");
    return ZQS_OK;
}

int launch_mac_to_reg4(const DevGrid& g, const float* u, const float* v, const float* w, float4* out,
                       cudaStream_t s, LaunchCounter& lc) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1), gr((L.W + 31) / 32, (L.H + 7) / 8, L.D);
    k_mac_to_reg4<false><<<gr, b, 0, s>>>(L, u, v, w, out);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_mac_to_reg4");
    return ZQS_OK;
}

int launch_reg4_dense(const DevGrid& g, const float4* /*unused*/, float4* dense, cudaStream_t s, LaunchCounter& lc) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1), gr((L.W + 31) / 32, (L.H + 7) / 8, L.D);
    k_mac_to_reg4<true><<<gr, b, 0, s>>>(L, g.u, g.v, g.w, dense);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_mac_to_reg4<dense>");
    return ZQS_OK;
}

}  // namespace zqs
