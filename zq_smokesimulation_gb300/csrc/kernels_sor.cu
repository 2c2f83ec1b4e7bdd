// Pressure projection: divergence, fixed-K red-black SOR, gradient subtraction.
//
// Restates ZQ_CUDA_PoissonSolver3D::Solve{Open,Closed}PoissonRedBlackwithOccupy3D_MAC,
// whose source is not part of the reference tree (call sites
// ZQ_SmokeSimulationUtils3D.cpp:2354-2363, 2424-2437).  The rule is the one the
// oracle states (oracle/zqs_oracle.cpp, project()):
//   div  = ((((u[i+1]-u[i]) + v[j+1]) - v[j]) + w[k+1]) - w[k]   (closed: minus the FP64 mean)
//   red cells ((i+j+k)&1)==0 then black, each free cell:
//     s  = p[x-] + p[x+] + p[y-] + p[y+] + p[z-] + p[z+]   (left to right)
//     p  = (1-omega)*p + omega*((s - div)/cnt)
//   u -= p_R - p_L on live faces (open domain faces use p = 0 outside).
// Non-free cells and everything outside the domain hold p = +0 permanently,
// so summing all six neighbours equals summing the free ones bit for bit (a
// running sum that starts at +0 is never -0, and x + (+0) == x otherwise).
//
// Two SOR kernels:
//   k_sor_colour   one launch per colour, in place (the plain form, also the
//                  colour-race self-check of the fused kernel);
//   k_sor_tb<S>    S half-sweeps per HBM pass (S/2 iterations): a CTA owns an
//                  xy tile plus an S-cell halo and streams a z chunk through a
//                  ring of S+2 shared-memory planes; half-sweep s runs on plane
//                  t-s at time t over the tile grown by S-s cells, so every
//                  value it reads is at the correct sweep.  Results are
//                  identical to S/2 iterations of k_sor_colour.
#include "zqs_internal.h"

#include <algorithm>
#include <vector>

namespace zqs {

namespace {

__global__ void k_divergence(Layout L, const float* __restrict__ u, const float* __restrict__ v,
                             const float* __restrict__ w, const uint8_t* __restrict__ flags, float* __restrict__ div,
                             float* __restrict__ p, double* __restrict__ part, int want_partials) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    double sum = 0.0, cnt = 0.0;
    if (i < L.W && j < L.H && k < L.D) {
        const int c = lidx(L, i, j, k);
        if (__ldg(flags + c) & F_FREE) {
            float d = ((((__ldg(u + c + 1) - __ldg(u + c)) + __ldg(v + c + L.px)) - __ldg(v + c)) +
                       __ldg(w + c + (int)L.plane)) -
                      __ldg(w + c);
            div[c] = d;
            p[c] = 0.0f;
            sum = (double)d;
            cnt = 1.0;
        }
    }
    if (want_partials) {
        // fixed-shape block reduction (deterministic)
        __shared__ double ss[256], sc[256];
        const int t = threadIdx.y * blockDim.x + threadIdx.x;
        ss[t] = sum;
        sc[t] = cnt;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (t < o) {
                ss[t] += ss[t + o];
                sc[t] += sc[t + o];
            }
            __syncthreads();
        }
        if (t == 0) {
            long long b = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
            part[2 * b] = ss[0];
            part[2 * b + 1] = sc[0];
        }
    }
}

// Single block: sums the partials in a fixed order, stores mean (as double) in out[0].
__global__ void k_reduce_mean(const double* __restrict__ part, long long nblocks, double* __restrict__ out) {
    __shared__ double ss[256], sc[256];
    double s = 0.0, c = 0.0;
    for (long long b = threadIdx.x; b < nblocks; b += 256) {
        s += part[2 * b];
        c += part[2 * b + 1];
    }
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = c;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            ss[threadIdx.x] += ss[threadIdx.x + o];
            sc[threadIdx.x] += sc[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sc[0] > 0.0 ? ss[0] / sc[0] : 0.0;
        out[1] = sc[0];
    }
}

__global__ void k_div_subtract_mean(Layout L, const uint8_t* __restrict__ flags, float* __restrict__ div,
                                    const double* __restrict__ mean) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    if (__ldg(flags + c) & F_FREE) {
        const float m = (float)mean[0];
        div[c] = div[c] - m;
    }
}

__global__ void k_div_subtract_const(Layout L, const uint8_t* __restrict__ flags, float* __restrict__ div, float m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    const int c = lidx(L, i, j, k);
    if (__ldg(flags + c) & F_FREE) div[c] = div[c] - m;
}

__device__ __forceinline__ float sor_update(float pc, float s, float d, int cnt, float omega, float om1) {
    float gs = (s - d) / (float)cnt;
    return om1 * pc + omega * gs;
}

// One colour, in place; one thread per cell.
__global__ void k_sor_colour(Layout L, float* __restrict__ p, const float* __restrict__ div,
                             const uint8_t* __restrict__ flags, int colour, float omega, float om1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= L.W || j >= L.H || k >= L.D) return;
    if (((i + j + k) & 1) != colour) return;
    const int c = lidx(L, i, j, k);
    const uint8_t f = __ldg(flags + c);
    const int cnt = (f & F_CNT_MASK) >> F_CNT_SHIFT;
    if (!(f & F_FREE) || cnt == 0) return;
    const int px = L.px, pl = (int)L.plane;
    float s = 0.0f;
    s = s + p[c - 1];
    s = s + p[c + 1];
    s = s + p[c - px];
    s = s + p[c + px];
    s = s + p[c - pl];
    s = s + p[c + pl];
    p[c] = sor_update(p[c], s, __ldg(div + c), cnt, omega, om1);
}

template <int S, int TX, int TY>
struct TbShape {
    static constexpr int RW = TX + 2 * S;
    static constexpr int RH = TY + 2 * S;
    static constexpr int PL = RW * RH;
    static constexpr int NP = S + 2;
    static constexpr size_t smem = (size_t)NP * PL * (sizeof(float) * 2 + 1);
};

__device__ __forceinline__ int ring(int z, int np) {
    int r = z % np;
    return r < 0 ? r + np : r;
}

// Temporally blocked red-black SOR: S half-sweeps (S even, red first) per pass,
// reading pin and writing pout.  Grid: (ceil(W/TX), ceil(H/TY), ceil(D/zc)).
template <int S, int TX, int TY>
__global__ void __launch_bounds__(256) k_sor_tb(Layout L, const float* __restrict__ pin, float* __restrict__ pout,
                                                const float* __restrict__ div, const uint8_t* __restrict__ flags,
                                                float omega, float om1, int zc) {
    using Sh = TbShape<S, TX, TY>;
    constexpr int RW = Sh::RW, RH = Sh::RH, PL = Sh::PL, NP = Sh::NP;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sp = reinterpret_cast<float*>(smem_raw);
    float* sd = sp + NP * PL;
    uint8_t* sf = reinterpret_cast<uint8_t*>(sd + NP * PL);
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, L.D);
    const int tid = threadIdx.x;
    const int nthr = blockDim.x;

    for (int t = z0 - S; t < z1 + S; t++) {
        {
            const int slot = ring(t, NP);
            float* P = sp + slot * PL;
            float* Dv = sd + slot * PL;
            uint8_t* F = sf + slot * PL;
            const bool zin = (t >= 0 && t < L.D);
            for (int idx = tid; idx < PL; idx += nthr) {
                const int lj = idx / RW, li = idx - lj * RW;
                const int i = x0 - S + li, j = y0 - S + lj;
                float pv = 0.0f, dv = 0.0f;
                uint8_t fv = 0;
                if (zin && i >= 0 && i < L.W && j >= 0 && j < L.H) {
                    const int c = lidx(L, i, j, t);
                    fv = __ldg(flags + c);
                    if (fv & F_FREE) {
                        pv = pin[c];
                        dv = __ldg(div + c);
                    }
                }
                P[idx] = pv;
                Dv[idx] = dv;
                F[idx] = fv;
            }
        }
        __syncthreads();
#pragma unroll
        for (int s = 1; s <= S; s++) {
            const int z = t - s;
            const int r = S - s;
            if (z >= max(z0 - r, 0) && z < min(z1 + r, L.D)) {
                const int colour = (s - 1) & 1;
                float* Pc = sp + ring(z, NP) * PL;
                const float* Pm = sp + ring(z - 1, NP) * PL;
                const float* Pp = sp + ring(z + 1, NP) * PL;
                const float* Dc = sd + ring(z, NP) * PL;
                const uint8_t* Fc = sf + ring(z, NP) * PL;
                const int rw = TX + 2 * r;
                const int halfw = rw >> 1;
                const int nupd = halfw * (TY + 2 * r);
                for (int q = tid; q < nupd; q += nthr) {
                    const int row = q / halfw;
                    const int m = q - row * halfw;
                    const int ly = row - r;
                    const int j = y0 + ly;
                    const int base = x0 - r + 2 * m;
                    const int i = base + ((base + j + z + colour) & 1);
                    const int si = (ly + S) * RW + (i - x0 + S);
                    const uint8_t f = Fc[si];
                    const int cnt = (f & F_CNT_MASK) >> F_CNT_SHIFT;
                    if (!(f & F_FREE) || cnt == 0) continue;
                    float sum = 0.0f;
                    sum = sum + Pc[si - 1];
                    sum = sum + Pc[si + 1];
                    sum = sum + Pc[si - RW];
                    sum = sum + Pc[si + RW];
                    sum = sum + Pm[si];
                    sum = sum + Pp[si];
                    Pc[si] = sor_update(Pc[si], sum, Dc[si], cnt, omega, om1);
                }
            }
            __syncthreads();
        }
        const int zo = t - S;
        if (zo >= z0 && zo < z1) {
            const float* P = sp + ring(zo, NP) * PL;
            const uint8_t* F = sf + ring(zo, NP) * PL;
            for (int idx = tid; idx < TX * TY; idx += nthr) {
                const int ly = idx / TX, lx = idx - ly * TX;
                const int i = x0 + lx, j = y0 + ly;
                if (i < L.W && j < L.H) {
                    const int si = (ly + S) * RW + (lx + S);
                    if (F[si] & F_FREE) pout[lidx(L, i, j, zo)] = P[si];
                }
            }
        }
        // The next load writes the slot of plane t+1-NP = t-S-1, whose last
        // reader (half-sweep S at this step) finished before the barrier above.
    }
}

// u -= p_R - p_L on live faces; OPEN also updates domain faces with p = 0 outside.
__global__ void k_gradient(Layout L, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w,
                           const float* __restrict__ p, const uint8_t* __restrict__ flags, int open) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > L.W || j > L.H || k > L.D) return;
    const int c = lidx(L, i, j, k);
    const int px = L.px, pl = (int)L.plane;
    const uint8_t fl = __ldg(flags + c);
    const float zero = 0.0f;
    if ((fl & F_UFACE) && (open || (i > 0 && i < L.W))) {
        float f = u[c];
        if (i == 0) f = f - (__ldg(p + c) - zero);
        else if (i == L.W) f = f - (zero - __ldg(p + c - 1));
        else f = f - (__ldg(p + c) - __ldg(p + c - 1));
        u[c] = f;
    }
    if ((fl & F_VFACE) && (open || (j > 0 && j < L.H))) {
        float f = v[c];
        if (j == 0) f = f - (__ldg(p + c) - zero);
        else if (j == L.H) f = f - (zero - __ldg(p + c - px));
        else f = f - (__ldg(p + c) - __ldg(p + c - px));
        v[c] = f;
    }
    if ((fl & F_WFACE) && (open || (k > 0 && k < L.D))) {
        float f = w[c];
        if (k == 0) f = f - (__ldg(p + c) - zero);
        else if (k == L.D) f = f - (zero - __ldg(p + c - pl));
        else f = f - (__ldg(p + c) - __ldg(p + c - pl));
        w[c] = f;
    }
}

// FP64 diagnostics per block: max|div u| and sum of squared residuals.
__global__ void k_stats(Layout L, const float* __restrict__ u, const float* __restrict__ v,
                        const float* __restrict__ w, const float* __restrict__ p, const float* __restrict__ div,
                        const uint8_t* __restrict__ flags, double* __restrict__ part) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    double mx = 0.0, r2 = 0.0, nf = 0.0;
    if (i < L.W && j < L.H && k < L.D) {
        const int c = lidx(L, i, j, k);
        const uint8_t f = flags[c];
        if (f & F_FREE) {
            const int px = L.px, pl = (int)L.plane;
            float d = ((((u[c + 1] - u[c]) + v[c + px]) - v[c]) + w[c + pl]) - w[c];
            mx = fabs((double)d);
            double s = 0.0;
            s += (double)p[c - 1];
            s += (double)p[c + 1];
            s += (double)p[c - px];
            s += (double)p[c + px];
            s += (double)p[c - pl];
            s += (double)p[c + pl];
            const int cnt = (f & F_CNT_MASK) >> F_CNT_SHIFT;
            double r = (double)div[c] - (s - (double)cnt * (double)p[c]);
            r2 = r * r;
            nf = 1.0;
        }
    }
    __shared__ double smx[256], sr2[256], snf[256];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    smx[t] = mx;
    sr2[t] = r2;
    snf[t] = nf;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o) {
            smx[t] = fmax(smx[t], smx[t + o]);
            sr2[t] += sr2[t + o];
            snf[t] += snf[t + o];
        }
        __syncthreads();
    }
    if (t == 0) {
        long long b = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
        part[3 * b] = smx[0];
        part[3 * b + 1] = sr2[0];
        part[3 * b + 2] = snf[0];
    }
}

template <int S, int TX, int TY>
int prepare_tb() {
    using Sh = TbShape<S, TX, TY>;
    cudaError_t e = cudaFuncSetAttribute(k_sor_tb<S, TX, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)Sh::smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_sor_tb)");
    return ZQS_OK;
}

template <int S, int TX, int TY>
int launch_tb(const DevGrid& g, const float* pin, float* pout, const KParams& kp, int zc, cudaStream_t st) {
    using Sh = TbShape<S, TX, TY>;
    const Layout& L = g.L;
    dim3 gr((L.W + TX - 1) / TX, (L.H + TY - 1) / TY, (L.D + zc - 1) / zc);
    k_sor_tb<S, TX, TY><<<gr, 256, Sh::smem, st>>>(L, pin, pout, g.div, g.flags, kp.omega, kp.om1, zc);
    return ZQS_OK;
}

int launch_tb_depth(int S, const DevGrid& g, const float* pin, float* pout, const KParams& kp, int zc,
                    cudaStream_t st) {
    switch (S) {
        case 2: return launch_tb<2, 32, 16>(g, pin, pout, kp, zc, st);
        case 4: return launch_tb<4, 32, 16>(g, pin, pout, kp, zc, st);
        case 6: return launch_tb<6, 32, 16>(g, pin, pout, kp, zc, st);
        case 8: return launch_tb<8, 32, 16>(g, pin, pout, kp, zc, st);
        default: set_error("SOR temporal depth must be 1..4 iterations"); return ZQS_EINVAL;
    }
}

}  // namespace

int sor_prepare() {
    static int done = 0;  // per process; one device
    if (done) return ZQS_OK;
    int rc = prepare_tb<2, 32, 16>();
    if (!rc) rc = prepare_tb<4, 32, 16>();
    if (!rc) rc = prepare_tb<6, 32, 16>();
    if (!rc) rc = prepare_tb<8, 32, 16>();
    if (!rc) done = 1;
    return rc;
}

int launch_project(DevGrid& g, const KParams& kp, int K, const SorConfig& cfg, cudaStream_t s, LaunchCounter& lc,
                   float** p_final) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    dim3 gc((L.W + 31) / 32, (L.H + 7) / 8, L.D);
    const bool closed = kp.solver == ZQS_SOLVER_CLOSED;
    k_divergence<<<gc, b, 0, s>>>(L, g.u, g.v, g.w, g.flags, g.div, g.p, g.red, closed ? 1 : 0);
    lc.n++;
    if (closed) {
        long long nblocks = (long long)gc.x * gc.y * gc.z;
        double* mean = g.red + g.red_len - 2;  // kept apart from the stats partials
        if (kp.mean_override) {
            k_div_subtract_const<<<gc, b, 0, s>>>(L, g.flags, g.div, kp.mean_value);
            lc.n++;
        } else {
            k_reduce_mean<<<1, 256, 0, s>>>(g.red, nblocks, mean);
            k_div_subtract_mean<<<gc, b, 0, s>>>(L, g.flags, g.div, mean);
            lc.n += 2;
        }
    }
    ZQS_LAUNCH_CHECK("divergence");
    float* cur = g.p;
    float* nxt = g.p2;
    if (cfg.split || cfg.temporal_depth <= 0) {
        for (int it = 0; it < K; it++) {
            k_sor_colour<<<gc, b, 0, s>>>(L, cur, g.div, g.flags, 0, kp.omega, kp.om1);
            k_sor_colour<<<gc, b, 0, s>>>(L, cur, g.div, g.flags, 1, kp.omega, kp.om1);
            lc.n += 2;
        }
        ZQS_LAUNCH_CHECK("k_sor_colour");
    } else {
        const int Smain = 2 * std::min(cfg.temporal_depth, 4);
        int remaining = 2 * K;
        // z chunk: keep a few waves of CTAs in flight
        const int tiles = ((L.W + 31) / 32) * ((L.H + 15) / 16);
        int zc = L.D;
        while (zc > 16 && (long long)tiles * ((L.D + zc - 1) / zc) < 2 * 152) zc = (zc + 1) / 2;
        while (remaining > 0) {
            int S = std::min(Smain, remaining);
            int rc = launch_tb_depth(S, g, cur, nxt, kp, zc, s);
            if (rc) return rc;
            lc.n++;
            std::swap(cur, nxt);
            remaining -= S;
        }
        ZQS_LAUNCH_CHECK("k_sor_tb");
    }
    dim3 gf((L.W + 1 + 31) / 32, (L.H + 1 + 7) / 8, L.D + 1);
    k_gradient<<<gf, b, 0, s>>>(L, g.u, g.v, g.w, cur, g.flags, closed ? 0 : 1);
    lc.n++;
    ZQS_LAUNCH_CHECK("k_gradient");
    if (p_final) *p_final = cur;
    return ZQS_OK;
}

int launch_stats(const DevGrid& g, const KParams& kp, const float* p, zqs_stats* out, cudaStream_t s) {
    const Layout& L = g.L;
    dim3 b(32, 8, 1);
    dim3 gc((L.W + 31) / 32, (L.H + 7) / 8, L.D);
    long long nblocks = (long long)gc.x * gc.y * gc.z;
    if (3 * nblocks + 2 > g.red_len) {
        set_error("stats: reduction scratch too small");
        return ZQS_EINVAL;
    }
    k_stats<<<gc, b, 0, s>>>(L, g.u, g.v, g.w, p, g.div, g.flags, g.red);
    ZQS_LAUNCH_CHECK("k_stats");
    std::vector<double> h(3 * nblocks);
    ZQS_CUDA_TRY(cudaMemcpyAsync(h.data(), g.red, sizeof(double) * 3 * nblocks, cudaMemcpyDeviceToHost, s));
    ZQS_CUDA_TRY(cudaStreamSynchronize(s));
    double mx = 0.0, r2 = 0.0, nf = 0.0;
    for (long long bb = 0; bb < nblocks; bb++) {
        mx = std::max(mx, h[3 * bb]);
        r2 += h[3 * bb + 1];
        nf += h[3 * bb + 2];
    }
    out->max_abs_div = mx;
    out->residual_l2 = std::sqrt(r2);
    out->free_cells = (int64_t)nf;
    (void)kp;
    return ZQS_OK;
}

}  // namespace zqs
