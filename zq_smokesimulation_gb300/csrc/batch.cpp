// Batched mixed-size runner (zqs_batch_* in include/zqs_capi.h).
//
// One instance table (InstDesc per member grid, device resident) and, per tile
// shape class, a prefix array of tile counts; every stage of the step is one
// persistent launch over the concatenated tile lists (kernels_*.cu, *_batch).
// Members are ordered by cell count, largest first, so the longest SOR tiles
// are handed out first.  The step is captured once per buffer parity and
// replayed as a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "zqs_batch.h"
#include "zqs_grid.h"

struct zqs_batch {
    std::vector<zqs_grid*> grids;
    std::vector<long long> gens;  // member generations the table was built from
    std::vector<int> order;       // table row -> member index
    std::vector<InstDesc> h_desc;
    void* dev = nullptr;
    size_t dev_bytes = 0;
    InstDesc* d_desc = nullptr;
    int* d_pre[TC_COUNT] = {};
    std::vector<int> h_pre[TC_COUNT];   // host copies of the prefix arrays
    std::vector<AdvHotTable> hot;       // advection parameter tables, kAdvHotMax instances each
    int total[TC_COUNT] = {};
    int n = 0;
    int K = 0;
    bool any_closed = false;
    SorBatchPlan plan;
    int variant = -1;      // as set by zqs_batch_set_sor_variant (-1: tuned)
    int zchunk = 0;
    int tuned_variant = -1;  // the batchable variant measured fastest on this batch
    float tuned_us = 0.0f;   // its time per SOR iteration
    int par = 0;          // table buffer index holding the current velocity and scalars
    bool built = false;
    cudaStream_t own = nullptr;
    bool use_graph = true;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    long long graph_launches[2] = {0, 0};
    int graph_pfin[2] = {0, 0};
    long long step_launches = 0;
    int blocks = 0;       // persistent grid of the 256-thread stages

    void drop_graphs() {
        for (int q = 0; q < 2; q++) {
            if (graph[q]) cudaGraphExecDestroy(graph[q]);
            graph[q] = nullptr;
        }
    }
};

namespace zqs {

int persistent_blocks(const void* kernel, int threads, size_t dyn_smem, int cap) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, int> resident;  // (kernel, device) -> blocks
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return std::max(1, cap);
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_pair(kernel, dev);
    auto it = resident.find(key);
    if (it == resident.end()) {
        int per_sm = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, dyn_smem) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return std::max(1, cap);
        }
        it = resident.emplace(key, std::max(1, per_sm) * std::max(1, sms)).first;
    }
    return std::max(1, std::min(cap, it->second));
}

}  // namespace zqs

namespace {

int check_members(zqs_batch* b) {
    const int n = (int)b->grids.size();
    for (int i = 0; i < n; i++) {
        zqs_grid* g = b->grids[i];
        int rc = g->ready();
        if (rc) {
            set_error("zqs_batch: member " + std::to_string(i) + ": " + std::string(zqs_last_error()));
            return rc;
        }
        if (g->params.adv_vel_mode != ZQS_ADV_VEL_INMAC_OUTMAC || g->params.adv_sca_mode != ZQS_ADV_SCA_MAC) {
            set_error("zqs_batch: member " + std::to_string(i) +
                      " must use ZQS_ADV_VEL_INMAC_OUTMAC and ZQS_ADV_SCA_MAC advection");
            return ZQS_EUNSUPPORTED;
        }
        if (g->params.solver == ZQS_SOLVER_COARSE_OPEN) {
            set_error("zqs_batch: member " + std::to_string(i) + " uses the coarse-grid solver (not batched)");
            return ZQS_EUNSUPPORTED;
        }
        if (g->params.sor_iters != b->grids[0]->params.sor_iters) {
            set_error("zqs_batch: every member must use the same sor_iters");
            return ZQS_EUNSUPPORTED;
        }
    }
    return ZQS_OK;
}

int ceil_div(int a, int b) { return (a + b - 1) / b; }

// Tiles of one instance for a tile class.
int class_tiles(const Layout& L, int cls, const SorBatchPlan& plan, const int zc[2]) {
    switch (cls) {
        case TC_CELL: return ceil_div(L.W, 32) * ceil_div(L.H, 8) * L.D;
        case TC_FACE: return ceil_div(L.W + 1, 32) * ceil_div(L.H + 1, 8) * (L.D + 1);
        case TC_ADVF: return ceil_div(L.W + 1, 32) * ceil_div(L.H + 1, 8) * 3 * (L.D + 1);
        case TC_SORM:
        case TC_SORR: {
            const int q = cls - TC_SORM;
            return ceil_div(L.W, plan.TX[q]) * ceil_div(L.H, plan.TY[q]) * ceil_div(L.D, zc[q]);
        }
        default: return 0;
    }
}

// z chunk per instance for SOR pass kind q: the common chunk whose static
// round-robin assignment of tiles to the resident CTAs has the shortest
// longest CTA (work of a tile = its planes + the 3S+1 pipeline fill steps).
void choose_batch_zc(const std::vector<Layout>& Ls, const SorBatchPlan& plan, int q, int forced,
                     std::vector<int>& zc) {
    const int n = (int)Ls.size();
    zc.assign(n, 1);
    int maxd = 1;
    for (const Layout& L : Ls) maxd = std::max(maxd, L.D);
    if (forced > 0) {
        for (int i = 0; i < n; i++) zc[i] = std::min(forced, Ls[i].D);
        return;
    }
    const int slots = std::max(1, plan.slots[q]);
    const int fill = 3 * plan.S[q] + 1;
    std::vector<long long> load(slots);
    long long best = -1;
    int best_z = maxd;
    for (int zt : {8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512}) {
        const int z = std::min(zt, maxd);
        std::fill(load.begin(), load.end(), 0);
        long long t = 0;
        for (int i = 0; i < n; i++) {
            const Layout& L = Ls[i];
            const int zi = std::min(z, L.D);
            const int cols = ceil_div(L.W, plan.TX[q]) * ceil_div(L.H, plan.TY[q]);
            const int chunks = ceil_div(L.D, zi);
            for (int c = 0; c < chunks; c++) {
                const int len = std::min(zi, L.D - c * zi) + fill;
                for (int col = 0; col < cols; col++) load[(size_t)((t++) % slots)] += len;
            }
        }
        const long long mk = *std::max_element(load.begin(), load.end());
        if (best < 0 || mk < best) {
            best = mk;
            best_z = z;
        }
        if (z == maxd) break;
    }
    for (int i = 0; i < n; i++) zc[i] = std::min(best_z, Ls[i].D);
}

int build_table_for(zqs_batch* b, int variant) {
    int rc = check_members(b);
    if (rc) return rc;
    rc = sor_batch_plan(variant, b->plan);
    if (rc) return rc;
    const int n = (int)b->grids.size();
    b->n = n;
    b->K = b->grids[0]->params.sor_iters;
    b->order.resize(n);
    std::iota(b->order.begin(), b->order.end(), 0);
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) {
        const Layout& a = b->grids[x]->g.L;
        const Layout& c = b->grids[y]->g.L;
        return (long long)a.W * a.H * a.D > (long long)c.W * c.H * c.D;
    });
    std::vector<Layout> Ls(n);
    for (int r = 0; r < n; r++) Ls[r] = b->grids[b->order[r]]->g.L;
    std::vector<int> zc0, zc1;
    choose_batch_zc(Ls, b->plan, 0, b->zchunk, zc0);
    choose_batch_zc(Ls, b->plan, 1, b->zchunk, zc1);

    b->h_desc.assign(n, InstDesc{});
    b->any_closed = false;
    std::vector<int> pre[TC_COUNT];
    for (int c = 0; c < TC_COUNT; c++) pre[c].assign(n + 1, 0);
    for (int r = 0; r < n; r++) {
        zqs_grid* g = b->grids[b->order[r]];
        InstDesc& d = b->h_desc[r];
        memset(&d, 0, sizeof(d));
        const DevGrid& G = g->g;
        d.L = G.L;
        d.vel[0][0] = G.u;
        d.vel[0][1] = G.v;
        d.vel[0][2] = G.w;
        d.vel[1][0] = G.u2;
        d.vel[1][1] = G.v2;
        d.vel[1][2] = G.w2;
        d.sca[0][0] = G.T;
        d.sca[0][1] = G.rho;
        d.sca[1][0] = G.T2;
        d.sca[1][1] = G.rho2;
        d.p[0] = G.p;
        d.p[1] = G.p2;
        d.div = G.div;
        d.flags = G.flags;
        d.t4a = G.t4a;
        d.t4b = G.t4b;
        d.q4[0] = G.qu;
        d.q4[1] = G.qv;
        d.q4[2] = G.qw;
        d.red = G.red;
        d.red_len = G.red_len;
        d.kp = g->kp;
        d.src = g->src;
        d.zc[0] = zc0[r];
        d.zc[1] = zc1[r];
        d.closed = g->params.solver == ZQS_SOLVER_CLOSED ? 1 : 0;
        b->any_closed = b->any_closed || d.closed;
        for (int c = 0; c < TC_COUNT; c++) {
            const long long next = (long long)pre[c][r] + class_tiles(d.L, c, b->plan, d.zc);
            if (next >= (1LL << 31)) {
                set_error("zqs_batch: tile count exceeds 32-bit indexing");
                return ZQS_EINVAL;
            }
            pre[c][r + 1] = (int)next;
        }
    }
    for (int c = 0; c < TC_COUNT; c++) {
        b->total[c] = pre[c][n];
        b->h_pre[c] = pre[c];
    }
    // the advection kernels' parameter tables, one per chunk of instances
    b->hot.clear();
    for (int c0 = 0; c0 < n; c0 += kAdvHotMax) {
        b->hot.emplace_back();
        AdvHotTable& T = b->hot.back();
        memset(&T, 0, sizeof(T));
        T.base = c0;
        T.n = std::min(kAdvHotMax, n - c0);
        for (int q = 0; q < T.n; q++) {
            const InstDesc& d = b->h_desc[c0 + q];
            AdvHot& a = T.h[q];
            a.L = d.L;
            a.kp = d.kp;
            for (int m = 0; m < 3; m++) {
                a.q[m] = d.q4[m];
                a.vel[0][m] = d.vel[0][m];
                a.vel[1][m] = d.vel[1][m];
            }
            a.flags = d.flags;
            for (int m = 0; m < 2; m++) {
                a.sca[0][m] = d.sca[0][m];
                a.sca[1][m] = d.sca[1][m];
            }
        }
    }

    // one device block: descriptors, then the prefix arrays
    const size_t desc_bytes = ((sizeof(InstDesc) * n + 255) / 256) * 256;
    const size_t pre_bytes = ((sizeof(int) * (n + 1) + 255) / 256) * 256;
    const size_t need = desc_bytes + TC_COUNT * pre_bytes;
    if (need > b->dev_bytes) {
        if (b->dev) {
            cudaStreamSynchronize(b->own);
            cudaFree(b->dev);
            b->dev = nullptr;
            b->dev_bytes = 0;
        }
        ZQS_CUDA_TRY(dev_alloc(&b->dev, need));
        b->dev_bytes = need;
    }
    char* base = (char*)b->dev;
    b->d_desc = (InstDesc*)base;
    for (int c = 0; c < TC_COUNT; c++) b->d_pre[c] = (int*)(base + desc_bytes + c * pre_bytes);
    // member grids may have work queued on their own streams: let it finish first
    for (zqs_grid* g : b->grids) ZQS_CUDA_TRY(cudaStreamSynchronize(g->own));
    ZQS_CUDA_TRY(cudaMemcpyAsync(b->d_desc, b->h_desc.data(), sizeof(InstDesc) * n, cudaMemcpyHostToDevice, b->own));
    for (int c = 0; c < TC_COUNT; c++)
        ZQS_CUDA_TRY(
            cudaMemcpyAsync(b->d_pre[c], pre[c].data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, b->own));
    ZQS_CUDA_TRY(cudaStreamSynchronize(b->own));
    b->gens.resize(n);
    for (int i = 0; i < n; i++) b->gens[i] = b->grids[i]->gen;
    b->par = 0;
    b->drop_graphs();
    b->built = true;
    return ZQS_OK;
}

// Time per iteration of the batch's main SOR pass with the tables as built
// (pressure of every member overwritten; the next projection restarts at 0).
int time_batch_sor(zqs_batch* b, float& us) {
    BatchLaunch bm{b->d_desc, b->d_pre[TC_SORM], b->n, b->total[TC_SORM]};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ZQS_CUDA_TRY(cudaEventCreate(&e0));
    cudaError_t e = cudaEventCreate(&e1);
    constexpr int kReps = 3;
    if (e == cudaSuccess) e = launch_sor_batch_pass(b->plan, 0, bm, 0, b->own);  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, b->own);
    for (int r = 0; r < kReps && e == cudaSuccess; r++) e = launch_sor_batch_pass(b->plan, 0, bm, (r + 1) & 1, b->own);
    if (e == cudaSuccess) e = cudaEventRecord(e1, b->own);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(e, "zqs_batch: SOR tuning");
    us = 1000.0f * ms / (kReps * (b->plan.S[0] / 2));
    return ZQS_OK;
}

// The tables for the configured variant; with variant -1 (and ZQS_AUTOTUNE
// not 0) every batchable variant is timed on this batch's own tile lists once
// and the fastest per iteration kept (all give bit-identical results).
int build_table(zqs_batch* b) {
    if (b->variant >= 0) return build_table_for(b, b->variant);
    const char* env = std::getenv("ZQS_AUTOTUNE");
    if ((env && env[0] == '0') || b->grids[0]->params.sor_iters == 0) return build_table_for(b, -1);
    if (b->tuned_variant < 0) {
        float best = 1e30f;
        for (int v = 0; v < sor_variant_count(); v++) {
            if (!sor_variant_batchable(v)) continue;
            int rc = build_table_for(b, v);
            if (rc) return rc;
            float us = 0.0f;
            rc = time_batch_sor(b, us);
            if (rc) return rc;
            if (us < best) {
                best = us;
                b->tuned_variant = v;
                b->tuned_us = us;
            }
        }
        if (b->tuned_variant < 0) return build_table_for(b, -1);
    }
    return build_table_for(b, b->tuned_variant);
}

// The table is current when no member changed and every member's current
// buffers are the table's buffers of parity par.
bool table_current(const zqs_batch* b) {
    if (!b->built) return false;
    for (int r = 0; r < b->n; r++) {
        const int m = b->order[r];
        const zqs_grid* g = b->grids[m];
        const InstDesc& d = b->h_desc[r];
        if (g->gen != b->gens[m]) return false;
        if (g->g.u != d.vel[b->par][0] || g->g.T != d.sca[b->par][0]) return false;
    }
    return true;
}

int issue_batch_step(zqs_batch* b, int par, cudaStream_t s, LaunchCounter& lc, int* pfin) {
    BatchLaunch bl[TC_COUNT];
    for (int c = 0; c < TC_COUNT; c++)
        bl[c] = BatchLaunch{b->d_desc, b->d_pre[c], b->n, b->total[c], b->h_pre[c].data()};
    int rc = launch_force_batch(bl[TC_CELL], bl[TC_FACE], par, par, b->blocks, s, lc);
    if (rc) return rc;
    rc = launch_mac_quads_batch(bl[TC_FACE], par, b->blocks, s, lc);
    if (rc) return rc;
    rc = launch_advect_velocity_batch(bl[TC_ADVF], b->hot, par, s, lc);
    if (rc) return rc;
    rc = launch_project_batch(bl[TC_CELL], bl[TC_FACE], bl[TC_SORM], bl[TC_SORR], b->plan, b->K, b->any_closed,
                              par ^ 1, b->blocks, s, lc, pfin);
    if (rc) return rc;
    rc = launch_mac_quads_batch(bl[TC_FACE], par ^ 1, b->blocks, s, lc);
    if (rc) return rc;
    return launch_advect_scalar_batch(bl[TC_CELL], b->hot, par ^ 1, par, s, lc);
}

}  // namespace

extern "C" {

ZQS_API int zqs_batch_create(zqs_batch** out, zqs_grid* const* grids, int n) {
    if (!out) {
        set_error("zqs_batch_create: out is NULL");
        return ZQS_EINVAL;
    }
    *out = nullptr;
    if (!grids || n < 1) {
        set_error("zqs_batch_create: need at least one grid");
        return ZQS_EINVAL;
    }
    for (int i = 0; i < n; i++) {
        if (!grids[i]) {
            set_error("zqs_batch_create: grid " + std::to_string(i) + " is NULL");
            return ZQS_EINVAL;
        }
        for (int j = 0; j < i; j++)
            if (grids[j] == grids[i]) {
                set_error("zqs_batch_create: grid " + std::to_string(i) + " appears twice");
                return ZQS_EINVAL;
            }
    }
    int rc = sor_prepare();
    if (rc) return rc;
    zqs_batch* b = new zqs_batch();
    b->grids.assign(grids, grids + n);
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(e, "zqs_batch_create");
    }
    b->blocks = std::max(1, sms) * 8;  // at most 8 resident 256-thread CTAs per SM (persistent_blocks)
    rc = build_table(b);
    if (rc) {
        if (b->dev) cudaFree(b->dev);
        cudaStreamDestroy(b->own);
        delete b;
        return rc;
    }
    *out = b;
    return ZQS_OK;
}

ZQS_API int zqs_batch_destroy(zqs_batch* b) {
    if (!b) return ZQS_OK;
    b->drop_graphs();
    if (b->own) cudaStreamSynchronize(b->own);
    if (b->dev) cudaFree(b->dev);
    if (b->own) cudaStreamDestroy(b->own);
    delete b;
    return ZQS_OK;
}

ZQS_API int zqs_batch_use_graph(zqs_batch* b, int enable) {
    if (!b) {
        set_error("zqs_batch_use_graph: NULL batch");
        return ZQS_EINVAL;
    }
    b->use_graph = enable != 0;
    if (!b->use_graph) b->drop_graphs();
    return ZQS_OK;
}

ZQS_API int zqs_batch_set_sor_variant(zqs_batch* b, int index, int zchunk) {
    if (!b || index < -1 || index >= sor_variant_count() || zchunk < 0) {
        set_error("zqs_batch_set_sor_variant: bad arguments");
        return ZQS_EINVAL;
    }
    if (index >= 0 && !sor_variant_batchable(index)) {
        set_error("zqs_batch_set_sor_variant: variant " + std::to_string(index) +
                  " has no batched form (register-column variants only) or does not fit");
        return ZQS_EUNSUPPORTED;
    }
    b->variant = index;
    b->zchunk = zchunk;
    b->tuned_variant = -1;
    b->built = false;  // rebuilt (tile lists change) at the next step
    b->drop_graphs();
    return ZQS_OK;
}

ZQS_API int zqs_batch_step(zqs_batch* b, int nsteps, void* stream) {
    if (!b || nsteps < 0) {
        set_error("zqs_batch_step: bad arguments");
        return ZQS_EINVAL;
    }
    cudaStream_t s = stream ? (cudaStream_t)stream : b->own;
    for (int step = 0; step < nsteps; step++) {
        if (!table_current(b)) {
            int rc = build_table(b);
            if (rc) return rc;
        }
        const int par = b->par;
        int pfin = 0;
        if (!b->use_graph) {
            LaunchCounter lc;
            int rc = issue_batch_step(b, par, s, lc, &pfin);
            if (rc) return rc;
            b->step_launches = lc.n;
        } else {
            if (!b->graph[par]) {
                LaunchCounter lc;
                ZQS_CUDA_TRY(cudaStreamBeginCapture(b->own, cudaStreamCaptureModeThreadLocal));
                int rc = issue_batch_step(b, par, b->own, lc, &pfin);
                cudaGraph_t graph = nullptr;
                cudaError_t e = cudaStreamEndCapture(b->own, &graph);
                if (rc) {
                    if (graph) cudaGraphDestroy(graph);
                    return rc;
                }
                if (e != cudaSuccess) return cuda_fail(e, "zqs_batch_step: cudaStreamEndCapture");
                e = cudaGraphInstantiate(&b->graph[par], graph, 0);
                cudaGraphDestroy(graph);
                if (e != cudaSuccess) {
                    b->graph[par] = nullptr;
                    return cuda_fail(e, "zqs_batch_step: cudaGraphInstantiate");
                }
                b->graph_launches[par] = lc.n;
                b->graph_pfin[par] = pfin;
            }
            ZQS_CUDA_TRY(cudaGraphLaunch(b->graph[par], s));
            pfin = b->graph_pfin[par];
            b->step_launches = b->graph_launches[par];
        }
        // every member's buffers advance as zqs_grid_step would advance them
        for (zqs_grid* g : b->grids) {
            g->swap_velocity();
            g->swap_scalars();
            g->p_last = pfin ? g->g.p2 : g->g.p;
        }
        b->par ^= 1;
    }
    return ZQS_OK;
}

ZQS_API int64_t zqs_batch_launch_count(const zqs_batch* b) { return b ? b->step_launches : 0; }

ZQS_API int zqs_batch_get_sor_choice(const zqs_batch* b, int* variant, float* us_per_iter) {
    if (!b) return set_error("zqs_batch_get_sor_choice: NULL batch"), ZQS_EINVAL;
    if (variant) *variant = b->plan.vmain;
    if (us_per_iter) *us_per_iter = (b->variant < 0 && b->plan.vmain == b->tuned_variant) ? b->tuned_us : 0.0f;
    return ZQS_OK;
}

ZQS_API int zqs_batch_synchronize(zqs_batch* b, void* stream) {
    if (!b) return set_error("NULL batch"), ZQS_EINVAL;
    ZQS_CUDA_TRY(cudaStreamSynchronize(stream ? (cudaStream_t)stream : b->own));
    return ZQS_OK;
}

}  // extern "C"
