// Host side of the reverse mode (zqs_grid_set_force, zqs_adjoint_* in
// include/zqs_capi.h).
//
// Forward: the grid steps with its CUDA graphs as usual; every
// checkpoint_every steps the five state fields (u, v, w, T, rho) are copied
// into a checkpoint slot, and the final state into the last slot.
// Backward, one segment at a time from the last: a private work grid restarts
// from the segment's checkpoint and re-runs its steps, keeping each step's
// start state in the segment slots; then the steps are reversed.  For one
// step, the velocity after force + attenuation (the advection input) and the
// vorticity are recomputed from its start state with the forward force
// kernels, the end state gives the projected velocity, and launch_adj_step
// runs the adjoint kernels (kernels_adjoint.cu).  Memory: (nsteps/k + 1) + k
// state slots of 5 padded fields, about 76 padded float fields of adjoint
// buffers (20 float, 14 float4), and one work grid.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "zqs_adjoint.h"
#include "zqs_grid.h"

namespace zqs {

namespace {

int copy3d_raw(void* dst, size_t dpitch, size_t dysize, const void* src, size_t spitch, size_t sysize,
               size_t rowbytes, size_t rows, size_t planes, cudaMemcpyKind kind, cudaStream_t s) {
    cudaMemcpy3DParms m;
    memset(&m, 0, sizeof(m));
    m.srcPtr = make_cudaPitchedPtr(const_cast<void*>(src), spitch, rowbytes, sysize);
    m.dstPtr = make_cudaPitchedPtr(dst, dpitch, rowbytes, dysize);
    m.extent = make_cudaExtent(rowbytes, rows, planes);
    m.kind = kind;
    ZQS_CUDA_TRY(cudaMemcpy3DAsync(&m, s));
    return ZQS_OK;
}

}  // namespace

int copy_dense_padded(float* padded, const float* dense, const Layout& L, int nx, int ny, int nz, bool src_on_device,
                      cudaStream_t s) {
    return copy3d_raw(padded, (size_t)L.px * 4, (size_t)L.py, dense, (size_t)nx * 4, (size_t)ny, (size_t)nx * 4, ny,
                      nz, src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s);
}

int copy_padded_dense(float* dense, const float* padded, const Layout& L, int nx, int ny, int nz, bool dst_on_device,
                      cudaStream_t s) {
    return copy3d_raw(dense, (size_t)nx * 4, (size_t)ny, padded, (size_t)L.px * 4, (size_t)L.py, (size_t)nx * 4, ny,
                      nz, dst_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s);
}

}  // namespace zqs

namespace {

// One saved state: u, v, w, T, rho as whole padded allocations (guards included).
struct Slot {
    float* base = nullptr;
    float* f(const Layout& L, int q) const { return base + (size_t)q * L.elems + L.plane; }
};

float* field_alloc(float* p, const Layout& L) { return p - L.plane; }

int save_state(const Slot& s, const DevGrid& G, cudaStream_t st) {
    const Layout& L = G.L;
    const float* src[5] = {G.u, G.v, G.w, G.T, G.rho};
    for (int q = 0; q < 5; q++)
        ZQS_CUDA_TRY(cudaMemcpyAsync(field_alloc(s.f(L, q), L), src[q] - L.plane, (size_t)L.elems * 4,
                                     cudaMemcpyDeviceToDevice, st));
    return ZQS_OK;
}

int load_state(const Slot& s, DevGrid& G, int nfields, cudaStream_t st) {
    const Layout& L = G.L;
    float* dst[5] = {G.u, G.v, G.w, G.T, G.rho};
    for (int q = 0; q < nfields; q++)
        ZQS_CUDA_TRY(cudaMemcpyAsync(dst[q] - L.plane, field_alloc(s.f(L, q), L), (size_t)L.elems * 4,
                                     cudaMemcpyDeviceToDevice, st));
    return ZQS_OK;
}

bool field_dims(const Layout& L, int field, int& nx, int& ny, int& nz) {
    nx = L.W;
    ny = L.H;
    nz = L.D;
    switch (field) {
        case ZQS_FIELD_U: nx++; return true;
        case ZQS_FIELD_V: ny++; return true;
        case ZQS_FIELD_W: nz++; return true;
        case ZQS_FIELD_TEMPERATURE:
        case ZQS_FIELD_DENSITY: return true;
        default: return false;
    }
}

}  // namespace

struct zqs_adjoint {
    zqs_grid* g = nullptr;   // the user's grid (not owned)
    zqs_grid* wg = nullptr;  // work grid for recomputation (owned)
    int nsteps = 0, every = 1, ncp = 0;
    void* mem = nullptr;
    size_t bytes = 0;
    std::vector<Slot> cp;   // ncp checkpoints + the final state
    std::vector<Slot> seg;  // start states 1..every-1 of the segment being reversed
    AdjBufs b{};
    // fixed inputs of one reversed step (the step's graph reads these):
    // fix0 = start state (its velocity becomes the advection input in place),
    // fix1 = velocity at the end of the step; t4a/t4b = vorticity and force
    Slot fix0, fix1;
    float4 *t4a = nullptr, *t4b = nullptr;
    float4* q4[3] = {};  // quad copies of fix1's velocity
    float4* q2[3] = {};  // quad copies of the advection input (fix0's velocity after the force stage)
    cudaGraphExec_t graph = nullptr;
    long long graph_gen = -1;
    long long graph_launches = 0;
    bool forward_done = false;
    bool backward_done = false;
    long long launches_fwd = 0, launches_bwd = 0;
};

// The launches of one reversed step on the session's fixed buffers: the
// forward force stage on the start state (advection input and vorticity),
// then the adjoint kernels.
int issue_adj_step(zqs_adjoint* a, int K, cudaStream_t s, LaunchCounter& lc) {
    zqs_grid* w = a->wg;
    const Layout& L = w->g.L;
    DevGrid view = w->g;
    view.u = a->fix0.f(L, 0);
    view.v = a->fix0.f(L, 1);
    view.w = a->fix0.f(L, 2);
    view.T = a->fix0.f(L, 3);
    view.rho = a->fix0.f(L, 4);
    view.t4a = a->t4a;
    view.t4b = a->t4b;
    int rc = launch_force(view, w->kp, true, s, lc);
    if (rc) return rc;
    // the samplers' quad copies: advection input (view) and end velocity
    view.qu = a->q2[0];
    view.qv = a->q2[1];
    view.qw = a->q2[2];
    if ((rc = launch_mac_quads(view, s, lc))) return rc;
    DevGrid end = view;
    end.u = a->fix1.f(L, 0);
    end.v = a->fix1.f(L, 1);
    end.w = a->fix1.f(L, 2);
    end.qu = a->q4[0];
    end.qv = a->q4[1];
    end.qw = a->q4[2];
    if ((rc = launch_mac_quads(end, s, lc))) return rc;
    AdjFwd f;
    f.u4 = a->fix1.f(L, 0);
    f.v4 = a->fix1.f(L, 1);
    f.w4 = a->fix1.f(L, 2);
    f.u2 = view.u;
    f.v2 = view.v;
    f.w2 = view.w;
    f.T0 = view.T;
    f.rho0 = view.rho;
    f.vort = view.t4a;
    f.flags = view.flags;
    for (int c = 0; c < 3; c++) {
        f.q4[c] = a->q4[c];
        f.q2[c] = a->q2[c];
    }
    return launch_adj_step(L, f, a->b, w->kp, w->src, K, s, lc);
}

extern "C" {

ZQS_API int zqs_grid_set_force(zqs_grid* g, const float* F, int src_on_device, void* stream) {
    if (!g) {
        set_error("zqs_grid_set_force: NULL grid");
        return ZQS_EINVAL;
    }
    const Layout& L = g->g.L;
    cudaStream_t s = g->pick(stream);
    if (!F) {
        g->fext_on = false;
        g->kp.fext = nullptr;
        g->drop_graphs();
        return ZQS_OK;
    }
    if (!g->fext_base) {
        ZQS_CUDA_TRY(dev_alloc(&g->fext_base, (size_t)L.elems * 3 * 4));
        ZQS_CUDA_TRY(cudaMemsetAsync(g->fext_base, 0, (size_t)L.elems * 3 * 4, s));
    }
    const size_t n = (size_t)L.W * L.H * L.D;
    for (int q = 0; q < 3; q++) {
        int rc = copy_dense_padded(g->fext_base + (size_t)q * L.elems + L.plane, F + q * n, L, L.W, L.H, L.D,
                                   src_on_device != 0, s);
        if (rc) return rc;
    }
    // the captured graphs read the force buffer at run time: only switching
    // the force on needs new graphs (work on stream s is ordered after the copy)
    if (!g->fext_on) {
        g->fext_on = true;
        g->kp.fext = g->fext_base + L.plane;
        g->drop_graphs();
    }
    return ZQS_OK;
}

ZQS_API int zqs_adjoint_create(zqs_adjoint** out, zqs_grid* g, int nsteps, int checkpoint_every) {
    if (!out || !g || nsteps < 1 || checkpoint_every < 1) {
        set_error("zqs_adjoint_create: bad arguments");
        return ZQS_EINVAL;
    }
    *out = nullptr;
    int rc = g->ready();
    if (rc) return rc;
    if (g->params.adv_vel_mode != ZQS_ADV_VEL_INMAC_OUTMAC || g->params.adv_sca_mode != ZQS_ADV_SCA_MAC) {
        set_error("zqs_adjoint_create: the reverse mode needs MAC velocity and MAC scalar advection");
        return ZQS_EUNSUPPORTED;
    }
    if (g->params.solver == ZQS_SOLVER_COARSE_OPEN) {
        set_error("zqs_adjoint_create: the reverse mode covers the fine-grid SOR solvers only");
        return ZQS_EUNSUPPORTED;
    }
    if (g->params.substeps > kAdjMaxSubsteps) {
        set_error("zqs_adjoint_create: at most 32 backtrace substeps are supported");
        return ZQS_EUNSUPPORTED;
    }
    const Layout& L = g->g.L;
    zqs_adjoint* a = new zqs_adjoint();
    a->g = g;
    a->nsteps = nsteps;
    a->every = std::min(checkpoint_every, nsteps);
    a->ncp = (nsteps + a->every - 1) / a->every;
    rc = zqs_grid_create(&a->wg, L.W, L.H, L.D);
    if (rc) {
        delete a;
        return rc;
    }
    auto fail = [&](int code) {
        if (a->mem) cudaFree(a->mem);
        zqs_grid_destroy(a->wg);
        delete a;
        return code;
    };
    // slots: ncp checkpoints + final + (every-1) segment states; adjoint fields
    const size_t fe = (size_t)L.elems;
    const size_t nslots = (size_t)a->ncp + 1 + (size_t)(a->every - 1) + 2;  // + fix0, fix1
    const size_t nflt = 9 + 8 + 3;        // gu.., gu3.., gu2.., gT, grho, gTa, grhoa, q, q2, acc, wt, gF(3)
    const size_t nf4 = 11;                // gom4, gg4, gw4, t4a, t4b, q4 (3), q2 (3)
    const size_t gqe = fe + 2;            // a quad accumulator with its float4 of margin (+1 spare)
    const long long nblocks = (long long)((L.W + 31) / 32) * ((L.H + 7) / 8) * L.D;
    const size_t red_len = (size_t)(2 * nblocks + 16);
    const size_t total = (nslots * 5 + nflt) * fe * 4 + nf4 * fe * 16 + 3 * gqe * 16 + red_len * 8 + 256;
    cudaError_t e = dev_alloc(&a->mem, total);
    if (e != cudaSuccess) return fail(cuda_fail(e, "zqs_adjoint_create: cudaMalloc"));
    e = cudaMemset(a->mem, 0, total);
    if (e != cudaSuccess) return fail(cuda_fail(e, "zqs_adjoint_create: clear"));
    a->bytes = total;
    char* p = (char*)a->mem;
    auto take = [&](size_t nbytes) -> char* {
        char* r = p;
        p += nbytes;
        return r;
    };
    a->cp.resize(a->ncp + 1);
    for (auto& s : a->cp) s.base = (float*)take(5 * fe * 4);
    a->seg.resize(a->every);  // index 0 unused (the checkpoint itself)
    for (int t = 1; t < a->every; t++) a->seg[t].base = (float*)take(5 * fe * 4);
    a->fix0.base = (float*)take(5 * fe * 4);
    a->fix1.base = (float*)take(5 * fe * 4);
    auto fld = [&]() -> float* { return (float*)take(fe * 4) + L.plane; };
    AdjBufs& b = a->b;
    b.gu = fld();
    b.gv = fld();
    b.gw = fld();
    b.gu3 = fld();
    b.gv3 = fld();
    b.gw3 = fld();
    b.gu2 = fld();
    b.gv2 = fld();
    b.gw2 = fld();
    b.gT = fld();
    b.grho = fld();
    b.gTa = fld();
    b.grhoa = fld();
    b.q = fld();
    b.q2 = fld();
    b.acc = fld();
    b.wt = fld();
    b.gF = (float*)take(3 * fe * 4) + L.plane;
    b.gom4 = (float4*)take(fe * 16) + L.plane;
    b.gg4 = (float4*)take(fe * 16) + L.plane;
    b.gw4 = (float4*)take(fe * 16) + L.plane;
    a->t4a = (float4*)take(fe * 16) + L.plane;
    a->t4b = (float4*)take(fe * 16) + L.plane;
    for (int c = 0; c < 3; c++) a->q4[c] = (float4*)take(fe * 16) + L.plane;
    for (int c = 0; c < 3; c++) a->q2[c] = (float4*)take(fe * 16) + L.plane;
    for (int c = 0; c < 3; c++) b.gq[c] = (float4*)take(gqe * 16) + L.plane + 1;
    b.red = (double*)take(red_len * 8);
    b.red_len = (long long)red_len;
    // the work grid: same parameters, occupancy and SOR setup
    zqs_grid* w = a->wg;
    rc = zqs_grid_set_params(w, &g->params);
    if (rc) return fail(rc);
    rc = zqs_grid_upload(w, ZQS_FIELD_OCCUPANCY, g->occ_dense, 1, nullptr);
    if (rc) return fail(rc);
    w->sor = g->sor;
    e = cudaStreamSynchronize(w->own);
    if (e != cudaSuccess) return fail(cuda_fail(e, "zqs_adjoint_create: work grid"));
    // sizes: the work grid's own allocation counts too
    a->bytes += (size_t)fe * 4 * 13 + (size_t)fe * 16 * 5 + (size_t)fe + (size_t)L.W * L.H * L.D;
    *out = a;
    return ZQS_OK;
}

ZQS_API int zqs_adjoint_destroy(zqs_adjoint* a) {
    if (!a) return ZQS_OK;
    if (a->graph) cudaGraphExecDestroy(a->graph);
    if (a->wg) {
        cudaStreamSynchronize(a->wg->own);
        zqs_grid_destroy(a->wg);
    }
    if (a->mem) cudaFree(a->mem);
    delete a;
    return ZQS_OK;
}

ZQS_API int zqs_adjoint_forward(zqs_adjoint* a, const float* F, int src_on_device, void* stream) {
    if (!a) {
        set_error("zqs_adjoint_forward: NULL session");
        return ZQS_EINVAL;
    }
    zqs_grid* g = a->g;
    int rc = g->ready();
    if (rc) return rc;
    cudaStream_t s = g->pick(stream);
    rc = zqs_grid_set_force(g, F, src_on_device, s);
    if (rc) return rc;
    long long n = 0;
    for (int t = 0; t < a->nsteps; t++) {
        if (t % a->every == 0) {
            rc = save_state(a->cp[t / a->every], g->g, s);
            if (rc) return rc;
        }
        rc = zqs_grid_step(g, 1, s);
        if (rc) return rc;
        n += g->step_launches;
    }
    rc = save_state(a->cp[a->ncp], g->g, s);
    if (rc) return rc;
    a->launches_fwd = n;
    a->forward_done = true;
    a->backward_done = false;
    return ZQS_OK;
}

ZQS_API int zqs_adjoint_backward(zqs_adjoint* a, const float* g_density, float* grad_F, int on_device,
                                 void* stream) {
    if (!a || !g_density) {
        set_error("zqs_adjoint_backward: NULL argument");
        return ZQS_EINVAL;
    }
    if (!a->forward_done) {
        set_error("zqs_adjoint_backward: run zqs_adjoint_forward first");
        return ZQS_ENOTREADY;
    }
    zqs_grid* g = a->g;
    zqs_grid* w = a->wg;
    const Layout& L = g->g.L;
    cudaStream_t s = g->pick(stream);
    // the work grid follows the grid's parameters, SOR setup and force
    // (its graphs are kept while none of them changes)
    int rc = ZQS_OK;
    if (memcmp(&w->params, &g->params, sizeof(zqs_params)) != 0) {
        rc = zqs_grid_set_params(w, &g->params);
        if (rc) return rc;
    }
    if (memcmp(&w->sor, &g->sor, sizeof(SorConfig)) != 0) {
        w->sor = g->sor;
        w->drop_graphs();
    }
    if (g->fext_on) {
        if (!w->fext_base) {
            ZQS_CUDA_TRY(dev_alloc(&w->fext_base, (size_t)L.elems * 3 * 4));
        }
        ZQS_CUDA_TRY(cudaMemcpyAsync(w->fext_base, g->fext_base, (size_t)L.elems * 3 * 4, cudaMemcpyDeviceToDevice,
                                     s));
        if (!w->fext_on) {
            w->fext_on = true;
            w->kp.fext = w->fext_base + L.plane;
            w->drop_graphs();
        }
    } else if (w->fext_on) {
        w->fext_on = false;
        w->kp.fext = nullptr;
        w->drop_graphs();
    }
    const AdjBufs& b = a->b;
    const size_t fe = (size_t)L.elems;
    LaunchCounter lc;
    // zero the adjoint state and gF, then seed gdensity
    float* zero_list[] = {b.gu, b.gv, b.gw, b.gT, b.grho};
    for (float* f : zero_list) ZQS_CUDA_TRY(cudaMemsetAsync(f - L.plane, 0, fe * 4, s));
    ZQS_CUDA_TRY(cudaMemsetAsync(b.gF - L.plane, 0, 3 * fe * 4, s));
    rc = copy_dense_padded(b.grho, g_density, L, L.W, L.H, L.D, on_device != 0, s);
    if (rc) return rc;
    rc = launch_adj_weights(L, w->g.flags, w->kp.omega, b.wt, s, lc);
    if (rc) return rc;
    const int K = g->params.sor_iters;
    if (K > 1) {  // before the first capture; q, q2 and acc are set up again by every reversed step
        rc = sor_adj_autotune(L, b.q, b.q2, b.wt, b.acc, w->kp.om1, s);
        if (rc) return rc;
    }
    for (int sg = a->ncp - 1; sg >= 0; sg--) {
        const int s0 = sg * a->every;
        const int s1 = std::min(s0 + a->every, a->nsteps);
        const int len = s1 - s0;
        auto state = [&](int t) -> const Slot& {
            if (t == 0) return a->cp[sg];
            if (t == len) return a->cp[sg + 1];
            return a->seg[t];
        };
        // recompute the segment's start states 1..len-1
        if (len > 1) {
            rc = load_state(a->cp[sg], w->g, 5, s);
            if (rc) return rc;
            for (int t = 1; t < len; t++) {
                rc = zqs_grid_step(w, 1, s);
                if (rc) return rc;
                lc.n += w->step_launches;
                rc = save_state(a->seg[t], w->g, s);
                if (rc) return rc;
            }
        }
        for (int t = len - 1; t >= 0; t--) {
            const Slot& S0 = state(t);
            const Slot& S1 = state(t + 1);
            // this step's inputs into the fixed buffers the step graph reads
            for (int q = 0; q < 5; q++)
                ZQS_CUDA_TRY(cudaMemcpyAsync(a->fix0.base + q * fe, S0.base + q * fe, fe * 4,
                                             cudaMemcpyDeviceToDevice, s));
            for (int q = 0; q < 3; q++)
                ZQS_CUDA_TRY(cudaMemcpyAsync(a->fix1.base + q * fe, S1.base + q * fe, fe * 4,
                                             cudaMemcpyDeviceToDevice, s));
            if (!a->graph || a->graph_gen != w->gen) {
                if (a->graph) cudaGraphExecDestroy(a->graph);
                a->graph = nullptr;
                LaunchCounter glc;
                ZQS_CUDA_TRY(cudaStreamBeginCapture(w->own, cudaStreamCaptureModeThreadLocal));
                rc = issue_adj_step(a, K, w->own, glc);
                cudaGraph_t gr = nullptr;
                cudaError_t e = cudaStreamEndCapture(w->own, &gr);
                if (rc) {
                    if (gr) cudaGraphDestroy(gr);
                    return rc;
                }
                if (e != cudaSuccess) return cuda_fail(e, "zqs_adjoint_backward: cudaStreamEndCapture");
                e = cudaGraphInstantiate(&a->graph, gr, 0);
                cudaGraphDestroy(gr);
                if (e != cudaSuccess) {
                    a->graph = nullptr;
                    return cuda_fail(e, "zqs_adjoint_backward: cudaGraphInstantiate");
                }
                a->graph_gen = w->gen;
                a->graph_launches = glc.n;
            }
            ZQS_CUDA_TRY(cudaGraphLaunch(a->graph, s));
            lc.n += a->graph_launches;
        }
    }
    if (grad_F) {
        const size_t n = (size_t)L.W * L.H * L.D;
        for (int q = 0; q < 3; q++) {
            rc = copy_padded_dense(grad_F + q * n, b.gF + (size_t)q * fe, L, L.W, L.H, L.D, on_device != 0, s);
            if (rc) return rc;
        }
    }
    a->launches_bwd = lc.n;
    a->backward_done = true;
    return ZQS_OK;
}

ZQS_API int zqs_adjoint_download(zqs_adjoint* a, int field, void* dst, int dst_on_device, void* stream) {
    if (!a || !dst) {
        set_error("zqs_adjoint_download: NULL argument");
        return ZQS_EINVAL;
    }
    if (!a->backward_done) {
        set_error("zqs_adjoint_download: run zqs_adjoint_backward first");
        return ZQS_ENOTREADY;
    }
    const Layout& L = a->g->g.L;
    int nx, ny, nz;
    if (!field_dims(L, field, nx, ny, nz)) {
        set_error("zqs_adjoint_download: field must be U, V, W, TEMPERATURE or DENSITY");
        return ZQS_EINVAL;
    }
    const float* src = field == ZQS_FIELD_U ? a->b.gu
                       : field == ZQS_FIELD_V ? a->b.gv
                       : field == ZQS_FIELD_W ? a->b.gw
                       : field == ZQS_FIELD_TEMPERATURE ? a->b.gT
                                                        : a->b.grho;
    return copy_padded_dense((float*)dst, src, L, nx, ny, nz, dst_on_device != 0, a->g->pick(stream));
}

ZQS_API int zqs_adjoint_get_info(const zqs_adjoint* a, zqs_adjoint_info* out) {
    if (!a || !out) {
        set_error("zqs_adjoint_get_info: NULL argument");
        return ZQS_EINVAL;
    }
    memset(out, 0, sizeof(*out));
    out->device_bytes = (int64_t)a->bytes;
    out->launches_forward = a->launches_fwd;
    out->launches_backward = a->launches_bwd;
    out->nsteps = a->nsteps;
    out->checkpoint_every = a->every;
    out->checkpoints = a->ncp + 1;
    return ZQS_OK;
}

}  // extern "C"
