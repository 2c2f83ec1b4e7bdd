// Internal definition of the zqs_grid handle, shared by the single-grid C ABI
// (capi.cpp) and the batched runner (batch.cpp).  Not installed.
#pragma once

#include <cstdlib>
#include <utility>

#include "zqs_internal.h"

using namespace zqs;  // internal header of two translation units

struct zqs_grid {
    DevGrid g{};
    void* base = nullptr;
    uint8_t* occ_dense = nullptr;
    cudaStream_t own = nullptr;
    zqs_params params{};
    bool has_params = false;
    bool has_occ = false;
    KParams kp{};
    SourceList src{};
    SorConfig sor{};               // as configured (temporal_depth 0: the tuned variant)
    SorConfig sor_eff{};           // as launched: sor with the tuned variant filled in
    SorChoice tuned{};             // sor_autotune's result for this grid's shape
    bool tune_done = false;
    float* p_last = nullptr;
    bool use_graph = true;
    cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
    int vel_par = 0, sca_par = 0;   // which buffer of each ping-pong pair is current
    long long step_launches = 0;
    long long graph_launches[4] = {0, 0, 0, 0};
    float* graph_p_last[4] = {nullptr, nullptr, nullptr, nullptr};
    long long gen = 0;  // bumped whenever parameters, occupancy or the SOR setup change
    float* fext_base = nullptr;  // external per-cell force, 3 padded cell fields (allocated on first use)
    bool fext_on = false;
    int coarse_tc = 1;            // coarse solver's obstacle-free blocks: 1 tensor cores, 0 FP32 SIMT
    uint8_t* obj_mask = nullptr;  // device copy of a moving object's voxel mask (grown on demand)
    size_t obj_mask_cap = 0;
    float* stage = nullptr;       // dense staging buffer of host transfers (grown on demand)
    size_t stage_cap = 0;
    cudaEvent_t stage_ev = nullptr;  // the staging buffer's last use

    cudaStream_t pick(void* s) const { return s ? (cudaStream_t)s : own; }

    void drop_graphs() {
        gen++;
        for (int q = 0; q < 4; q++) {
            if (graph[q]) cudaGraphExecDestroy(graph[q]);
            graph[q] = nullptr;
        }
    }
    void swap_velocity() {
        std::swap(g.u, g.u2);
        std::swap(g.v, g.v2);
        std::swap(g.w, g.w2);
        vel_par ^= 1;
    }
    void swap_scalars() {
        std::swap(g.T, g.T2);
        std::swap(g.rho, g.rho2);
        sca_par ^= 1;
    }
    int ready() const {
        if (!has_params) {
            set_error("grid has no parameters (call zqs_grid_set_params)");
            return ZQS_ENOTREADY;
        }
        if (!has_occ) {
            set_error("grid has no occupancy (upload ZQS_FIELD_OCCUPANCY)");
            return ZQS_ENOTREADY;
        }
        return ZQS_OK;
    }
    // The SOR configuration to launch.  With temporal_depth 0 and no explicit
    // variant the tuned variant and z chunk are used; the tuner runs on the
    // first call that is not inside a stream capture (it synchronises s), and
    // ZQS_AUTOTUNE=0 in the environment keeps the static default instead.
    int resolve_sor(cudaStream_t s) {
        sor_eff = sor;
        if (sor.split || sor.temporal_depth != 0 || sor.variant >= 0) return ZQS_OK;
        // no fine-grid SOR to tune (coarse solver, or no iterations yet)
        if (params.solver == ZQS_SOLVER_COARSE_OPEN || params.sor_iters == 0) return ZQS_OK;
        if (!tune_done) {
            const char* env = std::getenv("ZQS_AUTOTUNE");
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) cs = cudaStreamCaptureStatusActive;
            if (env && env[0] == '0') {
                tune_done = true;  // static default
            } else if (cs == cudaStreamCaptureStatusNone) {
                int rc = sor_autotune(g, kp, s, tuned);
                if (rc) return rc;
                tune_done = true;
            }
        }
        if (tuned.variant >= 0) {
            sor_eff.variant = tuned.variant;
            sor_eff.zchunk = tuned.zchunk;
        }
        return ZQS_OK;
    }
    // The launches of one step, issued on stream s (captured or direct).
    int issue_step(cudaStream_t s, LaunchCounter& lc) {
        int rc = launch_force(g, kp, true, s, lc);
        if (rc) return rc;
        rc = launch_advect_velocity(g, kp, params.adv_vel_mode, true, s, lc);
        if (rc) return rc;
        swap_velocity();
        rc = launch_project(g, kp, params.sor_iters, sor_eff, s, lc, &p_last);
        if (rc) return rc;
        rc = launch_advect_scalar(g, kp, params.adv_sca_mode, true, &src, s, lc);
        if (rc) return rc;
        swap_scalars();
        return ZQS_OK;
    }
};
