/*
 * zqs_capi.h -- C ABI of the GB300 smoke-step library (libzqs_gb300.so).
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes.  All
 * array arguments use the reference's unpadded x-fastest layouts:
 *   cell fields (occupancy, temperature, density, pressure):  W*H*D
 *   u faces  (W+1)*H*D,   v faces  W*(H+1)*D,   w faces  W*H*(D+1)
 * exactly as ZQ_SmokeGrid3D allocates them (ZQ_SmokeSimulation3D/ZQ_SmokeGrid3D.cpp:5-18).
 * On the device the library keeps its own padded layout (see zqs_grid_layout).
 *
 * Every entry point returns ZQS_OK (0) or a positive zqs_status; the message of
 * the last failure on the calling thread is available from zqs_last_error().
 * A zqs_grid handle is not thread-safe: use one handle per host thread.
 * Stream arguments are cudaStream_t passed as void*; NULL selects the handle's
 * own non-blocking stream.
 *
 * The legacy entry points of the reference (Advect_Velocity, AddForce3D, ...)
 * are declared in zqs_legacy.h and are thin shims over this API.
 */
#ifndef ZQS_CAPI_H
#define ZQS_CAPI_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define ZQS_API __attribute__((visibility("default")))
#else
#define ZQS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define ZQS_VERSION 1

typedef enum zqs_status {
    ZQS_OK = 0,
    ZQS_EINVAL = 1,        /* bad argument: null pointer, size, enum value   */
    ZQS_ENOMEM = 2,        /* device or pinned-host allocation failed         */
    ZQS_EUNSUPPORTED = 3,  /* mode not implemented (returned, never silent)    */
    ZQS_ETIMEOUT = 4,      /* a bounded device-side wait gave up              */
    ZQS_ECUDA = 5,         /* CUDA runtime error (message has the CUDA text)  */
    ZQS_ENOTREADY = 6      /* handle not configured (no params / occupancy)   */
} zqs_status;

/* Projection boundary handling (ZQ_SmokeSimulationUtils3D.cpp:2349-2440):
 * OPEN   = cells outside the domain are Dirichlet p = 0 (TOTAL_OPEN_POISSON_SOR)
 * CLOSED = outside is Neumann and the mean divergence over free cells is
 *          removed first (TOTAL_CLOSED_POISSON_SOR).                          */
/* OPEN / CLOSED: the fine-grid red-black SOR (TOTAL_{OPEN,CLOSED}_POISSON_SOR).
 * COARSE_OPEN: the coarse-grid projection of COARSE_{OPEN,CLOSED}_POISSON_SOR
 * (the reference runs the open coarse solver for both, Utils3D:3732-3746):
 * face-ratio SOR on the grid coarsened by sub_size, the correction mapped back,
 * then an exact projection inside every sub_size^3 block (Utils3D:3688-3794). */
typedef enum zqs_solver { ZQS_SOLVER_OPEN = 0, ZQS_SOLVER_CLOSED = 1, ZQS_SOLVER_COARSE_OPEN = 2 } zqs_solver;

/* Numeric values are those of ZQ_CUDA_Advection3D.h:7-21 (the CUDA header,
 * not the ZQ_SmokeSimulationPara3D enum). */
typedef enum zqs_adv_vel {
    ZQS_ADV_VEL_INREG_OUTREG = 0,
    ZQS_ADV_VEL_INREG_OUTREG_BFECC = 1,
    ZQS_ADV_VEL_INMAC_OUTMAC = 2,
    ZQS_ADV_VEL_INMAC_OUTMAC_BFECC = 3,
    ZQS_ADV_VEL_INREG_OUTMAC = 4,
    ZQS_ADV_VEL_INREG_OUTMAC_BFECC = 5
} zqs_adv_vel;

typedef enum zqs_adv_sca {
    ZQS_ADV_SCA_MAC = 0,
    ZQS_ADV_SCA_MAC_BFECC = 1,
    ZQS_ADV_SCA_REG = 2,
    ZQS_ADV_SCA_REG_BFECC = 3
} zqs_adv_sca;

typedef enum zqs_source_shape {
    ZQS_SOURCE_BOX = 0,     /* |i+.5-cx| <= hx && ... (ZQ_SmokeSimulationUtils3D.cpp:3869) */
    ZQS_SOURCE_SPHERE = 1   /* (i+.5-cx)^2 + (j+.5-cy)^2 + (k+.5-cz)^2 <= hx^2            */
} zqs_source_shape;

#define ZQS_MAX_SOURCES 16

/* A smoke source, in CELL units: cell (i,j,k) spans [i,i+1)x[j,j+1)x[k,k+1).
 * The reference stores unit-cube coordinates and multiplies by W/H/D in float
 * before use (ZQ_SmokeSimulationUtils3D.cpp:3853-3858); callers do that. */
typedef struct zqs_source {
    int32_t shape;
    float cx, cy, cz;
    float hx, hy, hz;       /* box half extents; sphere radius in hx */
    float density;
    float temperature;
} zqs_source;

/* Run parameters (a C mirror of the fields of ZQ_SmokeSimulationPara3D that
 * the per-step path reads, ZQ_SmokeSimulationUtils3D.h:50-125). */
typedef struct zqs_params {
    float voxel_size;       /* h  (reference: 1/width, Utils3D:323)              */
    float step_time;        /* dt (stepTime)                                     */
    int32_t substeps;       /* backtrace substeps ("steps", reference default 20) */
    float confine;          /* vorticity confinement eps (confineCoeff)          */
    float buoyancy;         /* beta: f_y += beta*(T - Tamb)                      */
    float gravity;          /* alpha: f_y -= alpha*rho  (0 reproduces reference)  */
    float tamb;             /* ambient temperature                               */
    float vel_atten;        /* per-step factors, e.g. exp(-dt*coeff) (Utils3D:2098) */
    float temp_atten;
    float dens_atten;
    int32_t solver;         /* zqs_solver                                        */
    int32_t sor_iters;      /* fixed red-black iteration count K (maxIter)       */
    float omega;            /* over-relaxation; 1 reproduces the reference       */
    int32_t adv_vel_mode;   /* zqs_adv_vel                                       */
    int32_t adv_sca_mode;   /* zqs_adv_sca                                       */
    int32_t backtrace_full; /* 0: reference rule (sample at the last point that
                               passed the domain/occupancy test BEFORE the final
                               move); 1: also test and use the final point       */
    int32_t n_sources;
    zqs_source sources[ZQS_MAX_SOURCES];
    int32_t sub_size;       /* COARSE_OPEN: block edge (subSize); divides W, H, D */
} zqs_params;

/* Fields addressable by upload/download. */
typedef enum zqs_field {
    ZQS_FIELD_U = 0,
    ZQS_FIELD_V = 1,
    ZQS_FIELD_W = 2,
    ZQS_FIELD_TEMPERATURE = 3,
    ZQS_FIELD_DENSITY = 4,
    ZQS_FIELD_PRESSURE = 5,    /* last projection's pressure (download only)  */
    ZQS_FIELD_OCCUPANCY = 6,   /* 1 byte per cell, nonzero = occupied         */
    ZQS_FIELD_DIVERGENCE = 7   /* last projection's right-hand side (download) */
} zqs_field;

/* Diagnostics of the last projection; all reductions in FP64. */
typedef struct zqs_stats {
    double max_abs_div;        /* max |div u| over free cells after projection */
    double residual_l2;        /* || div - L p ||_2 of the final pressure       */
    double div_mean_removed;   /* closed solver: mean divergence removed        */
    int64_t free_cells;
} zqs_stats;

/* Device layout of one grid: every field of a handle shares it. */
typedef struct zqs_grid_layout {
    int32_t W, H, D;
    int32_t pitch_x;           /* floats per row  (>= W+1, multiple of 4)      */
    int32_t rows;              /* rows per plane  (= H+1)                      */
    int32_t planes;            /* data planes     (= D+1)                      */
    int64_t plane_elems;       /* pitch_x * rows                               */
    int64_t field_elems;       /* elements allocated per field incl. guards    */
} zqs_grid_layout;

typedef struct zqs_grid zqs_grid;

ZQS_API int zqs_version(void);
ZQS_API const char* zqs_last_error(void);

/* Reference defaults of ZQ_SmokeSimulationPara3D (Utils3D:18-72) for a grid of
 * width W: h=1/W, dt=0.01, substeps=20, buoyancy 1, confine 0, Tamb 10, all
 * attenuation factors 1, open solver, K=100, omega 1, MAC advection modes, one
 * box source.  */
ZQS_API void zqs_params_default(zqs_params* p, int W, int H, int D);

ZQS_API int zqs_grid_create(zqs_grid** out, int W, int H, int D);
ZQS_API int zqs_grid_destroy(zqs_grid* g);
ZQS_API int zqs_grid_get_layout(const zqs_grid* g, zqs_grid_layout* out);
ZQS_API int zqs_grid_set_params(zqs_grid* g, const zqs_params* p);
ZQS_API int zqs_grid_get_params(const zqs_grid* g, zqs_params* p);

/* Copy a field in or out (reference layout).  *_on_device != 0 means the
 * pointer is device memory.  Asynchronous on the stream; host buffers must
 * stay valid until the stream is synchronised (pinned buffers overlap). */
ZQS_API int zqs_grid_upload(zqs_grid* g, int field, const void* src, int src_on_device, void* stream);
ZQS_API int zqs_grid_download(zqs_grid* g, int field, void* dst, int dst_on_device, void* stream);

/* One full timestep = F, T, A, P, S, R in the order of
 * ZQ_SmokeSimulation3D::UpdateOneFrame (ZQ_SmokeSimulation3D.cpp:156-243). */
ZQS_API int zqs_grid_step(zqs_grid* g, int nsteps, void* stream);

/* Enable/disable CUDA-graph replay of zqs_grid_step (default on). */
ZQS_API int zqs_grid_use_graph(zqs_grid* g, int enable);

/* Single stages, for drop-in use and per-stage parity. */
ZQS_API int zqs_stage_add_force(zqs_grid* g, void* stream);
ZQS_API int zqs_stage_attenuate(zqs_grid* g, void* stream);
ZQS_API int zqs_stage_advect_velocity(zqs_grid* g, int mode, int is_open, void* stream);
ZQS_API int zqs_stage_project(zqs_grid* g, void* stream);
ZQS_API int zqs_stage_advect_scalar(zqs_grid* g, int mode, void* stream);
ZQS_API int zqs_stage_reinject(zqs_grid* g, void* stream);

/* Cell-centred velocity (u,v,w,0) per cell, W*H*D float4 (MAC_to_Regular4). */
ZQS_API int zqs_grid_mac_to_regular4(zqs_grid* g, float* vel4, int dst_on_device, void* stream);

/* FP64 diagnostics of the current velocity/pressure; synchronises the stream. */
ZQS_API int zqs_grid_stats(zqs_grid* g, zqs_stats* out, void* stream);

/* SOR kernel selection: temporal_depth = red-black iterations fused per HBM
 * pass (1..4), or 0 (the default): the variant and z chunk an autotuner
 * measured fastest for this grid's shape on this device.  The tuner times
 * every fused variant that fits at a few z chunks (about 25 x 7 short runs of
 * one pass) on the first step or projection that is not issued inside a
 * stream capture, and keeps the choice per (device, shape) in memory and in
 * the file $ZQS_TUNE_CACHE (default $XDG_CACHE_HOME/zqs_gb300/sor_tune.txt or
 * ~/.cache/zqs_gb300/sor_tune.txt; ZQS_TUNE_CACHE="" keeps no file);
 * ZQS_AUTOTUNE=0 uses the fixed default variant instead.  All variants give
 * bit-identical results.  split_colours != 0 runs the plain
 * one-colour-per-launch kernel (the self-check path). */
ZQS_API int zqs_grid_set_sor_config(zqs_grid* g, int temporal_depth, int split_colours);

/* The fused SOR variant (index for zqs_sor_variant_info; -1 for the split
 * kernel), z chunk (0: automatic) and, when it was tuned, the measured time
 * per iteration in microseconds that the next projection uses; runs the tuner
 * first when it is due (synchronises the stream, not inside a capture). */
ZQS_API int zqs_grid_get_sor_choice(zqs_grid* g, int* variant, int* zchunk, float* us_per_iter, void* stream);

/* Fused SOR kernel variants (for tuning): iterations fused per HBM pass, xy
 * tile, cell pairs per thread, threads and shared memory per CTA, CTAs that fit
 * on one SM of the current device (0: does not fit), whether the update
 * weights are held in registers, registers per thread, x-adjacent cells per
 * thread (2: the pair forms, 4: the quad form), and how the CTA's threads
 * synchronise (0: a block barrier every two ring steps, 1: per-step mbarrier
 * waits that let warps run a step apart). */
typedef struct zqs_sor_variant {
    int32_t depth, tile_x, tile_y, pairs_per_thread, threads, ctas_per_sm;
    int64_t smem_bytes;
    int32_t weights_in_registers, registers;
    int32_t x_cells_per_thread; /* 2: one red-black pair per row, 4: two x-adjacent pairs */
    int32_t split_barrier;      /* 1: k_sor_reg_split (per-step mbarriers) */
} zqs_sor_variant;
ZQS_API int zqs_sor_variant_count(void);
ZQS_API int zqs_sor_variant_info(int index, zqs_sor_variant* out);
/* Select a fused variant (-1: default for the configured depth) and the z
 * planes each CTA streams (0: chosen from the grid and the device). */
ZQS_API int zqs_grid_set_sor_variant(zqs_grid* g, int index, int zchunk);

/* Wait for all work queued on the stream (NULL: the handle's own stream).
 * Returns ZQS_ETIMEOUT when a bounded device-side wait gave up since the last
 * check: a tensor-core wait of the coarse solver (below), or a per-step
 * barrier wait of the split-barrier SOR variants (a device-wide count). */
ZQS_API int zqs_grid_synchronize(zqs_grid* g, void* stream);

/* Kernel launches issued by the last zqs_grid_step call (for accounting). */
ZQS_API int64_t zqs_grid_launch_count(const zqs_grid* g);

/* ---- batched mixed-size instances -------------------------------------------
 * A batch advances many independent grids together: each stage of the step is
 * ONE persistent launch whose tile work list spans every member grid (sizes may
 * differ), and the whole batched step is replayed as one CUDA graph.  No
 * counterpart in the reference, which runs one grid per solver object
 * (ZQ_SmokeSimulation3D.cpp:156, UpdateOneFrame steps a single fineGrid).
 *
 * The batch refers to the grids; it does not own them and they must outlive it.
 * Every member must be ready (parameters and occupancy set), use the MAC
 * velocity advection (ZQS_ADV_VEL_INMAC_OUTMAC) and MAC scalar advection
 * (ZQS_ADV_SCA_MAC), and share sor_iters (ZQS_EUNSUPPORTED otherwise); other
 * parameters (dt, forces, solver, sources, sizes) may differ per grid.  Each
 * member ends in exactly the state zqs_grid_step would leave it in, bit for
 * bit, and can be read back with zqs_grid_download.  Parameter, occupancy or
 * SOR changes on a member, and steps taken on it alone, are picked up by the
 * next zqs_batch_step. */
typedef struct zqs_batch zqs_batch;

ZQS_API int zqs_batch_create(zqs_batch** out, zqs_grid* const* grids, int n);
ZQS_API int zqs_batch_destroy(zqs_batch* b);

/* Advance every member nsteps steps on the stream (NULL: the batch's own). */
ZQS_API int zqs_batch_step(zqs_batch* b, int nsteps, void* stream);
ZQS_API int zqs_batch_use_graph(zqs_batch* b, int enable);

/* Fused SOR variant of the batch (-1: default); it must be a register-column
 * variant (ZQS_EUNSUPPORTED otherwise).  zchunk 0 lets the batch pick each
 * member's z chunk for load balance; >0 forces it (clamped to each depth). */
ZQS_API int zqs_batch_set_sor_variant(zqs_batch* b, int index, int zchunk);

/* Kernel launches of one batched step (for accounting). */
ZQS_API int64_t zqs_batch_launch_count(const zqs_batch* b);
/* The batch's fused SOR variant: the one set by zqs_batch_set_sor_variant, or
 * (index -1, the default) the batchable variant that measured fastest per
 * iteration on this batch's own tile lists when its tables were first built
 * (ZQS_AUTOTUNE=0: the fixed default); us_per_iter is the measured time
 * (0 when nothing was measured). */
ZQS_API int zqs_batch_get_sor_choice(const zqs_batch* b, int* variant, float* us_per_iter);
ZQS_API int zqs_batch_synchronize(zqs_batch* b, void* stream);

/* Coarse solver, obstacle-free blocks (the dense block product of
 * SubProjection3DCuda): 1 (default) = tcgen05 tensor cores in TF32 with the
 * 3xTF32 split (relative error ~1e-6 against FP32), 0 = FP32 SIMT with
 * fused multiply-adds in face order (bit-identical to the oracle).  A
 * tensor-core wait that times out is reported by zqs_grid_synchronize
 * (ZQS_ETIMEOUT). */
ZQS_API int zqs_grid_set_coarse_gemm(zqs_grid* g, int mode);

/* ---- failure injection (test hooks) -----------------------------------------
 * Host-side only: neither hook faults, traps or hangs the GPU.
 * zqs_debug_inject_tc_stall(1): the coarse solver's tensor-core block products
 * launched from now on issue no operand copies, so their bounded mbarrier
 * waits give up after about 4096 polls with nothing in flight; the kernel
 * frees its tensor memory, skips the blocks and sets the error flag that
 * zqs_grid_synchronize reports as ZQS_ETIMEOUT.  0 restores normal launches.
 * (A CUDA graph keeps the setting it was captured with.)
 * zqs_debug_fail_alloc(n): the n-th device allocation the library makes from
 * now on (0 = the next one) fails as if the device were out of memory, so the
 * call that makes it returns ZQS_ENOMEM and releases what it had taken; -1
 * disables. */
ZQS_API int zqs_debug_inject_tc_stall(int enable);
ZQS_API int zqs_debug_fail_alloc(int nth);

/* ---- moving voxel objects ---------------------------------------------------
 * ZQ_ApplyMovingObject3D (ZQ_SmokeSimulationUtils3D.cpp:1933-2046): the grid's
 * occupancy becomes the objects' voxels (every other cell free; all six
 * domain walls occupied when closed_walls is 1, all but the y = H-1 layer
 * when it is 2, the open-top walls of wallsExceptTop), and for each object in
 * order every in-domain voxel's six faces take the object's velocity, vel
 * (cells per step, as in the reference's object files) times h/dt rounded
 * toward zero to an integer as the reference's int arithmetic does.  mask is
 * host memory, size[0]*size[1]*size[2] bytes with x fastest; a voxel lands
 * at pos - center + (x, y, z). */
typedef struct zqs_object {
    const uint8_t* mask;
    int32_t size[3], center[3], pos[3], vel[3];
} zqs_object;
ZQS_API int zqs_grid_stamp_objects(zqs_grid* g, const zqs_object* objects, int n, int closed_walls, void* stream);

/* ---- headless ray march of the density ---------------------------------------
 * The viewer's volume shader (SampleSmokeGUI/raycastingshader.h:10-70, its
 * uniforms set in ZQ_SmokeGUI.cpp:711-752) as a CUDA kernel writing an RGBA
 * float image to device memory; no graphics API.  Pixel (px, py), py counted
 * from the bottom row as gl_FragCoord is, casts a ray through
 * (px + 0.5 - (width-1)/2, py + 0.5 - (height-1)/2, -focal) turned by
 * inv_view (row-major); a ray that meets the box takes `steps` samples from
 * its entry point and writes (v, v, v, exp(-v)), v = density_scale times the
 * sum of steplen * density, steplen = (tfar - tnear) / steps / box_size[0];
 * other pixels get (0, 0, 0, 1).  The density is sampled as the viewer's
 * GL_LINEAR / GL_CLAMP texture: coordinates clamped to [0, 1] over the box,
 * texel centres at (i + 0.5) / n, zero outside the volume, exact trilinear
 * weights (not the hardware filter's 8-bit ones).  rgba holds
 * width * height * 4 floats in device memory, row py at py * width * 4. */
typedef struct zqs_camera {
    int32_t width, height;        /* image size in pixels */
    float focal;                  /* distance of the image plane in pixels */
    float inv_view[9];            /* eye-space -> world directions, row-major */
    float eye[3];                 /* ray origin */
    float box_min[3], box_max[3], box_size[3];
    int32_t steps;                /* samples per ray, 0..65536 */
    float density_scale;
} zqs_camera;
/* The viewer's start-up view of a W x H x D volume: fovy 40 (focal =
 * height / 2 / atan(fovy / 360 * pi), the viewer's formula), eye (0, 0, 2)
 * looking at the origin with y up, a box of height 1 with the volume's aspect
 * centred at the origin, 300 steps, density scale 1. */
ZQS_API void zqs_camera_default(zqs_camera* cam, int image_width, int image_height, int W, int H, int D);
/* density: device memory, W*H*D floats, x fastest. */
ZQS_API int zqs_render_density(const float* density, int W, int H, int D, const zqs_camera* cam, float* rgba,
                               void* stream);
/* The grid's current density. */
ZQS_API int zqs_grid_render(zqs_grid* g, const zqs_camera* cam, float* rgba, void* stream);

/* ---- external force and reverse mode ----------------------------------------
 * No counterpart in the reference.  An external per-cell force F is added to
 * the cell force of every step after the buoyancy terms (force stage, before
 * the face averaging).  F holds 3*W*H*D floats, component-major (x, y, z),
 * each component dense with x fastest; NULL removes it. */
ZQS_API int zqs_grid_set_force(zqs_grid* g, const float* F, int src_on_device, void* stream);

/* A reverse-mode session over nsteps steps of a grid with a control force F,
 * for losses on the final density.  The forward pass keeps the state every
 * checkpoint_every steps; the backward pass recomputes each segment from its
 * checkpoint and runs the adjoint kernels of every stage in reverse order
 * (transposed-trilinear scatters with FP32 atomics for the advections, the
 * transposed force stencil, the red-black SOR transposed half-sweep by
 * half-sweep).  Requires MAC velocity and scalar advection and at most 32
 * backtrace substeps (ZQS_EUNSUPPORTED otherwise).  Results of the backward
 * pass vary in the last bits from run to run (atomic accumulation order). */
typedef struct zqs_adjoint zqs_adjoint;

typedef struct zqs_adjoint_info {
    int64_t device_bytes;       /* memory the session holds (checkpoints, segment, adjoint fields, work grid) */
    int64_t launches_forward;   /* kernel launches of the last forward pass */
    int64_t launches_backward;  /* kernel launches of the last backward pass */
    int32_t nsteps, checkpoint_every, checkpoints;
    int32_t pad;
} zqs_adjoint_info;

ZQS_API int zqs_adjoint_create(zqs_adjoint** out, zqs_grid* g, int nsteps, int checkpoint_every);
ZQS_API int zqs_adjoint_destroy(zqs_adjoint* a);

/* Sets F (as zqs_grid_set_force) and advances the grid nsteps steps from its
 * current state, keeping the checkpoints; the grid ends in the final state. */
ZQS_API int zqs_adjoint_forward(zqs_adjoint* a, const float* F, int src_on_device, void* stream);

/* g_density: dL/d(final density), W*H*D floats dense (e.g. 2*(rho - target)
 * for L = sum (rho - target)^2).  grad_F receives dL/dF (3*W*H*D floats, the
 * layout of F).  The grid is not modified. */
ZQS_API int zqs_adjoint_backward(zqs_adjoint* a, const float* g_density, float* grad_F, int on_device,
                                 void* stream);

/* After zqs_adjoint_backward: dL/d(initial state) for ZQS_FIELD_U/V/W,
 * ZQS_FIELD_TEMPERATURE or ZQS_FIELD_DENSITY, in the field's dense layout. */
ZQS_API int zqs_adjoint_download(zqs_adjoint* a, int field, void* dst, int dst_on_device, void* stream);
ZQS_API int zqs_adjoint_get_info(const zqs_adjoint* a, zqs_adjoint_info* out);

#ifdef __cplusplus
}
#endif

#endif /* ZQS_CAPI_H */
