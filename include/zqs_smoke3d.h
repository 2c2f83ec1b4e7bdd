/* C++ host API of libzqs_gb300.so with the reference's class and function names:
 * ZQ_SmokeGrid3D (ZQ_SmokeGrid3D.h:7-68), ZQ_SmokeSimulationPara3D and the
 * step's free functions (ZQ_SmokeSimulationUtils3D.h:41-169) and
 * ZQ_SmokeSimulation3D (ZQ_SmokeSimulation3D.h:13-48), for host code written
 * against the reference (main.cpp:13-18 style: Init(config), Run(folder)).
 *
 * Storage: every grid keeps host arrays in the reference layouts (x fastest;
 * u (W+1)HD, v W(H+1)D, w WH(D+1), cells WHD) behind the same `T*& Get*Ptr()`
 * accessors, plus a device grid (zqs_grid) created on first GPU use.  The free
 * functions are synchronous and move data each call, like the reference;
 * ZQ_SmokeSimulation3D keeps the state on the GPU between frames and copies it
 * back only when the host arrays are asked for (GetFineGrid, exports).
 *
 * Differences, kept as parameters or documented: the projection is the
 * fine-grid red-black SOR (TOTAL_*_POISSON_SOR) or the coarse-grid projection
 * (COARSE_*_POISSON_SOR); the octree, flux and PCG solvers of the reference
 * map to the fine-grid SOR of the same open/closed kind, with a notice; moving objects,
 * guiding control and the wavelet / compressed export formats are not
 * available (Init or the export returns false). */
#ifndef ZQS_SMOKE3D_H
#define ZQS_SMOKE3D_H

#include <stdint.h>

#include <vector>

#include "zqs_capi.h"

#if defined(__GNUC__)
#define ZQS_CXX_API __attribute__((visibility("default")))
#else
#define ZQS_CXX_API
#endif

enum GlobalSolverType3D {
    CLOSED_POISSON,
    CLOSED_FLUX,
    OPEN_POISSON,
    OPEN_FLUX,
    COARSE_OPEN_POISSON_SOR,
    COARSE_CLOSED_POISSON_SOR,
    COARSE_OPEN_FLUX_SOR,
    COARSE_CLOSED_FLUX_SOR,
    TOTAL_OPEN_POISSON_SOR,
    TOTAL_CLOSED_POISSON_SOR,
    TOTAL_OPEN_FLUX_SOR,
    TOTAL_CLOSED_FLUX_SOR,
    CLOSED_OCTREE_POISSON,
    CLOSED_OCTREE_FLUX,
    OPEN_OCTREE_POISSON,
    OPEN_OCTREE_FLUX,
    OPEN_OCTREE_POISSON_SOR,
    CLOSED_OCTREE_POISSON_SOR
};

/* A box source in unit coordinates (ZQ_SmokeSimulationUtils3D.h:41-48);
 * sphere = true makes it a sphere of radius half_xlen (new). */
class ZQS_CXX_API ZQ_SmokeSource3D {
public:
    float cx = 0.5f, cy = 0.1f, cz = 0.5f;
    float half_xlen = 0.1f, half_ylen = 0.05f, half_zlen = 0.1f;
    float reinjectDensity = 1.0f;
    float reinjectTemperature = 200.0f;
    bool sphere = false;
};

class ZQS_CXX_API ZQ_SmokeSimulationPara3D {
public:
    enum InternalObject { INT_OBJ_NULL, INT_OBJ_SPHERE, INT_OBJ_BOX, INT_OBJ_OVAL, INT_OBJ_SPECIAL1 };
    enum AdvectVelocityType {
        ADV_VEL_INMAC_OUTMAC,
        ADV_VEL_INMAC_OUTMAC_BFECC,
        ADV_VEL_INREG_OUTREG,
        ADV_VEL_INREG_OUTREG_BFECC,
        ADV_VEL_INREG_OUTMAC,
        ADV_VEL_INREG_OUTMAC_BFECC
    };
    enum AdvectScalarType { ADV_SCA_MAC, ADV_SCA_MAC_BFECC, ADV_SCA_REG, ADV_SCA_REG_BFECC };
    enum ExportType { EXPORT_DI3, EXPORT_ZQWV, EXPORT_ZQCI };
    enum AddForceType { ADD_FORCE_ENTIRE, ADD_FORCE_SLICE };

    ZQ_SmokeSimulationPara3D();

    /* The reference's fields and defaults (ZQ_SmokeSimulationUtils3D.cpp:18-72). */
    int width, height, depth;
    int coarseWidth, coarseHeight, coarseDepth;
    int subSize;
    float gravityCoeff;     /* density weight alpha: f_y -= alpha * rho (unused by the reference) */
    float buoyancyCoeff;    /* f_y += buoyancy * (T - Tamb) */
    float confineCoeff;
    std::vector<ZQ_SmokeSource3D> sources;
    float velAttenCoeff;    /* factors exp(-stepTime * coeff) */
    float Tamb;
    float voxelSize;
    float stepTime;
    float tempAttenCoeff;
    float densityAttenCoeff;
    int steps;              /* backtrace substeps */
    int frameCount;
    int maxIter;            /* SOR iterations */
    int innerIter;
    GlobalSolverType3D globalGridSolver;
    int subGridSolver;
    int octree_thresh1, octree_thresh2, octree_thresh3;
    bool useMovingObject;
    char movingObjectFile[200];
    bool useGuidingControl;
    float guidingCoeff;
    bool guidingNaiveBlend;
    char guidingFold[200];
    bool exportGuide;
    bool exportOccupy;
    bool randDensity;
    float maxDensity;
    float maxTemperature;
    InternalObject intobj;
    AdvectVelocityType advVelType;
    AdvectScalarType advScaType;
    ExportType exportType;
    float export_quality;
    AddForceType addforce_type;

    /* Added (config keys in parentheses): over-relaxation (omega), attenuation
     * factors used as given instead of exp(-dt*coeff) when >= 0
     * (velAttenFactor, tempAttenFactor, densityAttenFactor), the final-point
     * backtrace (backtraceFull), closed walls except an open top with the open
     * solver (wallsExceptTop), inclusive occupied cell boxes (obstacleBox
     * x0 x1 y0 y1 z0 z1), seeded velocity noise on live faces
     * (noiseAmp, seed). */
    float omega;
    float velAttenFactor, tempAttenFactor, densityAttenFactor;
    bool backtraceFull;
    bool wallsExceptTop;
    std::vector<int> obstacleBoxes;  /* 6 ints per box */
    float noiseAmp;
    uint64_t seed;

    /* Reads the reference's whitespace "key value" format (case-insensitive
     * keys, unknown keys ignored) plus the keys above and "sphereSource
     * cx cy cz r density temperature" (unit coordinates). */
    bool LoadFromFile(const char* file, bool display = true);

    /* The run parameters of the C ABI that this configuration gives. */
    bool ToParams(zqs_params* out) const;
};

class ZQS_CXX_API ZQ_SmokeGrid3D {
public:
    ZQ_SmokeGrid3D(const unsigned int width, const unsigned int height, const unsigned int depth);
    ~ZQ_SmokeGrid3D();
    ZQ_SmokeGrid3D(const ZQ_SmokeGrid3D&) = delete;
    ZQ_SmokeGrid3D& operator=(const ZQ_SmokeGrid3D&) = delete;

    int GetWidth() const { return width; }
    int GetHeight() const { return height; }
    int GetDepth() const { return depth; }

    bool*& GetOccupyPtr();
    float*& GetPressurePtr();
    float*& GetTemperaturePtr();
    float*& GetDensityPtr();
    float*& GetVelocityUptr();
    float*& GetVelocityVptr();
    float*& GetVelocityWptr();
    float*& GetFaceUnOccupyRatioUPtr() { return ratioU; }
    float*& GetFaceUnOccupyRatioVPtr() { return ratioV; }
    float*& GetFaceUnOccupyRatioWPtr() { return ratioW; }
    float*& GetVolumeUnOccupyRatioPtr() { return ratioVol; }

    void BuildFaceUnOccupyRatio();
    void ClearFaceUnOccupyRatio();
    void BuildVolumeUnOccupyRatio();
    void ClearVolumeUnOccupyRatio();

    ZQ_SmokeGrid3D* Clone() const;

    /* .di3 only: a 16-byte type tag "float", int32 width, height, depth,
     * channels (1), one flag byte (0), then the floats.  .zqwv / .zqci return
     * false. */
    bool ExportDensity(const char* file, float quality = 0.9999f) const;
    bool ExportOccupy(const char* file) const;   /* no-op returning true, as the reference */
    bool ExportVelocity(const char* file) const; /* no-op returning true, as the reference */
    /* raw FP32 u, v, w, density, temperature (ZQ_SmokeGrid3D.cpp:83-121) */
    bool ExportGuide(const char* file) const;
    /* Added: reads a file written by ExportGuide back into the grid (resume). */
    bool ImportGuide(const char* file);

    /* Added: the device grid (created on first use); null on failure. */
    zqs_grid* DeviceGrid();
    /* Added: host arrays -> device (all fields) and device -> host. */
    bool Upload();
    bool Download();
    /* Added: the device state is newer than the host arrays (kept by
     * ZQ_SmokeSimulation3D; the accessors above download first). */
    void MarkHostStale() { host_stale = true; }

private:
    void SyncHost() const;
    int width, height, depth;
    std::vector<uint8_t> occ_store;
    std::vector<float> pressure_store, temperature_store, density_store, u_store, v_store, w_store;
    std::vector<float> ratioU_store, ratioV_store, ratioW_store, ratioVol_store;
    bool* occ;
    float *pressure, *temperature, *density, *u, *v, *w;
    float *ratioU, *ratioV, *ratioW, *ratioVol;
    zqs_grid* dev;
    mutable bool host_stale;
};

/* The step's free functions (ZQ_SmokeSimulationUtils3D.h:127-169 subset):
 * host arrays in, GPU stage, host arrays out; false on failure with the
 * message in zqs_last_error(). */
ZQS_CXX_API void MACtoRegular4(int width, int height, int depth, const float* mac_u, const float* mac_v,
                               const float* mac_w, float* vel4);
ZQS_CXX_API void Regular4toMAC(int width, int height, int depth, const float* vel4, float* mac_u, float* mac_v,
                               float* mac_w);
ZQS_CXX_API bool ZQ_InitFineGrid3D(ZQ_SmokeGrid3D* fineGrid, const ZQ_SmokeSimulationPara3D& para);
ZQS_CXX_API bool ZQ_AddForce3D(ZQ_SmokeGrid3D* fineGrid, const ZQ_SmokeSimulationPara3D& para);
ZQS_CXX_API bool ZQ_Attenuation3D(ZQ_SmokeGrid3D* fineGrid, const ZQ_SmokeSimulationPara3D& para);
ZQS_CXX_API bool ZQ_AdvectVelocity3D(ZQ_SmokeGrid3D* fineGrid, const ZQ_SmokeSimulationPara3D& para);
ZQS_CXX_API bool ZQ_SolveOpenPressure3DSOR(ZQ_SmokeGrid3D* fineGrid, const ZQ_SmokeSimulationPara3D& para);
ZQS_CXX_API bool ZQ_SolveClosedPressure3DSOR(ZQ_SmokeGrid3D* fineGrid, const ZQ_SmokeSimulationPara3D& para);
/* The projection the configuration selects (ZQ_TotalProjection3D, Utils3D:3688-3794):
 * the coarse-grid solver for COARSE_{OPEN,CLOSED}_POISSON_SOR, else the
 * fine-grid SOR of the same open/closed kind. */
ZQS_CXX_API bool ZQ_TotalProjection3D(ZQ_SmokeGrid3D* fineGrid, const ZQ_SmokeSimulationPara3D& para);
ZQS_CXX_API bool ZQ_AdvectScalar3D(ZQ_SmokeGrid3D* fineGrid, const ZQ_SmokeSimulationPara3D& para);
ZQS_CXX_API bool ZQ_ReinjectTemperatureDensity3D(ZQ_SmokeGrid3D* fineGrid, const ZQ_SmokeSimulationPara3D& para);
/* One frame through the free functions above (force, attenuation, velocity
 * advection, projection, scalar advection, reinjection). */
ZQS_CXX_API bool ZQ_UpdateOneFrame3D(ZQ_SmokeGrid3D* fineGrid, const ZQ_SmokeSimulationPara3D& para);

/* A moving voxel object (ZQ_SmokeMovingObject3D.h:6-35): a solid mask of
 * sizex*sizey*sizez voxels (x fastest) placed at pos - c, moved by vels[curstep]
 * cells per step. */
class ZQS_CXX_API ZQ_SmokeMovingObject3D {
public:
    class Velocity {
    public:
        int x, y, z;
        Velocity(int u = 0, int v = 0, int w = 0) : x(u), y(v), z(w) {}
    };
    ZQ_SmokeMovingObject3D();
    ~ZQ_SmokeMovingObject3D();
    ZQ_SmokeMovingObject3D(const ZQ_SmokeMovingObject3D&) = delete;  /* owns occupy */
    ZQ_SmokeMovingObject3D& operator=(const ZQ_SmokeMovingObject3D&) = delete;
    int cx, cy, cz;        // rotation centre
    int posx, posy, posz;  // position in the grid
    int sizex, sizey, sizez;
    int curstep;
    std::vector<Velocity> vels;
    bool* occupy;
    void GetCenter(int& cx, int& cy, int& cz) const;
    void GetPos(int& posx, int& posy, int& posz) const;
    void GetSize(int& sizex, int& sizey, int& sizez) const;
    /* vels[curstep], 0 past the end */
    void GetCurVel(int& u, int& v, int& w) const;
    const bool*& GetOccupyPtr() const;
    /* pos += vels[curstep] (when in range), curstep++ */
    void UpdateOneStep();
};
/* The reference's object file (ZQ_SmokeMovingObject3D.cpp:101-123): count, then
 * per object sizes, centre, position, step count, the step velocities and the
 * voxel mask, whitespace-separated integers. */
ZQS_CXX_API bool LoadMovingObjects3D(const char* file, std::vector<ZQ_SmokeMovingObject3D*>& mvobjs);
/* ZQ_ApplyMovingObject3D (Utils3D:1933-2046): the occupancy becomes the objects'
 * voxels (all six walls too for the closed solvers) and the voxels' faces take
 * the objects' velocities; on the GPU, host arrays in and out. */
ZQS_CXX_API bool ZQ_ApplyMovingObject3D(ZQ_SmokeGrid3D* fineGrid, const std::vector<ZQ_SmokeMovingObject3D*>& mvobjs,
                                        const ZQ_SmokeSimulationPara3D& para);

/* Headless counterpart of the viewer's volume display (SampleSmokeGUI:
 * LoadDataToVolumeTex, ZQ_SmokeGUI.cpp:521-680; DrawVolumeData and its
 * sequence mode, :680-752), rendered by zqs_render_density on the GPU.
 *
 * ZQ_LoadVolume3D: a .di3 file (16-byte type tag "float", int32 width,
 * height, depth, channels, one flag byte, the floats; channels averaged into
 * one), or else a raw file of N^3 floats whose first and last axes the viewer
 * swaps (tmp[i N^2 + j N + k] = raw[k N^2 + j N + i]).  .zqci / .zqwv
 * (ZQlib formats) return false. */
ZQS_CXX_API bool ZQ_LoadVolume3D(const char* file, int N, std::vector<float>& data, int& W, int& H, int& D);
/* Ray march a host density (W*H*D floats, x fastest) into host RGBA floats
 * (cam.width * cam.height * 4, bottom row first). */
ZQS_CXX_API bool ZQ_RenderVolume3D(const float* density, int W, int H, int D, const zqs_camera& cam,
                                   std::vector<float>& rgba);
/* Binary PPM of an RGBA render over a black background: rgb clamped to
 * [0, 1], * 255 + 0.5 truncated, top row first. */
ZQS_CXX_API bool ZQ_WriteRenderPPM(const char* file, const std::vector<float>& rgba, int width, int height);
/* The viewer's sequence mode: files fold/<prefix><baseID+n><suffix>, n < num,
 * each shown in the viewer's start-up view (zqs_camera_default) and written
 * to outFold/render<baseID+n>.ppm.  N: edge of raw files (ignored for .di3). */
ZQS_CXX_API bool ZQ_RenderSequence3D(const char* fold, const char* prefix, int baseID, int num, const char* suffix,
                                     int N, int imageWidth, int imageHeight, const char* outFold);

class ZQS_CXX_API ZQ_SmokeSimulation3D {
public:
    ZQ_SmokeSimulation3D();
    ~ZQ_SmokeSimulation3D();
    ZQ_SmokeSimulation3D(const ZQ_SmokeSimulation3D&) = delete;  /* owns the grid and the objects */
    ZQ_SmokeSimulation3D& operator=(const ZQ_SmokeSimulation3D&) = delete;

    bool Init(const char* file);
    /* frameCount frames; frame i's density to <fold>/frame<i>.di3 (plus
     * <fold>/<i>.guidedat when exportGuide is set). */
    bool Run(const char* fold);
    /* One step on the resident device grid (a CUDA graph replay); the guide
     * grid must be null (guiding control is not available). */
    bool UpdateOneFrame(const void* guideGrid = nullptr);

    /* Added accessors. */
    const ZQ_SmokeSimulationPara3D& GetPara() const { return para; }
    ZQ_SmokeGrid3D* GetFineGrid();
    bool GetParams(zqs_params* out) const { return para.ToParams(out); }

private:
    ZQ_SmokeSimulationPara3D para;
    ZQ_SmokeGrid3D* fineGrid;
    std::vector<ZQ_SmokeMovingObject3D*> mvobjs;
    int frame;  // frames run; the objects are re-applied from the second on (ZQ_SmokeSimulation3D.cpp:161-173)
};

#endif /* ZQS_SMOKE3D_H */
