// C++ host API with the reference's class and function names (include/zqs_smoke3d.h),
// built on the handle ABI of capi.cpp.  Restates the host side of the
// reference step: ZQ_SmokeSimulationPara3D (ZQ_SmokeSimulationUtils3D.cpp:18-352),
// ZQ_InitFineGrid3D (:1523-1664), the stage wrappers (:2049-2168, 2349-2440,
// 3796-3904), ZQ_SmokeGrid3D (ZQ_SmokeGrid3D.cpp:5-121) and
// ZQ_SmokeSimulation3D::Init/Run/UpdateOneFrame (ZQ_SmokeSimulation3D.cpp:60-243).
#include <cuda_runtime.h>
#include <strings.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/zqs_smoke3d.h"

namespace {

bool key_is(const char* a, const char* b) { return strcasecmp(a, b) == 0; }

// SplitMix64 uniform draws, the generator of the Python workloads module:
// x_n = splitmix64(seed + n*0x9E3779B97F4A7C15) for n = offset+1, ...;
// u_n = (x_n >> 40) * 2^-24; U(lo, hi) = lo + (hi - lo) * u_n in float.
float uniform_at(uint64_t seed, uint64_t n1, float lo, float hi) {
    uint64_t z = seed + n1 * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    const float u = (float)(z >> 40) * (1.0f / 16777216.0f);
    return lo + (hi - lo) * u;
}

bool is_closed(GlobalSolverType3D s) {
    switch (s) {
        case CLOSED_POISSON:
        case CLOSED_FLUX:
        case COARSE_CLOSED_POISSON_SOR:
        case COARSE_CLOSED_FLUX_SOR:
        case TOTAL_CLOSED_POISSON_SOR:
        case TOTAL_CLOSED_FLUX_SOR:
        case CLOSED_OCTREE_POISSON:
        case CLOSED_OCTREE_FLUX:
        case CLOSED_OCTREE_POISSON_SOR: return true;
        default: return false;
    }
}

bool fail(const char* what) {
    fprintf(stderr, "zqs: %s: %s\n", what, zqs_last_error());
    return false;
}

}  // namespace

// ----------------------------------------------------------------- parameters

ZQ_SmokeSimulationPara3D::ZQ_SmokeSimulationPara3D() {
    width = height = depth = 128;
    subSize = 4;
    coarseWidth = width / subSize;
    coarseHeight = height / subSize;
    coarseDepth = depth / subSize;
    gravityCoeff = 0;
    buoyancyCoeff = 1;
    confineCoeff = 0;
    Tamb = 10;
    voxelSize = (float)(1.0 / width);
    ZQ_SmokeSource3D s;
    s.reinjectTemperature = Tamb * 20;
    sources.push_back(s);
    velAttenCoeff = 0;
    densityAttenCoeff = 0;
    tempAttenCoeff = 0;
    stepTime = 0.01f;
    steps = 20;
    frameCount = 100;
    maxIter = 100;
    innerIter = 30;
    globalGridSolver = COARSE_OPEN_POISSON_SOR;
    subGridSolver = CLOSED_POISSON;
    octree_thresh1 = 2;
    octree_thresh2 = 4;
    octree_thresh3 = 16;
    useMovingObject = false;
    movingObjectFile[0] = 0;
    useGuidingControl = false;
    guidingCoeff = 0;
    guidingNaiveBlend = true;
    exportGuide = false;
    guidingFold[0] = 0;
    exportOccupy = false;
    randDensity = false;
    maxDensity = 0.8f;
    maxTemperature = 20.0f;
    intobj = INT_OBJ_NULL;
    advVelType = ADV_VEL_INREG_OUTREG;
    advScaType = ADV_SCA_REG;
    exportType = EXPORT_DI3;
    export_quality = 0.9999f;
    addforce_type = ADD_FORCE_ENTIRE;
    omega = 1.0f;
    velAttenFactor = tempAttenFactor = densityAttenFactor = -1.0f;
    backtraceFull = false;
    wallsExceptTop = false;
    noiseAmp = 0.0f;
    seed = 0;
}

bool ZQ_SmokeSimulationPara3D::LoadFromFile(const char* file, bool display) {
    FILE* config = fopen(file, "r");
    if (!config) return false;
    sources.clear();
    obstacleBoxes.clear();
    char s[1000];
    while (fgets(s, sizeof(s), config)) {
        char arg1[100] = {0}, arg2[100] = {0};
        if (sscanf(s, "%99s%99s", arg1, arg2) < 1) continue;
        auto on = [&]() { return key_is(arg2, "true"); };
        if (key_is(arg1, "resolution")) sscanf(s, "%*s%d%d%d", &width, &height, &depth);
        else if (key_is(arg1, "subSize")) subSize = atoi(arg2);
        else if (key_is(arg1, "Tamb")) Tamb = (float)atof(arg2);
        else if (key_is(arg1, "velAttenCoeff")) velAttenCoeff = (float)atof(arg2);
        else if (key_is(arg1, "tempAttenCoeff")) tempAttenCoeff = (float)atof(arg2);
        else if (key_is(arg1, "densityAttenCoeff")) densityAttenCoeff = (float)atof(arg2);
        else if (key_is(arg1, "confineCoeff")) confineCoeff = (float)atof(arg2);
        else if (key_is(arg1, "source")) {
            ZQ_SmokeSource3D src;
            sscanf(s, "%*s%f%f%f%f%f%f%f%f", &src.cx, &src.cy, &src.cz, &src.half_xlen, &src.half_ylen,
                   &src.half_zlen, &src.reinjectDensity, &src.reinjectTemperature);
            sources.push_back(src);
        } else if (key_is(arg1, "sphereSource")) {
            ZQ_SmokeSource3D src;
            src.sphere = true;
            sscanf(s, "%*s%f%f%f%f%f%f", &src.cx, &src.cy, &src.cz, &src.half_xlen, &src.reinjectDensity,
                   &src.reinjectTemperature);
            src.half_ylen = src.half_zlen = src.half_xlen;
            sources.push_back(src);
        } else if (key_is(arg1, "steps")) steps = atoi(arg2);
        else if (key_is(arg1, "stepTime")) stepTime = (float)atof(arg2);
        else if (key_is(arg1, "frameCount")) frameCount = atoi(arg2);
        else if (key_is(arg1, "maxIter") || key_is(arg1, "sorIters")) maxIter = atoi(arg2);
        else if (key_is(arg1, "innerIter")) innerIter = atoi(arg2);
        else if (key_is(arg1, "globalGridSolver")) {
            static const struct {
                const char* name;
                GlobalSolverType3D v;
            } names[] = {{"CLOSED_POISSON", CLOSED_POISSON},
                         {"OPEN_POISSON", OPEN_POISSON},
                         {"CLOSED_FLUX", CLOSED_FLUX},
                         {"OPEN_FLUX", OPEN_FLUX},
                         {"CLOSED_OCTREE_FLUX", CLOSED_OCTREE_FLUX},
                         {"OPEN_OCTREE_FLUX", OPEN_OCTREE_FLUX},
                         {"CLOSED_OCTREE_POISSON", CLOSED_OCTREE_POISSON},
                         {"OPEN_OCTREE_POISSON", OPEN_OCTREE_POISSON},
                         {"TOTAL_OPEN_POISSON_SOR", TOTAL_OPEN_POISSON_SOR},
                         {"TOTAL_CLOSED_POISSON_SOR", TOTAL_CLOSED_POISSON_SOR},
                         {"TOTAL_OPEN_FLUX_SOR", TOTAL_OPEN_FLUX_SOR},
                         {"TOTAL_CLOSED_FLUX_SOR", TOTAL_CLOSED_FLUX_SOR},
                         {"COARSE_OPEN_POISSON_SOR", COARSE_OPEN_POISSON_SOR},
                         {"COARSE_CLOSED_POISSON_SOR", COARSE_CLOSED_POISSON_SOR},
                         {"COARSE_OPEN_FLUX_SOR", COARSE_OPEN_FLUX_SOR},
                         {"COARSE_CLOSED_FLUX_SOR", COARSE_CLOSED_FLUX_SOR},
                         {"OPEN_OCTREE_POISSON_SOR", OPEN_OCTREE_POISSON_SOR},
                         {"CLOSED_OCTREE_POISSON_SOR", CLOSED_OCTREE_POISSON_SOR}};
            globalGridSolver = OPEN_FLUX;  // the reference's fallback for unknown names
            for (const auto& n : names)
                if (key_is(arg2, n.name)) globalGridSolver = n.v;
        } else if (key_is(arg1, "octree_thresh1")) octree_thresh1 = atoi(arg2);
        else if (key_is(arg1, "octree_thresh2")) octree_thresh2 = atoi(arg2);
        else if (key_is(arg1, "octree_thresh3")) octree_thresh3 = atoi(arg2);
        else if (key_is(arg1, "useMovingObject")) useMovingObject = on();
        else if (key_is(arg1, "movingObjectFile")) snprintf(movingObjectFile, sizeof(movingObjectFile), "%s", arg2);
        else if (key_is(arg1, "useGuidingControl")) useGuidingControl = on();
        else if (key_is(arg1, "guidingCoeff")) guidingCoeff = (float)atof(arg2);
        else if (key_is(arg1, "guidingNaiveBlend")) guidingNaiveBlend = on();
        else if (key_is(arg1, "guidingFold")) snprintf(guidingFold, sizeof(guidingFold), "%s", arg2);
        else if (key_is(arg1, "exportGuide")) exportGuide = strcmp(arg2, "true") == 0;  // case-sensitive there
        else if (key_is(arg1, "exportOccupy")) exportOccupy = on();
        else if (key_is(arg1, "randDensity")) randDensity = on();
        else if (key_is(arg1, "intobj")) {
            if (key_is(arg2, "sphere")) intobj = INT_OBJ_SPHERE;
            else if (key_is(arg2, "oval")) intobj = INT_OBJ_OVAL;
            else if (key_is(arg2, "box")) intobj = INT_OBJ_BOX;
            else if (key_is(arg2, "special1")) intobj = INT_OBJ_SPECIAL1;
            else intobj = INT_OBJ_NULL;
        } else if (key_is(arg1, "advVelType")) {
            if (key_is(arg2, "inMAC_outMAC")) advVelType = ADV_VEL_INMAC_OUTMAC;
            else if (key_is(arg2, "inMAC_outMAC_BFECC")) advVelType = ADV_VEL_INMAC_OUTMAC_BFECC;
            else if (key_is(arg2, "inReg_outReg")) advVelType = ADV_VEL_INREG_OUTREG;
            else if (key_is(arg2, "inReg_outReg_BFECC")) advVelType = ADV_VEL_INREG_OUTREG_BFECC;
            else if (key_is(arg2, "inReg_outMAC")) advVelType = ADV_VEL_INREG_OUTMAC;
            else if (key_is(arg2, "inReg_outMAC_BFECC")) advVelType = ADV_VEL_INREG_OUTMAC_BFECC;
            else {
                printf("unknown para: %s: %s\n", arg1, arg2);
                fclose(config);
                return false;
            }
        } else if (key_is(arg1, "advScaType")) {
            if (key_is(arg2, "MAC")) advScaType = ADV_SCA_MAC;
            else if (key_is(arg2, "MAC_BFECC")) advScaType = ADV_SCA_MAC_BFECC;
            else if (key_is(arg2, "Reg")) advScaType = ADV_SCA_REG;
            else if (key_is(arg2, "Reg_BFECC")) advScaType = ADV_SCA_REG_BFECC;
            else {
                printf("unknown para: %s: %s\n", arg1, arg2);
                fclose(config);
                return false;
            }
        } else if (key_is(arg1, "exportType")) {
            if (key_is(arg2, "DI3")) exportType = EXPORT_DI3;
            else if (key_is(arg2, "ZQWV")) exportType = EXPORT_ZQWV;
            else if (key_is(arg2, "ZQCI")) exportType = EXPORT_ZQCI;
            else {
                printf("unknown para: %s: %s\n", arg1, arg2);
                fclose(config);
                return false;
            }
        } else if (key_is(arg1, "exportQuality")) export_quality = (float)atof(arg2);
        else if (key_is(arg1, "AddForceType")) {
            if (key_is(arg2, "ENTIRE")) addforce_type = ADD_FORCE_ENTIRE;
            else if (key_is(arg2, "SLICE")) addforce_type = ADD_FORCE_SLICE;
            else {
                printf("unknown para: %s: %s\n", arg1, arg2);
                fclose(config);
                return false;
            }
        } else if (key_is(arg1, "maxDensity")) maxDensity = (float)atof(arg2);
        else if (key_is(arg1, "maxTemperature")) maxTemperature = (float)atof(arg2);
        // keys added by this library
        else if (key_is(arg1, "omega")) omega = (float)atof(arg2);
        else if (key_is(arg1, "buoyancyCoeff") || key_is(arg1, "beta")) buoyancyCoeff = (float)atof(arg2);
        else if (key_is(arg1, "gravityCoeff") || key_is(arg1, "alpha")) gravityCoeff = (float)atof(arg2);
        else if (key_is(arg1, "velAttenFactor")) velAttenFactor = (float)atof(arg2);
        else if (key_is(arg1, "tempAttenFactor")) tempAttenFactor = (float)atof(arg2);
        else if (key_is(arg1, "densityAttenFactor")) densityAttenFactor = (float)atof(arg2);
        else if (key_is(arg1, "backtraceFull")) backtraceFull = on();
        else if (key_is(arg1, "wallsExceptTop")) wallsExceptTop = on();
        else if (key_is(arg1, "noiseAmp")) noiseAmp = (float)atof(arg2);
        else if (key_is(arg1, "seed")) seed = strtoull(arg2, nullptr, 10);
        else if (key_is(arg1, "obstacleBox")) {
            int b[6];
            if (sscanf(s, "%*s%d%d%d%d%d%d", &b[0], &b[1], &b[2], &b[3], &b[4], &b[5]) == 6)
                obstacleBoxes.insert(obstacleBoxes.end(), b, b + 6);
        }
    }
    fclose(config);
    if (subSize < 1 || width % subSize != 0 || height % subSize != 0 || depth % subSize != 0) {
        printf("Error: Grid[%d x %d x %d] cannot be divided by subSize[%d]\n", width, height, depth, subSize);
        return false;
    }
    coarseWidth = width / subSize;
    coarseHeight = height / subSize;
    coarseDepth = depth / subSize;
    voxelSize = (float)(1.0 / width);
    if (sources.empty()) {
        printf("ERROR: no smoke source exist\n");
        return false;
    }
    if (display) {
        printf("resolution %d %d %d, steps %d, stepTime %g, frames %d, SOR %d iterations (omega %g), %s solver\n",
               width, height, depth, steps, stepTime, frameCount, maxIter, omega,
               (is_closed(globalGridSolver) && !wallsExceptTop) ? "closed" : "open");
    }
    return true;
}

bool ZQ_SmokeSimulationPara3D::ToParams(zqs_params* p) const {
    if (!p || width < 2 || height < 2 || depth < 2) return false;
    if ((int)sources.size() > ZQS_MAX_SOURCES) return false;
    zqs_params_default(p, width, height, depth);
    p->voxel_size = voxelSize;
    p->step_time = stepTime;
    p->substeps = steps;
    p->confine = confineCoeff;
    p->buoyancy = buoyancyCoeff;
    p->gravity = gravityCoeff;
    p->tamb = Tamb;
    // exp(-stepTime * coeff) in float (ZQ_SmokeSimulationUtils3D.cpp:2098-2100)
    p->vel_atten = velAttenFactor >= 0.0f ? velAttenFactor : std::exp(-stepTime * velAttenCoeff);
    p->temp_atten = tempAttenFactor >= 0.0f ? tempAttenFactor : std::exp(-stepTime * tempAttenCoeff);
    p->dens_atten = densityAttenFactor >= 0.0f ? densityAttenFactor : std::exp(-stepTime * densityAttenCoeff);
    p->solver = (is_closed(globalGridSolver) && !wallsExceptTop) ? ZQS_SOLVER_CLOSED : ZQS_SOLVER_OPEN;
    // both coarse Poisson SOR settings run the open coarse solver, as the
    // reference's ZQ_TotalProjection3D does (Utils3D:3732-3746)
    if (globalGridSolver == COARSE_OPEN_POISSON_SOR || globalGridSolver == COARSE_CLOSED_POISSON_SOR)
        p->solver = ZQS_SOLVER_COARSE_OPEN;
    p->sub_size = subSize;
    p->sor_iters = maxIter;
    p->omega = omega;
    // the Para enum order differs from the CUDA header's (mapping of ZQ_SmokeSimulationUtils3D.cpp:2124-2148)
    switch (advVelType) {
        case ADV_VEL_INMAC_OUTMAC: p->adv_vel_mode = ZQS_ADV_VEL_INMAC_OUTMAC; break;
        case ADV_VEL_INMAC_OUTMAC_BFECC: p->adv_vel_mode = ZQS_ADV_VEL_INMAC_OUTMAC_BFECC; break;
        case ADV_VEL_INREG_OUTREG: p->adv_vel_mode = ZQS_ADV_VEL_INREG_OUTREG; break;
        case ADV_VEL_INREG_OUTREG_BFECC: p->adv_vel_mode = ZQS_ADV_VEL_INREG_OUTREG_BFECC; break;
        case ADV_VEL_INREG_OUTMAC: p->adv_vel_mode = ZQS_ADV_VEL_INREG_OUTMAC; break;
        case ADV_VEL_INREG_OUTMAC_BFECC: p->adv_vel_mode = ZQS_ADV_VEL_INREG_OUTMAC_BFECC; break;
    }
    switch (advScaType) {
        case ADV_SCA_MAC: p->adv_sca_mode = ZQS_ADV_SCA_MAC; break;
        case ADV_SCA_MAC_BFECC: p->adv_sca_mode = ZQS_ADV_SCA_MAC_BFECC; break;
        case ADV_SCA_REG: p->adv_sca_mode = ZQS_ADV_SCA_REG; break;
        case ADV_SCA_REG_BFECC: p->adv_sca_mode = ZQS_ADV_SCA_REG_BFECC; break;
    }
    p->backtrace_full = backtraceFull ? 1 : 0;
    // sources in cell units: centre and half extents times the grid size (Utils3D:3855-3860)
    p->n_sources = (int)sources.size();
    for (size_t i = 0; i < sources.size(); i++) {
        const ZQ_SmokeSource3D& s = sources[i];
        zqs_source& d = p->sources[i];
        d.shape = s.sphere ? ZQS_SOURCE_SPHERE : ZQS_SOURCE_BOX;
        d.cx = s.cx * (float)width;
        d.cy = s.cy * (float)height;
        d.cz = s.cz * (float)depth;
        d.hx = s.half_xlen * (float)width;
        d.hy = s.sphere ? d.hx : s.half_ylen * (float)height;
        d.hz = s.sphere ? d.hx : s.half_zlen * (float)depth;
        d.density = s.reinjectDensity;
        d.temperature = s.reinjectTemperature;
    }
    return true;
}

// ----------------------------------------------------------------- grid

ZQ_SmokeGrid3D::ZQ_SmokeGrid3D(const unsigned int w_, const unsigned int h_, const unsigned int d_)
    : width((int)w_), height((int)h_), depth((int)d_), dev(nullptr), host_stale(false) {
    const size_t n = (size_t)width * height * depth;
    occ_store.assign(n, 0);
    pressure_store.assign(n, 0.0f);
    temperature_store.assign(n, 0.0f);
    density_store.assign(n, 0.0f);
    u_store.assign((size_t)(width + 1) * height * depth, 0.0f);
    v_store.assign((size_t)width * (height + 1) * depth, 0.0f);
    w_store.assign((size_t)width * height * (depth + 1), 0.0f);
    occ = reinterpret_cast<bool*>(occ_store.data());
    pressure = pressure_store.data();
    temperature = temperature_store.data();
    density = density_store.data();
    u = u_store.data();
    v = v_store.data();
    w = w_store.data();
    ratioU = ratioV = ratioW = ratioVol = nullptr;
}

ZQ_SmokeGrid3D::~ZQ_SmokeGrid3D() {
    if (dev) zqs_grid_destroy(dev);
}

void ZQ_SmokeGrid3D::SyncHost() const {
    if (host_stale && dev) const_cast<ZQ_SmokeGrid3D*>(this)->Download();
}

bool*& ZQ_SmokeGrid3D::GetOccupyPtr() {
    SyncHost();
    return occ;
}
float*& ZQ_SmokeGrid3D::GetPressurePtr() {
    SyncHost();
    return pressure;
}
float*& ZQ_SmokeGrid3D::GetTemperaturePtr() {
    SyncHost();
    return temperature;
}
float*& ZQ_SmokeGrid3D::GetDensityPtr() {
    SyncHost();
    return density;
}
float*& ZQ_SmokeGrid3D::GetVelocityUptr() {
    SyncHost();
    return u;
}
float*& ZQ_SmokeGrid3D::GetVelocityVptr() {
    SyncHost();
    return v;
}
float*& ZQ_SmokeGrid3D::GetVelocityWptr() {
    SyncHost();
    return w;
}

void ZQ_SmokeGrid3D::BuildFaceUnOccupyRatio() {
    ratioU_store.assign((size_t)(width + 1) * height * depth, 0.0f);
    ratioV_store.assign((size_t)width * (height + 1) * depth, 0.0f);
    ratioW_store.assign((size_t)width * height * (depth + 1), 0.0f);
    ratioU = ratioU_store.data();
    ratioV = ratioV_store.data();
    ratioW = ratioW_store.data();
}
void ZQ_SmokeGrid3D::ClearFaceUnOccupyRatio() {
    ratioU_store.clear();
    ratioV_store.clear();
    ratioW_store.clear();
    ratioU = ratioV = ratioW = nullptr;
}
void ZQ_SmokeGrid3D::BuildVolumeUnOccupyRatio() {
    ratioVol_store.assign((size_t)width * height * depth, 0.0f);
    ratioVol = ratioVol_store.data();
}
void ZQ_SmokeGrid3D::ClearVolumeUnOccupyRatio() {
    ratioVol_store.clear();
    ratioVol = nullptr;
}

ZQ_SmokeGrid3D* ZQ_SmokeGrid3D::Clone() const {
    SyncHost();
    ZQ_SmokeGrid3D* t = new ZQ_SmokeGrid3D(width, height, depth);
    t->occ_store = occ_store;
    t->pressure_store = pressure_store;
    t->temperature_store = temperature_store;
    t->density_store = density_store;
    t->u_store = u_store;
    t->v_store = v_store;
    t->w_store = w_store;
    t->occ = reinterpret_cast<bool*>(t->occ_store.data());
    t->pressure = t->pressure_store.data();
    t->temperature = t->temperature_store.data();
    t->density = t->density_store.data();
    t->u = t->u_store.data();
    t->v = t->v_store.data();
    t->w = t->w_store.data();
    if (ratioU) {
        t->BuildFaceUnOccupyRatio();
        t->ratioU_store = ratioU_store;
        t->ratioV_store = ratioV_store;
        t->ratioW_store = ratioW_store;
        t->ratioU = t->ratioU_store.data();
        t->ratioV = t->ratioV_store.data();
        t->ratioW = t->ratioW_store.data();
    }
    if (ratioVol) {
        t->ratioVol_store = ratioVol_store;
        t->ratioVol = t->ratioVol_store.data();
    }
    return t;
}

bool ZQ_SmokeGrid3D::ExportDensity(const char* file, float quality) const {
    (void)quality;
    if (!file) return false;
    const size_t len = strlen(file);
    if (len < 4 || strcasecmp(file + len - 4, ".di3") != 0) return false;  // .zqwv/.zqci: not available
    SyncHost();
    FILE* f = fopen(file, "wb");
    if (!f) return false;
    char tag[16] = {0};
    memcpy(tag, "float", 5);
    const int32_t hdr[4] = {width, height, depth, 1};
    const uint8_t flag = 0;
    const size_t n = (size_t)width * height * depth;
    bool ok = fwrite(tag, 1, 16, f) == 16 && fwrite(hdr, 4, 4, f) == 4 && fwrite(&flag, 1, 1, f) == 1 &&
              fwrite(density, 4, n, f) == n;
    fclose(f);
    return ok;
}

bool ZQ_SmokeGrid3D::ExportOccupy(const char* file) const {
    (void)file;
    return true;
}
bool ZQ_SmokeGrid3D::ExportVelocity(const char* file) const {
    (void)file;
    return true;
}

bool ZQ_SmokeGrid3D::ExportGuide(const char* file) const {
    if (!file) return false;
    SyncHost();
    FILE* f = fopen(file, "wb");
    if (!f) return false;
    const size_t nu = u_store.size(), nv = v_store.size(), nw = w_store.size(), n = density_store.size();
    bool ok = fwrite(u, 4, nu, f) == nu && fwrite(v, 4, nv, f) == nv && fwrite(w, 4, nw, f) == nw &&
              fwrite(density, 4, n, f) == n && fwrite(temperature, 4, n, f) == n;
    fclose(f);
    return ok;
}

bool ZQ_SmokeGrid3D::ImportGuide(const char* file) {
    if (!file) return false;
    SyncHost();
    FILE* f = fopen(file, "rb");
    if (!f) return false;
    const size_t nu = u_store.size(), nv = v_store.size(), nw = w_store.size(), n = density_store.size();
    bool ok = fread(u, 4, nu, f) == nu && fread(v, 4, nv, f) == nv && fread(w, 4, nw, f) == nw &&
              fread(density, 4, n, f) == n && fread(temperature, 4, n, f) == n;
    fclose(f);
    host_stale = false;
    return ok;
}

zqs_grid* ZQ_SmokeGrid3D::DeviceGrid() {
    if (!dev && zqs_grid_create(&dev, width, height, depth) != ZQS_OK) dev = nullptr;
    return dev;
}

bool ZQ_SmokeGrid3D::Upload() {
    zqs_grid* g = DeviceGrid();
    if (!g) return false;
    if (zqs_grid_upload(g, ZQS_FIELD_OCCUPANCY, occ_store.data(), 0, nullptr) ||
        zqs_grid_upload(g, ZQS_FIELD_U, u, 0, nullptr) || zqs_grid_upload(g, ZQS_FIELD_V, v, 0, nullptr) ||
        zqs_grid_upload(g, ZQS_FIELD_W, w, 0, nullptr) ||
        zqs_grid_upload(g, ZQS_FIELD_TEMPERATURE, temperature, 0, nullptr) ||
        zqs_grid_upload(g, ZQS_FIELD_DENSITY, density, 0, nullptr))
        return false;
    host_stale = false;
    return zqs_grid_synchronize(g, nullptr) == ZQS_OK;
}

bool ZQ_SmokeGrid3D::Download() {
    if (!dev) return false;
    if (zqs_grid_download(dev, ZQS_FIELD_OCCUPANCY, occ_store.data(), 0, nullptr) ||
        zqs_grid_download(dev, ZQS_FIELD_U, u, 0, nullptr) || zqs_grid_download(dev, ZQS_FIELD_V, v, 0, nullptr) ||
        zqs_grid_download(dev, ZQS_FIELD_W, w, 0, nullptr) ||
        zqs_grid_download(dev, ZQS_FIELD_TEMPERATURE, temperature, 0, nullptr) ||
        zqs_grid_download(dev, ZQS_FIELD_DENSITY, density, 0, nullptr) ||
        zqs_grid_download(dev, ZQS_FIELD_PRESSURE, pressure, 0, nullptr))
        return false;
    host_stale = false;
    return zqs_grid_synchronize(dev, nullptr) == ZQS_OK;
}

// ----------------------------------------------------------------- free functions

void MACtoRegular4(int W, int H, int D, const float* mu, const float* mv, const float* mw, float* vel4) {
    // centre = 0.5*(lo + hi), .w = 0 (ZQ_SmokeSimulationUtils3D.cpp:355-373)
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                const size_t c = ((size_t)k * H + j) * W + i;
                vel4[c * 4 + 0] = 0.5f * (mu[((size_t)k * H + j) * (W + 1) + i] + mu[((size_t)k * H + j) * (W + 1) + i + 1]);
                vel4[c * 4 + 1] = 0.5f * (mv[((size_t)k * (H + 1) + j) * W + i] + mv[((size_t)k * (H + 1) + j + 1) * W + i]);
                vel4[c * 4 + 2] = 0.5f * (mw[c] + mw[c + (size_t)W * H]);
                vel4[c * 4 + 3] = 0.0f;
            }
}

void Regular4toMAC(int W, int H, int D, const float* vel4, float* mu, float* mv, float* mw) {
    // face = 0.5*(c[-1] + c), one-sided at domain faces (GPU semantics, ZQ_CUDA_MACtoRegular.cu:29-99)
    for (int k = 0; k < D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i <= W; i++) {
                const size_t f = ((size_t)k * H + j) * (W + 1) + i;
                const size_t c = ((size_t)k * H + j) * W + i;
                if (i == 0) mu[f] = vel4[c * 4 + 0];
                else if (i == W) mu[f] = vel4[(c - 1) * 4 + 0];
                else mu[f] = 0.5f * (vel4[(c - 1) * 4 + 0] + vel4[c * 4 + 0]);
            }
    for (int k = 0; k < D; k++)
        for (int j = 0; j <= H; j++)
            for (int i = 0; i < W; i++) {
                const size_t f = ((size_t)k * (H + 1) + j) * W + i;
                const size_t c = ((size_t)k * H + j) * W + i;
                if (j == 0) mv[f] = vel4[c * 4 + 1];
                else if (j == H) mv[f] = vel4[(c - W) * 4 + 1];
                else mv[f] = 0.5f * (vel4[(c - W) * 4 + 1] + vel4[c * 4 + 1]);
            }
    for (int k = 0; k <= D; k++)
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) {
                const size_t f = ((size_t)k * H + j) * W + i;
                const size_t pl = (size_t)W * H;
                if (k == 0) mw[f] = vel4[f * 4 + 2];
                else if (k == D) mw[f] = vel4[(f - pl) * 4 + 2];
                else mw[f] = 0.5f * (vel4[(f - pl) * 4 + 2] + vel4[f * 4 + 2]);
            }
}

bool ZQ_InitFineGrid3D(ZQ_SmokeGrid3D* g, const ZQ_SmokeSimulationPara3D& para) {
    if (!g) return false;
    const int W = para.width, H = para.height, D = para.depth;
    if (g->GetWidth() != W || g->GetHeight() != H || g->GetDepth() != D) return false;
    bool* occ = g->GetOccupyPtr();
    memset(occ, 0, (size_t)W * H * D);
    memset(g->GetPressurePtr(), 0, sizeof(float) * W * H * D);
    auto at = [&](int i, int j, int k) -> bool& { return occ[((size_t)k * H + j) * W + i]; };
    const bool closed = is_closed(para.globalGridSolver) && !para.wallsExceptTop;
    if (closed || para.wallsExceptTop) {
        // the six border layers of the closed solvers (Utils3D:1536-1584); the
        // open-top variant leaves the y = H-1 layer free
        for (int k = 0; k < D; k++)
            for (int j = 0; j < H; j++) at(0, j, k) = at(W - 1, j, k) = true;
        for (int k = 0; k < D; k++)
            for (int i = 0; i < W; i++) {
                at(i, 0, k) = true;
                if (closed) at(i, H - 1, k) = true;
            }
        for (int j = 0; j < H; j++)
            for (int i = 0; i < W; i++) at(i, j, 0) = at(i, j, D - 1) = true;
    }
    switch (para.intobj) {  // Utils3D:1587-1655 (integer divisions kept)
        case ZQ_SmokeSimulationPara3D::INT_OBJ_SPHERE:
            for (int k = 0; k < D; k++)
                for (int j = 0; j < H; j++)
                    for (int i = 0; i < W; i++) {
                        const double dz = k + 0.5 - D / 2, dy = j + 0.5 - H / 2, dx = i + 0.5 - W / 2;
                        if (dz * dz + dy * dy + dx * dx < W * W / 400.0) at(i, j, k) = true;
                    }
            break;
        case ZQ_SmokeSimulationPara3D::INT_OBJ_BOX:
            for (int k = 0; k < D; k++)
                for (int j = 0; j < H; j++)
                    for (int i = 0; i < W; i++)
                        if (std::fabs(k + 0.5 - D / 2) < D / 20 && std::fabs(j + 0.5 - H / 2) < H / 20 &&
                            std::fabs(i + 0.5 - W / 2) < W / 10)
                            at(i, j, k) = true;
            break;
        case ZQ_SmokeSimulationPara3D::INT_OBJ_OVAL:
            // the reference loops i over the height and j over the width and
            // indexes (row j, column i); kept, bounded to the grid
            for (int k = 0; k < D; k++)
                for (int i = 0; i < H; i++)
                    for (int j = 0; j < W; j++) {
                        const double a = std::sqrt((i + 0.5 - 3.0 * W / 7) * (i + 0.5 - 3.0 * W / 7) +
                                                   (j + 0.5 - H / 2) * (j + 0.5 - H / 2) +
                                                   (k + 0.5 - D / 2) * (k + 0.5 - D / 2));
                        const double b = std::sqrt((i + 0.5 - 4.0 * W / 7) * (i + 0.5 - 4.0 * W / 7) +
                                                   (j + 0.5 - H / 2) * (j + 0.5 - H / 2) +
                                                   (k + 0.5 - D / 2) * (k + 0.5 - D / 2));
                        if (a + b < W / 5.0 && i < W && j < H) at(i, j, k) = true;
                    }
            break;
        case ZQ_SmokeSimulationPara3D::INT_OBJ_SPECIAL1:
            for (int k = 0; k < D; k++)
                for (int j = 0; j < H; j++)
                    for (int i = 0; i < W; i++)
                        if ((j == H / 2 + 13 || j == H / 2 + 14) && (i % 4 == 0 || i % 4 == 3) && i >= 4 && i < W - 4)
                            at(i, j, k) = true;
            break;
        default: break;
    }
    for (size_t b = 0; b + 6 <= para.obstacleBoxes.size(); b += 6) {
        const int* o = &para.obstacleBoxes[b];
        for (int k = std::max(o[4], 0); k <= std::min(o[5], D - 1); k++)
            for (int j = std::max(o[2], 0); j <= std::min(o[3], H - 1); j++)
                for (int i = std::max(o[0], 0); i <= std::min(o[1], W - 1); i++) at(i, j, k) = true;
    }
    float* u = g->GetVelocityUptr();
    float* v = g->GetVelocityVptr();
    float* w = g->GetVelocityWptr();
    const size_t nu = (size_t)(W + 1) * H * D, nv = (size_t)W * (H + 1) * D, nw = (size_t)W * H * (D + 1);
    memset(u, 0, nu * 4);
    memset(v, 0, nv * 4);
    memset(w, 0, nw * 4);
    memset(g->GetTemperaturePtr(), 0, sizeof(float) * W * H * D);
    memset(g->GetDensityPtr(), 0, sizeof(float) * W * H * D);
    if (para.noiseAmp > 0.0f) {
        // seeded noise U(-a, a) on the open-rule live faces: u faces, then v, then w
        auto freec = [&](int i, int j, int k) { return !at(i, j, k); };
        const float a = para.noiseAmp;
        for (int k = 0; k < D; k++)
            for (int j = 0; j < H; j++)
                for (int i = 0; i <= W; i++) {
                    const size_t f = ((size_t)k * H + j) * (W + 1) + i;
                    const bool live = i == 0 ? freec(0, j, k) : i == W ? freec(W - 1, j, k)
                                                                      : freec(i, j, k) && freec(i - 1, j, k);
                    u[f] = live ? uniform_at(para.seed, f + 1, -a, a) : 0.0f;
                }
        for (int k = 0; k < D; k++)
            for (int j = 0; j <= H; j++)
                for (int i = 0; i < W; i++) {
                    const size_t f = ((size_t)k * (H + 1) + j) * W + i;
                    const bool live = j == 0 ? freec(i, 0, k) : j == H ? freec(i, H - 1, k)
                                                                      : freec(i, j, k) && freec(i, j - 1, k);
                    v[f] = live ? uniform_at(para.seed, nu + f + 1, -a, a) : 0.0f;
                }
        for (int k = 0; k <= D; k++)
            for (int j = 0; j < H; j++)
                for (int i = 0; i < W; i++) {
                    const size_t f = ((size_t)k * H + j) * W + i;
                    const bool live = k == 0 ? freec(i, j, 0) : k == D ? freec(i, j, D - 1)
                                                                      : freec(i, j, k) && freec(i, j, k - 1);
                    w[f] = live ? uniform_at(para.seed, nu + nv + f + 1, -a, a) : 0.0f;
                }
    }
    return true;
}

namespace {

// Device grid with this configuration's parameters and the host state.
zqs_grid* prepare(ZQ_SmokeGrid3D* g, const ZQ_SmokeSimulationPara3D& para, int solver_override = -1) {
    zqs_params p;
    if (!para.ToParams(&p)) return nullptr;
    if (solver_override >= 0) p.solver = solver_override;
    zqs_grid* d = g->DeviceGrid();
    if (!d) return nullptr;
    if (zqs_grid_set_params(d, &p) != ZQS_OK) return nullptr;
    if (!g->Upload()) return nullptr;
    return d;
}

bool finish(ZQ_SmokeGrid3D* g, int rc, const char* what) {
    if (rc != ZQS_OK) return fail(what);
    g->MarkHostStale();
    return g->Download() ? true : fail(what);
}

}  // namespace

bool ZQ_AddForce3D(ZQ_SmokeGrid3D* g, const ZQ_SmokeSimulationPara3D& para) {
    zqs_grid* d = g ? prepare(g, para) : nullptr;
    return d ? finish(g, zqs_stage_add_force(d, nullptr), "ZQ_AddForce3D") : false;
}

bool ZQ_Attenuation3D(ZQ_SmokeGrid3D* g, const ZQ_SmokeSimulationPara3D& para) {
    zqs_grid* d = g ? prepare(g, para) : nullptr;
    return d ? finish(g, zqs_stage_attenuate(d, nullptr), "ZQ_Attenuation3D") : false;
}

bool ZQ_AdvectVelocity3D(ZQ_SmokeGrid3D* g, const ZQ_SmokeSimulationPara3D& para) {
    zqs_params p;
    if (!para.ToParams(&p)) return false;
    zqs_grid* d = g ? prepare(g, para) : nullptr;
    return d ? finish(g, zqs_stage_advect_velocity(d, p.adv_vel_mode, 1, nullptr), "ZQ_AdvectVelocity3D") : false;
}

bool ZQ_SolveOpenPressure3DSOR(ZQ_SmokeGrid3D* g, const ZQ_SmokeSimulationPara3D& para) {
    zqs_grid* d = g ? prepare(g, para, ZQS_SOLVER_OPEN) : nullptr;
    return d ? finish(g, zqs_stage_project(d, nullptr), "ZQ_SolveOpenPressure3DSOR") : false;
}

bool ZQ_SolveClosedPressure3DSOR(ZQ_SmokeGrid3D* g, const ZQ_SmokeSimulationPara3D& para) {
    zqs_grid* d = g ? prepare(g, para, ZQS_SOLVER_CLOSED) : nullptr;
    return d ? finish(g, zqs_stage_project(d, nullptr), "ZQ_SolveClosedPressure3DSOR") : false;
}

bool ZQ_TotalProjection3D(ZQ_SmokeGrid3D* g, const ZQ_SmokeSimulationPara3D& para) {
    zqs_grid* d = g ? prepare(g, para) : nullptr;
    return d ? finish(g, zqs_stage_project(d, nullptr), "ZQ_TotalProjection3D") : false;
}

bool ZQ_AdvectScalar3D(ZQ_SmokeGrid3D* g, const ZQ_SmokeSimulationPara3D& para) {
    zqs_params p;
    if (!para.ToParams(&p)) return false;
    zqs_grid* d = g ? prepare(g, para) : nullptr;
    return d ? finish(g, zqs_stage_advect_scalar(d, p.adv_sca_mode, nullptr), "ZQ_AdvectScalar3D") : false;
}

bool ZQ_ReinjectTemperatureDensity3D(ZQ_SmokeGrid3D* g, const ZQ_SmokeSimulationPara3D& para) {
    zqs_grid* d = g ? prepare(g, para) : nullptr;
    return d ? finish(g, zqs_stage_reinject(d, nullptr), "ZQ_ReinjectTemperatureDensity3D") : false;
}

bool ZQ_UpdateOneFrame3D(ZQ_SmokeGrid3D* g, const ZQ_SmokeSimulationPara3D& para) {
    if (!ZQ_AddForce3D(g, para) || !ZQ_Attenuation3D(g, para) || !ZQ_AdvectVelocity3D(g, para)) return false;
    if (!ZQ_TotalProjection3D(g, para)) return false;
    return ZQ_AdvectScalar3D(g, para) && ZQ_ReinjectTemperatureDensity3D(g, para);
}

// ----------------------------------------------------------------- moving objects

ZQ_SmokeMovingObject3D::ZQ_SmokeMovingObject3D()
    : cx(0), cy(0), cz(0), posx(0), posy(0), posz(0), sizex(0), sizey(0), sizez(0), curstep(0), occupy(nullptr) {}

ZQ_SmokeMovingObject3D::~ZQ_SmokeMovingObject3D() { delete[] occupy; }

void ZQ_SmokeMovingObject3D::GetCenter(int& x, int& y, int& z) const { x = cx, y = cy, z = cz; }
void ZQ_SmokeMovingObject3D::GetPos(int& x, int& y, int& z) const { x = posx, y = posy, z = posz; }
void ZQ_SmokeMovingObject3D::GetSize(int& x, int& y, int& z) const { x = sizex, y = sizey, z = sizez; }

void ZQ_SmokeMovingObject3D::GetCurVel(int& u, int& v, int& w) const {
    const bool in = curstep >= 0 && (size_t)curstep < vels.size();
    u = in ? vels[curstep].x : 0;
    v = in ? vels[curstep].y : 0;
    w = in ? vels[curstep].z : 0;
}

const bool*& ZQ_SmokeMovingObject3D::GetOccupyPtr() const { return (const bool*&)occupy; }

void ZQ_SmokeMovingObject3D::UpdateOneStep() {
    if (curstep >= 0 && (size_t)curstep < vels.size()) {
        posx += vels[curstep].x;
        posy += vels[curstep].y;
        posz += vels[curstep].z;
    }
    curstep++;
}

bool LoadMovingObjects3D(const char* file, std::vector<ZQ_SmokeMovingObject3D*>& mvobjs) {
    FILE* in = file ? fopen(file, "r") : nullptr;
    if (!in) return false;
    auto next = [&](int& x) { return fscanf(in, "%d", &x) == 1; };
    int count = 0;
    bool ok = next(count) && count >= 0;
    for (int q = 0; ok && q < count; q++) {
        auto* o = new ZQ_SmokeMovingObject3D();
        int nsteps = 0;
        ok = next(o->sizex) && next(o->sizey) && next(o->sizez) && next(o->cx) && next(o->cy) && next(o->cz) &&
             next(o->posx) && next(o->posy) && next(o->posz) && next(nsteps) && o->sizex >= 0 && o->sizey >= 0 &&
             o->sizez >= 0 && nsteps >= 0;
        for (int t = 0; ok && t < nsteps; t++) {
            int a, b, c;
            ok = next(a) && next(b) && next(c);
            if (ok) o->vels.emplace_back(a, b, c);
        }
        const size_t n = ok ? (size_t)o->sizex * o->sizey * o->sizez : 0;
        if (ok) o->occupy = new bool[n > 0 ? n : 1];
        for (size_t b = 0; ok && b < n; b++) {
            int x = 0;
            ok = next(x);
            o->occupy[b] = x != 0;
        }
        if (ok) mvobjs.push_back(o);
        else delete o;
    }
    fclose(in);
    return ok;
}

namespace {

// The objects' current positions and velocities stamped into the device grid.
bool stamp_objects(zqs_grid* d, const std::vector<ZQ_SmokeMovingObject3D*>& mvobjs,
                   const ZQ_SmokeSimulationPara3D& para) {
    static_assert(sizeof(bool) == 1, "object masks are passed as bytes");
    std::vector<zqs_object> objs;
    for (const ZQ_SmokeMovingObject3D* m : mvobjs) {
        if (!m || !m->occupy) continue;
        zqs_object o;
        o.mask = reinterpret_cast<const uint8_t*>(m->occupy);
        m->GetSize(o.size[0], o.size[1], o.size[2]);
        m->GetCenter(o.center[0], o.center[1], o.center[2]);
        m->GetPos(o.pos[0], o.pos[1], o.pos[2]);
        m->GetCurVel(o.vel[0], o.vel[1], o.vel[2]);
        objs.push_back(o);
    }
    // the reference rebuilds the six walls for its closed solvers; the open-top
    // walls of wallsExceptTop are kept the same way
    const int walls = para.wallsExceptTop ? 2 : is_closed(para.globalGridSolver) ? 1 : 0;
    if (zqs_grid_stamp_objects(d, objs.data(), (int)objs.size(), walls, nullptr) != ZQS_OK)
        return fail("ZQ_ApplyMovingObject3D");
    return zqs_grid_synchronize(d, nullptr) == ZQS_OK || fail("ZQ_ApplyMovingObject3D");
}

}  // namespace

bool ZQ_ApplyMovingObject3D(ZQ_SmokeGrid3D* g, const std::vector<ZQ_SmokeMovingObject3D*>& mvobjs,
                            const ZQ_SmokeSimulationPara3D& para) {
    zqs_grid* d = g ? prepare(g, para) : nullptr;
    if (!d || !stamp_objects(d, mvobjs, para)) return false;
    g->MarkHostStale();
    return g->Download() || fail("ZQ_ApplyMovingObject3D");
}

// ----------------------------------------------------------------- headless viewer

bool ZQ_LoadVolume3D(const char* file, int N, std::vector<float>& data, int& W, int& H, int& D) {
    if (!file) return false;
    const size_t len = strlen(file);
    auto ext = [&](const char* e) { return len >= strlen(e) && strcasecmp(file + len - strlen(e), e) == 0; };
    if (ext(".zqci") || ext(".zqwv")) return false;
    FILE* f = fopen(file, "rb");
    if (!f) return false;
    bool ok = false;
    if (ext(".di3")) {
        char tag[16];
        int32_t hdr[4];
        uint8_t flag;
        if (fread(tag, 1, 16, f) == 16 && strncmp(tag, "float", 5) == 0 && fread(hdr, 4, 4, f) == 4 &&
            fread(&flag, 1, 1, f) == 1 && hdr[0] > 0 && hdr[1] > 0 && hdr[2] > 0 && hdr[3] > 0) {
            W = hdr[0], H = hdr[1], D = hdr[2];
            const int ch = hdr[3];
            const size_t n = (size_t)W * H * D;
            std::vector<float> raw(n * ch);
            if (fread(raw.data(), 4, raw.size(), f) == raw.size()) {
                data.assign(n, 0.0f);
                for (size_t c = 0; c < n; c++) {
                    float s = 0.0f;
                    for (int q = 0; q < ch; q++) s += raw[c * ch + q];
                    data[c] = ch == 1 ? s : s / (float)ch;
                }
                ok = true;
            }
        }
    } else if (N > 0) {
        const size_t n = (size_t)N * N * N;
        std::vector<float> raw(n);
        if (fread(raw.data(), 4, n, f) == n) {
            W = H = D = N;
            data.assign(n, 0.0f);
            for (int i = 0; i < N; i++)
                for (int j = 0; j < N; j++)
                    for (int k = 0; k < N; k++)
                        data[((size_t)i * N + j) * N + k] = raw[((size_t)k * N + j) * N + i];
            ok = true;
        }
    }
    fclose(f);
    return ok;
}

bool ZQ_RenderVolume3D(const float* density, int W, int H, int D, const zqs_camera& cam, std::vector<float>& rgba) {
    if (!density || W <= 0 || H <= 0 || D <= 0 || cam.width <= 0 || cam.height <= 0) return false;
    const size_t nv = (size_t)W * H * D, ni = (size_t)cam.width * cam.height * 4;
    float *dv = nullptr, *di = nullptr;
    bool ok = cudaMalloc(&dv, nv * sizeof(float)) == cudaSuccess && cudaMalloc(&di, ni * sizeof(float)) == cudaSuccess &&
              cudaMemcpy(dv, density, nv * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok) ok = zqs_render_density(dv, W, H, D, &cam, di, nullptr) == ZQS_OK || fail("ZQ_RenderVolume3D");
    if (ok) {
        rgba.resize(ni);
        ok = cudaMemcpy(rgba.data(), di, ni * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess;
    }
    cudaFree(dv);
    cudaFree(di);
    return ok;
}

bool ZQ_WriteRenderPPM(const char* file, const std::vector<float>& rgba, int width, int height) {
    if (!file || width <= 0 || height <= 0 || rgba.size() < (size_t)width * height * 4) return false;
    FILE* f = fopen(file, "wb");
    if (!f) return false;
    fprintf(f, "P6\n%d %d\n255\n", width, height);
    std::vector<uint8_t> row((size_t)width * 3);
    bool ok = true;
    for (int y = height - 1; y >= 0 && ok; y--) {  // top row first
        for (int x = 0; x < width; x++)
            for (int c = 0; c < 3; c++) {
                const float v = std::min(std::max(rgba[((size_t)y * width + x) * 4 + c], 0.0f), 1.0f);
                row[(size_t)x * 3 + c] = (uint8_t)(v * 255.0f + 0.5f);
            }
        ok = fwrite(row.data(), 1, row.size(), f) == row.size();
    }
    fclose(f);
    return ok;
}

bool ZQ_RenderSequence3D(const char* fold, const char* prefix, int baseID, int num, const char* suffix, int N,
                         int imageWidth, int imageHeight, const char* outFold) {
    if (!fold || !prefix || !suffix || !outFold || num < 0) return false;
    for (int n = 0; n < num; n++) {
        const std::string in = std::string(fold) + "/" + prefix + std::to_string(baseID + n) + suffix;
        std::vector<float> vol, img;
        int W = 0, H = 0, D = 0;
        if (!ZQ_LoadVolume3D(in.c_str(), N, vol, W, H, D)) {
            fprintf(stderr, "zqs: cannot read %s\n", in.c_str());
            return false;
        }
        zqs_camera cam;
        zqs_camera_default(&cam, imageWidth, imageHeight, W, H, D);
        if (!ZQ_RenderVolume3D(vol.data(), W, H, D, cam, img)) return false;
        const std::string out = std::string(outFold) + "/render" + std::to_string(baseID + n) + ".ppm";
        if (!ZQ_WriteRenderPPM(out.c_str(), img, imageWidth, imageHeight)) return false;
    }
    return true;
}

// ----------------------------------------------------------------- simulation

ZQ_SmokeSimulation3D::ZQ_SmokeSimulation3D() : fineGrid(nullptr), frame(0) {}

ZQ_SmokeSimulation3D::~ZQ_SmokeSimulation3D() {
    delete fineGrid;
    for (ZQ_SmokeMovingObject3D* o : mvobjs) delete o;
}

bool ZQ_SmokeSimulation3D::Init(const char* file) {
    if (!para.LoadFromFile(file, true)) return false;
    for (ZQ_SmokeMovingObject3D* o : mvobjs) delete o;
    mvobjs.clear();
    frame = 0;
    if (para.useMovingObject && !LoadMovingObjects3D(para.movingObjectFile, mvobjs)) {
        printf("cannot read the moving objects of %s\n", para.movingObjectFile);
        return false;
    }
    if (para.exportType != ZQ_SmokeSimulationPara3D::EXPORT_DI3) {
        printf("only the .di3 export is available in this library\n");
        return false;
    }
    const GlobalSolverType3D s = para.globalGridSolver;
    if (s != TOTAL_OPEN_POISSON_SOR && s != TOTAL_CLOSED_POISSON_SOR && s != COARSE_OPEN_POISSON_SOR &&
        s != COARSE_CLOSED_POISSON_SOR)
        printf("note: globalGridSolver %d runs as the fine-grid %s red-black SOR\n", (int)s,
               is_closed(s) && !para.wallsExceptTop ? "closed" : "open");
    delete fineGrid;
    fineGrid = new ZQ_SmokeGrid3D(para.width, para.height, para.depth);
    if (!ZQ_InitFineGrid3D(fineGrid, para)) return false;
    zqs_params p;
    if (!para.ToParams(&p)) return false;
    zqs_grid* d = prepare(fineGrid, para);
    if (!d) return fail("Init");
    // the objects at their start positions (_initRegular, ZQ_SmokeSimulation3D.cpp:293-310)
    if (para.useMovingObject) {
        if (!stamp_objects(d, mvobjs, para)) return false;
        fineGrid->MarkHostStale();
    }
    return true;
}

bool ZQ_SmokeSimulation3D::UpdateOneFrame(const void* guideGrid) {
    if (!fineGrid || guideGrid) return false;
    zqs_grid* d = fineGrid->DeviceGrid();
    if (!d) return fail("UpdateOneFrame");
    // re-applied from the second frame on, advanced after the step
    // (ZQ_SmokeSimulation3D.cpp:161-173, 232-241)
    frame++;
    if (para.useMovingObject && frame > 1 && !stamp_objects(d, mvobjs, para)) return false;
    if (zqs_grid_step(d, 1, nullptr) != ZQS_OK) return fail("UpdateOneFrame");
    fineGrid->MarkHostStale();
    if (para.useMovingObject)
        for (ZQ_SmokeMovingObject3D* o : mvobjs)
            if (o) o->UpdateOneStep();
    return true;
}

ZQ_SmokeGrid3D* ZQ_SmokeSimulation3D::GetFineGrid() {
    if (fineGrid) fineGrid->GetDensityPtr();  // brings the host arrays up to date
    return fineGrid;
}

bool ZQ_SmokeSimulation3D::Run(const char* fold) {
    if (!fineGrid || !fold) return false;
    std::string base(fold);
    for (int i = 0; i < para.frameCount; i++) {
        if (!UpdateOneFrame(nullptr)) return false;
        const std::string name = base + "/frame" + std::to_string(i) + ".di3";
        if (!fineGrid->ExportDensity(name.c_str(), para.export_quality)) return false;
        if (para.exportGuide) {
            const std::string gname = base + "/" + std::to_string(i) + ".guidedat";
            if (!fineGrid->ExportGuide(gname.c_str())) return false;
        }
    }
    return true;
}
