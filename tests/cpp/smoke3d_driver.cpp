// Test driver of the C++ host API (include/zqs_smoke3d.h), built and run by
// tests/test_smoke3d.py against libzqs_gb300.so.
//   smoke3d_driver parse  <config> <outdir>   parameters and initial state only (no GPU)
//   smoke3d_driver run    <config> <outdir>   ZQ_SmokeSimulation3D::Init + Run (resident)
//   smoke3d_driver stages <config> <outdir>   ZQ_InitFineGrid3D + ZQ_UpdateOneFrame3D per frame
//                                             (+ ZQ_ApplyMovingObject3D as the class does)
//   smoke3d_driver loadvol <file> <outdir> [N] ZQ_LoadVolume3D, then vol.bin: int32 W, H, D and the floats (no GPU)
//   smoke3d_driver sequence <fold> <outdir> <prefix> <baseID> <num> <suffix> <N> <imgW> <imgH>
//                                             ZQ_RenderSequence3D into <outdir>
//   smoke3d_driver objects <file> <outdir>    LoadMovingObjects3D, then objects.txt: per object
//                                             size, centre, step count, mask sum and the
//                                             positions and current velocities over 4 steps (no GPU)
// Outputs in <outdir>: params.bin (zqs_params bytes), occupancy.bin (W*H*D bytes),
// init.guidedat (u, v, w, density, temperature) and frame files.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "zqs_smoke3d.h"

static bool write_bytes(const std::string& path, const void* p, size_t n) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = fwrite(p, 1, n, f) == n;
    fclose(f);
    return ok;
}

static bool dump_setup(const ZQ_SmokeSimulationPara3D& para, ZQ_SmokeGrid3D& g, const std::string& out) {
    zqs_params p;
    if (!para.ToParams(&p)) return false;
    const size_t n = (size_t)para.width * para.height * para.depth;
    return write_bytes(out + "/params.bin", &p, sizeof(p)) && write_bytes(out + "/occupancy.bin", g.GetOccupyPtr(), n) &&
           g.ExportGuide((out + "/init.guidedat").c_str());
}

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s parse|run|stages|objects|loadvol|sequence <config> <outdir> ...\n", argv[0]);
        return 2;
    }
    const std::string mode = argv[1], cfg = argv[2], out = argv[3];
    if (mode == "loadvol") {
        std::vector<float> vol;
        int W = 0, H = 0, D = 0;
        if (!ZQ_LoadVolume3D(cfg.c_str(), argc > 4 ? atoi(argv[4]) : 0, vol, W, H, D)) return 3;
        const int32_t dims[3] = {W, H, D};
        return write_bytes(out + "/vol.bin", dims, sizeof(dims)) &&
                       write_bytes(out + "/vol_data.bin", vol.data(), vol.size() * sizeof(float))
                   ? 0
                   : 4;
    }
    if (mode == "sequence") {
        if (argc != 11) return 2;
        return ZQ_RenderSequence3D(cfg.c_str(), argv[4], atoi(argv[5]), atoi(argv[6]), argv[7], atoi(argv[8]),
                                   atoi(argv[9]), atoi(argv[10]), out.c_str())
                   ? 0
                   : 3;
    }
    if (mode == "parse") {
        ZQ_SmokeSimulationPara3D para;
        if (!para.LoadFromFile(cfg.c_str(), false)) return 3;
        ZQ_SmokeGrid3D g(para.width, para.height, para.depth);
        if (!ZQ_InitFineGrid3D(&g, para)) return 4;
        return dump_setup(para, g, out) ? 0 : 5;
    }
    if (mode == "run") {
        ZQ_SmokeSimulation3D sim;
        if (!sim.Init(cfg.c_str())) return 3;
        ZQ_SmokeGrid3D* g = sim.GetFineGrid();
        if (!g || !dump_setup(sim.GetPara(), *g, out)) return 4;
        if (!sim.Run(out.c_str())) return 5;
        // the host arrays follow the device state on request
        ZQ_SmokeGrid3D* after = sim.GetFineGrid();
        return after->ExportGuide((out + "/final.guidedat").c_str()) ? 0 : 6;
    }
    if (mode == "objects") {
        std::vector<ZQ_SmokeMovingObject3D*> objs;
        if (!LoadMovingObjects3D(cfg.c_str(), objs)) return 3;
        FILE* f = fopen((out + "/objects.txt").c_str(), "w");
        if (!f) return 4;
        fprintf(f, "%d\n", (int)objs.size());
        for (ZQ_SmokeMovingObject3D* o : objs) {
            int sum = 0;
            for (int b = 0; b < o->sizex * o->sizey * o->sizez; b++) sum += o->GetOccupyPtr()[b] ? 1 : 0;
            fprintf(f, "%d %d %d %d %d %d %d %d", o->sizex, o->sizey, o->sizez, o->cx, o->cy, o->cz,
                    (int)o->vels.size(), sum);
            for (int t = 0; t < 4; t++) {
                int x, y, z, u, v, w;
                o->GetPos(x, y, z);
                o->GetCurVel(u, v, w);
                fprintf(f, " %d %d %d %d %d %d", x, y, z, u, v, w);
                o->UpdateOneStep();
            }
            fprintf(f, "\n");
            delete o;
        }
        fclose(f);
        return 0;
    }
    if (mode == "stages") {
        ZQ_SmokeSimulationPara3D para;
        if (!para.LoadFromFile(cfg.c_str(), false)) return 3;
        ZQ_SmokeGrid3D g(para.width, para.height, para.depth);
        if (!ZQ_InitFineGrid3D(&g, para)) return 4;
        std::vector<ZQ_SmokeMovingObject3D*> objs;
        if (para.useMovingObject) {
            if (!LoadMovingObjects3D(para.movingObjectFile, objs)) return 10;
            if (!ZQ_ApplyMovingObject3D(&g, objs, para)) return 11;
        }
        for (int i = 0; i < para.frameCount; i++) {
            if (para.useMovingObject && i > 0 && !ZQ_ApplyMovingObject3D(&g, objs, para)) return 11;
            if (!ZQ_UpdateOneFrame3D(&g, para)) return 5;
            for (ZQ_SmokeMovingObject3D* o : objs) o->UpdateOneStep();
            const std::string name = out + "/stage_frame" + std::to_string(i) + ".di3";
            if (!g.ExportDensity(name.c_str())) return 6;
        }
        for (ZQ_SmokeMovingObject3D* o : objs) delete o;
        // Clone, and a guide round trip through ImportGuide
        ZQ_SmokeGrid3D* c = g.Clone();
        const std::string gd = out + "/stage_final.guidedat";
        if (!c->ExportGuide(gd.c_str())) return 7;
        ZQ_SmokeGrid3D back(para.width, para.height, para.depth);
        if (!back.ImportGuide(gd.c_str())) return 8;
        const bool same = std::memcmp(back.GetDensityPtr(), g.GetDensityPtr(),
                                      sizeof(float) * para.width * para.height * para.depth) == 0;
        delete c;
        return same ? 0 : 9;
    }
    return 2;
}
