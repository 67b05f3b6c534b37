// The time loop of the reference's solver (src/main.cpp:38-104) around sdfibm_gb300::SolidCloud, with the fluid
// solve replaced by a fixed velocity field read from a file: construction (initialCorrect), saveState, then per
// step interact, evolve, saveState, fixInternal, and a restart dictionary at the end.
//
//   cloud_client SOLIDDICT MESH U_FILE STEPS DT OUTDIR
//
// MESH holds "nx ny nz ox oy oz hx hy hz"; U_FILE 3 N float32 values (x, y, z planes).  OUTDIR receives cloud.out,
// meanfield.out (when the dictionary asks for it) and solidDict.restart; stdout the total solid volume and the
// force on solid 0 of the last step.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iterator>
#include <sstream>
#include <string>
#include <vector>

#include <unistd.h>

#include "sdfibm_cloud.hpp"

int main(int argc, char** argv) {
    if (argc < 7) {
        std::fprintf(stderr, "usage: cloud_client SOLIDDICT MESH U_FILE STEPS DT OUTDIR\n");
        return 2;
    }
    std::ifstream df(argv[1]);
    const std::string dict((std::istreambuf_iterator<char>(df)), std::istreambuf_iterator<char>());
    sdfibm_mesh_desc mesh{};
    {
        std::ifstream mf(argv[2]);
        mf >> mesh.nx >> mesh.ny >> mesh.nz >> mesh.origin[0] >> mesh.origin[1] >> mesh.origin[2] >> mesh.h[0] >>
            mesh.h[1] >> mesh.h[2];
        if (!mf) return 3;
    }
    const size_t N = (size_t)mesh.nx * mesh.ny * mesh.nz;
    std::vector<float> U(3 * N);
    {
        std::ifstream uf(argv[3], std::ios::binary);
        uf.read(reinterpret_cast<char*>(U.data()), (std::streamsize)(U.size() * sizeof(float)));
        if (!uf) return 4;
    }
    const int steps = std::atoi(argv[4]);
    const double dt = std::atof(argv[5]);
    if (chdir(argv[6]) != 0) return 5;
    try {
        sdfibm_gb300::SolidCloud cloud(dict, mesh, 1.0, 0.0, U.data(), "cloud.out");
        cloud.saveState();  // the initial condition
        for (int s = 1; s <= steps; ++s) {
            const double t = s * dt;
            cloud.U() = U;  // the fluid solver's velocity
            cloud.interact(t, dt);
            cloud.evolve(t, dt);
            cloud.saveState();
            if (cloud.isOnFluid()) cloud.fixInternal(dt);
        }
        cloud.saveRestart("solidDict.restart", 17);
        const double* ft = cloud.fluidForceTorque(0);
        std::printf("volume %.17g\nforce0 %.17g %.17g %.17g\nsolids %d\n", cloud.totalSolidVolume(), ft[0], ft[1],
                    ft[2], cloud.size());
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
