// Drives the drop-in FluidSystemSPH and Grid the way the reference's front end
// does (Erosion/main.cpp:100-105, :170-183, :220-313, :476-516) and writes what
// it saw to a binary file for the parity test:
//   int32 count, then per particle 27 floats + int32 NeighbId   (after step 1)
//   same after step 10
//   int32 surface floats, floats; int32 index count, uint32 indices  (Grid::UpdateGrid)
//   int32 count after Reset() + AddParticles(125)
//   with a collision map and queries: int32 n, then per query int32 hit and
//   6 floats contact + normal (Grid::collision on a Grid(dx, 256, dz))
//
// usage: shim_main out.bin heightmap512.bin ordered|fast [collision_map512.bin queries.bin]
//   queries.bin: int32 dx, int32 dz, int32 n, n * 9 floats (cur, next, vel)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fluid_system.h"

static void write_records(FILE* f, FluidSystemSPH& sys, int n) {
    std::fwrite(&n, 4, 1, f);
    for (int i = 0; i < n; i++) {
        FluidParticle p = sys.GetParticle(i);
        float r[27];
        const sph_shim::vec3* v[] = {&p.Position, &p.Velocity, &p.Acceleration};
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) r[3 * a + c] = (*v[a])[c];
        r[9] = p.Density;
        r[10] = p.Pressure;
        const sph_shim::vec3* w[] = {&p.PressureForce, &p.ViscosityForce, &p.GravityForce, &p.SurfaceForce,
                                     &p.SurfaceNormal};
        for (int a = 0; a < 5; a++)
            for (int c = 0; c < 3; c++) r[11 + 3 * a + c] = (*w[a])[c];
        r[26] = 0.0f;
        std::fwrite(r, 4, 27, f);
        std::fwrite(&p.NeighbId, 4, 1, f);
    }
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const bool ordered = argc > 3 && std::strcmp(argv[3], "ordered") == 0;
    FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 3;
    std::vector<unsigned char> img(512 * 512);
    FILE* hm = std::fopen(argv[2], "rb");
    if (!hm || std::fread(img.data(), 1, img.size(), hm) != img.size()) return 4;
    std::fclose(hm);

    Grid grid(50, 255, 50);
    grid.LoadHeightfield(img.data());
    grid.UpdateGrid(50, 255, 50);

    FluidSystemSPH fluidsph(ordered ? (SPH_FLAG_RECORD | SPH_FLAG_ORDERED) : SPH_FLAG_RECORD);
#ifdef SPH_SHIM_HAS_GLM
    fluidsph.SetOrigin(glm::vec3(0.0));  // as Erosion/main.cpp:170
#else
    fluidsph.SetOrigin(sph_shim::vec3(0.0f));
#endif
    fluidsph.Initialize(1000);
    fluidsph.Run(grid);  // deltaT = 0: paused, as the front end starts
    fluidsph.SetDeltaTime(0.01f);  // the F key
    fluidsph.Run(grid);
    write_records(f, fluidsph, 1000);
    for (int s = 1; s < 10; s++) fluidsph.Run(grid);
    write_records(f, fluidsph, 1000);

    std::vector<float> surf = grid.GetSurfaceParts();
    std::vector<unsigned> idx = grid.GetIndices();
    int ns = (int)surf.size(), ni = (int)idx.size();
    std::fwrite(&ns, 4, 1, f);
    std::fwrite(surf.data(), 4, ns, f);
    std::fwrite(&ni, 4, 1, f);
    std::fwrite(idx.data(), 4, ni, f);

    // live parameter edit through the pointer getters, then the mouse buttons
    *fluidsph.GetMass() = 0.021f;
#ifdef SPH_SHIM_HAS_GLM
    glm::vec3* gr = fluidsph.GetGrav();  // as Erosion/main.cpp:283-290
    gr->y = -9.81f;
#else
    fluidsph.GetGrav()->y = -9.81f;
#endif
    fluidsph.Run(grid);
    fluidsph.Reset();
    fluidsph.AddParticles(125);
    fluidsph.Run(grid);
    int count = (int)(fluidsph.GetPositions().size() / 3);
    std::fwrite(&count, 4, 1, f);

    if (argc > 5) {
        std::vector<unsigned char> cmap(512 * 512);
        FILE* cm = std::fopen(argv[4], "rb");
        if (!cm || std::fread(cmap.data(), 1, cmap.size(), cm) != cmap.size()) return 5;
        std::fclose(cm);
        FILE* qf = std::fopen(argv[5], "rb");
        int hdr[3];
        if (!qf || std::fread(hdr, 4, 3, qf) != 3) return 6;
        std::vector<float> q((size_t)hdr[2] * 9);
        if (std::fread(q.data(), 4, q.size(), qf) != q.size()) return 7;
        std::fclose(qf);
        Grid cg(hdr[0], 256, hdr[1]);
        cg.LoadHeightfield(cmap.data());
        std::fwrite(&hdr[2], 4, 1, f);
        for (int i = 0; i < hdr[2]; i++) {
            const float* r = &q[(size_t)9 * i];
            sph_shim::vec3 cp(0.0f), nr(0.0f);
            const int32_t hit = cg.collision(sph_shim::vec3(r[0], r[1], r[2]), sph_shim::vec3(r[3], r[4], r[5]),
                                             sph_shim::vec3(r[6], r[7], r[8]), cp, nr) ? 1 : 0;
            const float o[6] = {cp.x, cp.y, cp.z, nr.x, nr.y, nr.z};
            std::fwrite(&hit, 4, 1, f);
            std::fwrite(o, 4, 6, f);
        }
    }
    std::fclose(f);
    return 0;
}
