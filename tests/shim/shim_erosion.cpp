// Drives the drop-in with the terrain coupling on: the front end's Grid
// (Erosion/main.cpp:100-105) becomes the step's terrain, the fluid erodes
// it, and Grid::UpdateGrid then returns the eroded surface.
//
// usage: shim_erosion out.bin heightmap512.bin steps
// out.bin: int32 nsurf, the surface floats before; the same after the steps;
//          int32 nidx, the indices before; the same after;
//          int64 total units, int64 sediment units, int32 particles,
//          int32 nan particles (after the steps); int32 voxels at the surface
//          that are VOXEL_MAT after the last UpdateGrid
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fluid_system.h"

template <class T>
static void put(FILE* f, const std::vector<T>& v) {
    const int n = (int)v.size();
    std::fwrite(&n, 4, 1, f);
    std::fwrite(v.data(), sizeof(T), v.size(), f);
}

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 3;
    std::vector<unsigned char> img(512 * 512);
    FILE* hm = std::fopen(argv[2], "rb");
    if (!hm || std::fread(img.data(), 1, img.size(), hm) != img.size()) return 4;
    std::fclose(hm);
    const int steps = std::atoi(argv[3]);

    Grid grid(48, 255, 40);
    grid.LoadHeightfield(img.data());
    grid.UpdateGrid(48, 255, 40);
    const std::vector<float> s0 = grid.GetSurfaceParts();
    const std::vector<unsigned> i0 = grid.GetIndices();

    FluidSystemSPH fluid(SPH_FLAG_RECORD);
    fluid.SetOrigin(sph_shim::vec3(0.0f));
    fluid.Initialize(1000);  // the reference's default block, above the terrain
    fluid.SetDeltaTime(0.002f);
    fluid.SetTerrain(true, 0.1f / 255.0f);  // grey level 255 at a quarter of the box's height
    fluid.SetErosion(true, 0.2f, 20.0f, 5.0f);
    for (int s = 0; s < steps; s++) fluid.Run(grid);
    grid.UpdateGrid(48, 255, 40);
    const std::vector<float> s1 = grid.GetSurfaceParts();
    const std::vector<unsigned> i1 = grid.GetIndices();
    const sph_diag d = fluid.GetDiagnostics();

    put(f, s0);
    put(f, s1);
    put(f, i0);
    put(f, i1);
    std::fwrite(&d.total_units, 8, 1, f);
    std::fwrite(&d.sediment_units, 8, 1, f);
    std::fwrite(&d.n, 4, 1, f);
    std::fwrite(&d.nan_particles, 4, 1, f);
    int mat = 0;
    for (int z = 0; z < 40; z++)
        for (int x = 0; x < 48; x++) {
            int y = (int)s1[6 * ((size_t)z * 48 + x) + 1];
            if (y < 0) y = 0;
            if (y > 254) y = 254;
            mat += grid.GetVoxel(x, y, z).type == VoxelType::VOXEL_MAT;
        }
    std::fwrite(&mat, 4, 1, f);
    std::fclose(f);
    return 0;
}
