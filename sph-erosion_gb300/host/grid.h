// Drop-in Grid for the reference's front end (Erosion/grid.h:26-841),
// backed by libsph_gb300.so.  Same class name, constructor and methods; the
// surface mesh of UpdateGrid/genIndices is computed on the GPU
// (sph_terrain_mesh_u8) with the reference's arithmetic, bit for bit.
//
// The voxel array and the 512 x 512 8-bit heightfield stay on the host, as
// in the reference (the front end reads them for drawing).  collision() is
// the reference's triangle contact on this integer grid
// (sph_grid_collision_u8); the reference's step does not call it
// (Erosion/fluid_system.h:335-340), and the step's terrain contact is the
// scene's FP32 heightfield (sph_scene_set_terrain).
#pragma once
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "sph_erosion.h"
#include "sph_vec3.h"

enum class VoxelType { VOXEL_AIR = 0, VOXEL_WAT, VOXEL_MAT };

struct Voxel {
    float density;
    sph_shim::vec3 position;
    sph_shim::vec3 velocity;
    VoxelType type;

    Voxel() : density(0), position(0.0f), velocity(0.0f), type(VoxelType::VOXEL_AIR) {}
    explicit Voxel(VoxelType t) : density(0), position(0.0f), velocity(0.0f), type(t) {}
};

class Grid {
   public:
    Grid(int dimX = 512, int dimY = 512, int dimZ = 512)
        : m_DimX(dimX), m_DimY(dimY), m_DimZ(dimZ), m_Dim((float)dimX, (float)dimY, (float)dimZ),
          m_Grid((size_t)dimX * dimY * dimZ), m_map(512 * 512, 0) {}

    Voxel GetVoxel(int x, int y, int z) const { return m_Grid[x + m_DimX * (y + m_DimY * z)]; }

    void SetVoxel(int x, int y, int z, VoxelType type) {
        Voxel& v = m_Grid[x + m_DimX * (y + m_DimY * z)];
        v.type = type;
        v.position = sph_shim::vec3((float)x, (float)y, (float)z);
    }

    // Copies 512 * 512 bytes, x-major (grid.h:98-102).
    void LoadHeightfield(unsigned char* img) { std::memcpy(m_map.data(), img, m_map.size()); }

    unsigned char GetHeightfieldAt(int x, int y) { return m_map[(size_t)512 * x + y]; }

    // Surface vertices + normals and triangle indices (grid.h:138-176).
    void UpdateGrid(int dimx, int dimy, int dimz) {
        m_DimX = dimx;
        m_DimY = dimy;
        m_DimZ = dimz;
        m_Dim = sph_shim::vec3((float)dimx, (float)dimy, (float)dimz);
        m_Grid.assign((size_t)dimx * dimy * dimz, Voxel());
        surfaceParts.assign((size_t)dimx * dimz * 6, 0.0f);
        int64_t ni = 0;
        check(sph_terrain_mesh_u8(m_map.data(), dimx, dimy, dimz, nullptr, nullptr, 0, &ni));
        indices.assign((size_t)ni, 0u);
        check(sph_terrain_mesh_u8(m_map.data(), dimx, dimy, dimz, surfaceParts.data(), indices.data(), ni, &ni));
        for (int z = 0; z < dimz; z++)
            for (int x = 0; x < dimx; x++) SetVoxel(x, (int)surfaceParts[6 * ((size_t)z * dimx + x) + 1], z,
                                                    VoxelType::VOXEL_MAT);
    }

    // The reference's triangle contact against this grid (grid.h:462-805),
    // run on the GPU with the reference's arithmetic.  Its only call site is
    // commented out (fluid_system.h:335-340); the step's own terrain contact
    // is against the scene's heightfield.  As in the reference, contactP and
    // norm are written only on a hit.
    bool collision(const sph_shim::vec3& posCurr, const sph_shim::vec3& posNext, const sph_shim::vec3& velNext,
                   sph_shim::vec3& contactP, sph_shim::vec3& norm) {
        int32_t hit = 0;
        sph_shim::vec3 cp, nr;
        check(sph_grid_collision_u8(m_map.data(), m_DimX, m_DimZ, 1, &posCurr.x, &posNext.x, &velNext.x, &cp.x,
                                    &nr.x, &hit));
        if (hit) {
            contactP = cp;
            norm = nr;
        }
        return hit != 0;
    }

    std::vector<unsigned int> GetIndices() { return indices; }
    size_t GetIndicesSize() const { return indices.size(); }
    sph_shim::vec3 GetDim() const { return m_Dim; }
    std::vector<float> GetSurfaceParts() { return surfaceParts; }
    size_t GetSurfacePartsSize() const { return surfaceParts.size(); }
    std::vector<float> GetFluidParts() { return fluidParts; }
    size_t GetFluidPartsSize() const { return fluidParts.size(); }

   private:
    static void check(int rc) {
        if (rc != SPH_OK) throw std::runtime_error(std::string("sph: ") + sph_last_error());
    }

    int m_DimX, m_DimY, m_DimZ;
    sph_shim::vec3 m_Dim;
    std::vector<Voxel> m_Grid;
    std::vector<unsigned char> m_map;
    std::vector<float> surfaceParts;
    std::vector<float> fluidParts;
    std::vector<unsigned int> indices;
};
