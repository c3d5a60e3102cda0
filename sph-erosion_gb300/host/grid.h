// Drop-in Grid for the reference's front end (Erosion/grid.h:26-841),
// backed by libsph_gb300.so.  Same class name, constructor and methods; the
// surface mesh of UpdateGrid/genIndices is computed on the GPU
// (sph_terrain_mesh_u8) with the reference's arithmetic, bit for bit.
//
// The voxel array and the 512 x 512 8-bit heightfield stay on the host, as
// in the reference (the front end reads them for drawing).  collision() is
// the reference's triangle contact on this integer grid
// (sph_grid_collision_u8); the reference's step does not call it
// (Erosion/fluid_system.h:335-340).
//
// Terrain coupling (no counterpart in the reference, off until the fluid
// system turns it on): a FluidSystemSPH with terrain on takes this grid's
// heightfield, the dimX x dimZ block that UpdateGrid meshes, as its step's
// terrain, and from then on UpdateGrid and GetSurfaceParts return that
// terrain as the step has eroded it, in this grid's units (vertex (x, h, z),
// h in grey levels), until the heightfield or the dimensions change.
#pragma once
#include <cstdint>
#include <cstring>
#include <memory>
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

// The scene a fluid system made from a grid's heightfield (shared by the
// two; the fluid system clears `sys` when it goes away).
struct sph_terrain_link {
    sph_system* sys = nullptr;
    int scene = -1;
    float metres_per_level = 0.0f;
    int dimx = 0, dimz = 0;
    uint64_t version = 0;  // the grid's heightfield version it was made from
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
    void LoadHeightfield(unsigned char* img) {
        std::memcpy(m_map.data(), img, m_map.size());
        ++m_version;
    }

    unsigned char GetHeightfieldAt(int x, int y) { return m_map[(size_t)512 * x + y]; }

    // Surface vertices + normals and triangle indices (grid.h:138-176).  When
    // a fluid system erodes this grid's heightfield at these dimensions, the
    // eroded surface (sph_scene_terrain_mesh_levels), else the reference's.
    void UpdateGrid(int dimx, int dimy, int dimz) {
        if (dimx != m_DimX || dimz != m_DimZ) ++m_version;
        m_DimX = dimx;
        m_DimY = dimy;
        m_DimZ = dimz;
        m_Dim = sph_shim::vec3((float)dimx, (float)dimy, (float)dimz);
        m_Grid.assign((size_t)dimx * dimy * dimz, Voxel());
        surfaceParts.assign((size_t)dimx * dimz * 6, 0.0f);
        int64_t ni = 0;
        if (eroding()) {
            ni = (int64_t)6 * (dimx - 1) * (dimz - 1);
            indices.assign((size_t)ni, 0u);
            check(sph_scene_terrain_mesh_levels(m_link->sys, m_link->scene, m_link->metres_per_level,
                                                surfaceParts.data(), indices.data()));
        } else {
            check(sph_terrain_mesh_u8(m_map.data(), dimx, dimy, dimz, nullptr, nullptr, 0, &ni));
            indices.assign((size_t)ni, 0u);
            check(sph_terrain_mesh_u8(m_map.data(), dimx, dimy, dimz, surfaceParts.data(), indices.data(), ni,
                                      &ni));
        }
        for (int z = 0; z < dimz; z++)
            for (int x = 0; x < dimx; x++) {
                int y = (int)surfaceParts[6 * ((size_t)z * dimx + x) + 1];
                if (y < 0) y = 0;
                if (y > dimy - 1) y = dimy - 1;
                SetVoxel(x, y, z, VoxelType::VOXEL_MAT);
            }
    }

    // ---- terrain coupling (no counterpart in the reference) ----
    // Version of the heightfield and dimensions: changes on LoadHeightfield
    // and when UpdateGrid changes dimX or dimZ.
    uint64_t HeightfieldVersion() const { return m_version; }
    int DimX() const { return m_DimX; }
    int DimZ() const { return m_DimZ; }
    // Heights of the dimX x dimZ block in metres (grey level x
    // metres_per_level), z-major: out[z * dimX + x] = map[512 x + z].
    std::vector<float> BlockHeights(float metres_per_level) const {
        std::vector<float> h((size_t)m_DimX * m_DimZ);
        for (int z = 0; z < m_DimZ; z++)
            for (int x = 0; x < m_DimX; x++)
                h[(size_t)z * m_DimX + x] = (float)m_map[(size_t)512 * x + z] * metres_per_level;
        return h;
    }
    void Link(std::shared_ptr<sph_terrain_link> link) { m_link = std::move(link); }
    // True while UpdateGrid shows the eroded surface.
    bool eroding() const {
        return m_link && m_link->sys && m_link->version == m_version && m_link->dimx == m_DimX &&
               m_link->dimz == m_DimZ;
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
    uint64_t m_version = 1;
    std::shared_ptr<sph_terrain_link> m_link;
    sph_shim::vec3 m_Dim;
    std::vector<Voxel> m_Grid;
    std::vector<unsigned char> m_map;
    std::vector<float> surfaceParts;
    std::vector<float> fluidParts;
    std::vector<unsigned int> indices;
};
