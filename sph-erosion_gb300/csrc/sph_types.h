// Device-side scene descriptor and layout constants shared by the kernels
// and the host engine.
#pragma once
#include <stdint.h>

namespace sph {

// Keys per scan chunk.  Each scene's key range is padded to a whole number
// of chunks so that the scan kernel never handles a ragged tail.
constexpr int kChunkBits = 12;
constexpr int kChunk = 1 << kChunkBits;
constexpr int kScanThreads = 256;           // 16 keys per thread
constexpr int kMaxTile = 256;    // particles per work tile: 128 or 256
constexpr int kRangeAlign = 512; // particle and terrain ranges start on this boundary

enum SceneFlags : int {
    kFlagTerrain = 1,
    kFlagErosion = 2,
    kFlagRecord = 4,
    kFlagOrdered = 8,
};

// Per-particle record floats written in record mode (sorted order):
// acc3 fpress3 fvisc3 fgrav3 fsurf3 normal3
constexpr int kRecFloats = 18;

// One scene as the kernels see it.  All offsets are global indices into the
// system's arenas.  FP32 constants are computed on the host with the same
// expressions as the reference so that they carry the same bits.
struct SceneDev {
    // ranges
    int p_off, n, p_cap;     // particles [p_off, p_off + n), capacity p_cap
    int k_off, nkeys, k_cap; // keys [k_off, k_off + nkeys), nkeys includes the end sentinel
    int c_off, nchunks;      // scan chunk sums
    int t_off, tw, td;       // terrain vertices (tw along x, td along z)
    int tab_off;             // row numbers (Morton order): row (y, z) at tab_off + z * ny + y
    int nx, ny, nz, reach;   // cell grid and stencil reach in cells
    int flags;
    int xsub;                // x cells per y/z cell: 2 at reach 1 (cells of h or more), else 1
    // grid
    float lo[3];
    float inv_cell;          // per metre, along y and z
    float inv_cell_x;        // per metre, along x: xsub * inv_cell
    float hcell;             // h in cell units, enlarged to cover FP32 rounding (row trimming)
    // physics (Erosion/fluid_system.h:460-479)
    float h, hh;             // h and h*h
    float smax;              // largest s with sqrtf(s) <= h: s <= smax <=> length <= h
    float cthr;              // dist < cthr <=> (double)dist < 1e-4 (fluid_system.h:438)
    float mass, p0, k, visc, sigma, dt, cr;
    float g[3];
    float c_poly6, c_grad, c_spiky, inv_sqrt3;
    // box: centre, half extents, axis weights (exactly 1 for a cube)
    float box_c[3], box_l[3], box_w[3];
    // terrain
    float t_xlo, t_ylo, t_zlo, t_isx, t_isz, t_wmax, t_dmax, height_unit;
    // erosion
    float k_capacity, k_pick, k_dep, layer;
};

// Work item of a persistent kernel: (scene, first index of the tile).
struct Work {
    int scene;
    int start;
};

}  // namespace sph
