// Kernel launchers of the simulation step (implemented in sph_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_types.h"

namespace sph {

// Device pointers of one system's arenas, passed by value to every launcher.
struct DevArrays {
    const SceneDev* scenes;
    int* steps_left;          // per scene: -1 unlimited, 0 inactive, >0 remaining
    const Work* ptiles;       // particle tiles
    const int* n_ptiles;
    const Work* ctiles;       // scan chunks (start = chunk index within the scene)
    const int* n_ctiles;
    const Work* ttiles;       // terrain tiles
    const int* n_ttiles;
    const int* scene_list;    // active scene ids (diagnostics)
    // particles
    float4* pos;   // x y z id(bits)      current state
    float4* vel;   // vx vy vz sediment(bits)
    float4* spos;  // sorted copies
    float4* svel;
    float4* dyn;   // density, P/rho^2, m/rho, P
    uint32_t* key;
    uint32_t* slot;
    uint32_t* perm;
    int32_t* nbid;
    int32_t* snbid;
    float* rec;    // kRecFloats per particle (record mode)
    // keys
    uint32_t* counts;
    uint32_t* offsets;
    uint32_t* chunk_sum;
    const uint32_t* tab;
    // terrain
    const float* tbase;
    long long* tdelta;
    float* theight;
    // in-range neighbour lists written by the density pass and read by the
    // force pass (variant bit 3), in traversal order.  Each work tile of T
    // particles starting at sorted index t owns kNbCap * T entries from
    // t * kNbCap on, slot-major: entry q of the tile's lane l at q * T + l,
    // so lanes at the same slot touch consecutive words and a tile's list
    // stays in one compact region.  ncnt[p] = in-range count (may exceed
    // kNbCap: that particle's force pass then walks the cells).
    uint32_t* nlist;
    int32_t* ncnt;
    // packed neighbour records (variant bit 7), two float4 per sorted
    // particle: (x, y, z, P/rho^2) and (vx, vy, vz, m/rho)
    float4* fdat;
    // status word: bit 0 = ordered-mode neighbour overflow, bit 1 =
    // inconsistent sort counts, bit 2 = a bounded wait of the TMA force
    // pipeline ran out
    unsigned* status;
    // work counters of the dynamically scheduled neighbour kernels
    // ([0] density, [1] force), cleared by the reorder kernel every step;
    // null where no kernel is scheduled that way
    unsigned* ctr;
    int tile;      // lanes per work tile (the list stride)
};

// Slots per particle of the in-range neighbour lists.
constexpr int kNbCap = 192;

struct LaunchShape {
    int tile;        // threads per particle tile
    int grid_p;      // persistent grid of particle kernels
    int grid_c;      // persistent grid of the scan
    int grid_t;      // persistent grid of the terrain kernel
    int variant;     // sph_system_config.variant bits (bit 3 only with lists allocated)
    int grid_dyn;    // grid of the dynamically scheduled neighbour kernels
    const void* fmap;  // host copy of the CUtensorMap over the packed records (null: none)
};

// Once per process and device: opt the list-traversal kernels into >48 KB of
// dynamic shared memory.
void configure_kernels();
void launch_keys(const DevArrays& a, const LaunchShape& s, cudaStream_t st);
void launch_scan(const DevArrays& a, const LaunchShape& s, cudaStream_t st);
void launch_scatter(const DevArrays& a, const LaunchShape& s, cudaStream_t st);
void launch_reorder(const DevArrays& a, const LaunchShape& s, cudaStream_t st);
void launch_density(const DevArrays& a, const LaunchShape& s, cudaStream_t st);
void launch_density_ordered(const DevArrays& a, const LaunchShape& s, cudaStream_t st);
void launch_force(const DevArrays& a, const LaunchShape& s, cudaStream_t st);
void launch_force_ordered(const DevArrays& a, const LaunchShape& s, cudaStream_t st);
void launch_terrain(const DevArrays& a, const LaunchShape& s, cudaStream_t st);
void launch_tick(const DevArrays& a, int nscenes, cudaStream_t st);

// Inspection and on-demand kernels.
void launch_neighbour_counts(const DevArrays& a, const LaunchShape& s, int32_t* out_by_id, cudaStream_t st);
// [rows visited, candidates tested, in-range pairs] of one scene's sorted state.
void launch_traversal_stats(const DevArrays& a, int scene, unsigned long long* out, cudaStream_t st);
// Scatter a scene's state into id order: any output may be null.
void launch_gather_by_id(const float4* pos, const float4* vel, const float4* dyn, int p_off, int n, float* pos3,
                         float* vel3, float* dens, int32_t* sed, cudaStream_t st);
// Per-scene FP64 partial sums: kDiagBlocks blocks per listed scene.
constexpr int kDiagBlocks = 32;
constexpr int kDiagDoubles = 8;  // mass-weighted momentum xyz, kinetic, potential, (pad)
void launch_diag(const DevArrays& a, int nlist, double* partial, long long* isums, int* nan_count,
                 cudaStream_t st);

}  // namespace sph
