/* sph_erosion.h - C ABI of the GB300 SPH-erosion simulation step.
 *
 * Every entry point returns an int status (SPH_OK = 0, negative on error);
 * sph_last_error() gives the message of the calling thread's last failure.
 * No C++ exception crosses this boundary and no device code traps.  Calls
 * on one system handle are not thread-safe; different handles are.
 *
 * A system owns one CUDA stream and the device memory of all of its scenes.
 * A scene is one independent fluid + terrain simulation (the state of one
 * reference FluidSystemSPH plus its Grid).  sph_system_step advances every
 * active scene of a system in one launch per stage.
 *
 * Each declaration names the reference interface it replaces
 * (Erosion/fluid_system.h and Erosion/grid.h of victor-kataev/SPH-Erosion).
 */
#ifndef SPH_EROSION_H
#define SPH_EROSION_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SPH_API __attribute__((visibility("default")))
#else
#define SPH_API
#endif

#define SPH_OK 0
#define SPH_ERR_INVALID (-1)   /* bad argument or handle */
#define SPH_ERR_CUDA (-2)      /* a CUDA call failed */
#define SPH_ERR_NOMEM (-3)     /* device or host allocation failed */
#define SPH_ERR_CAPACITY (-4)  /* request exceeds a configured capacity or budget */
#define SPH_ERR_STATE (-5)     /* call not valid in the current state */
#define SPH_ERR_DEVICE (-6)    /* a kernel reported an error status */

/* flags of sph_params.flags */
#define SPH_FLAG_RECORD 1  /* keep every FluidParticle field of the last step (GetParticle) */
#define SPH_FLAG_ORDERED 2 /* sum each particle's neighbours in ascending id order (validation) */

typedef struct sph_system sph_system;

/* Simulation parameters: the members of FluidSystemSPH
 * (Erosion/fluid_system.h:460-479) plus the box, grid and erosion settings
 * that the reference hard-codes or lacks. */
typedef struct sph_params {
    float gravity[3];       /* g */
    float dt;               /* deltaT; 0 = paused (fluid_system.h:342) */
    float rest_density;     /* p0 */
    float mass;             /* MASS */
    float viscosity;        /* visc */
    float surface_tension;  /* surf_tens */
    float gas_stiffness;    /* k */
    float restitution;      /* cR, used by the terrain contact */
    float smoothing_radius; /* h */
    float box_center[3];    /* the reference box is centred at 0 ... */
    float box_half[3];      /* ... with half extent len on every axis */
    float cell_mult;        /* uniform-grid cell edge / h, >= 0.25 (default 1) */
    int erosion;            /* 1 = exchange sediment with the terrain */
    float k_capacity;       /* carried volume fraction per m/s of speed */
    float k_pickup;         /* 1/s */
    float k_deposit;        /* 1/s */
    float erosion_layer;    /* contact layer above the surface, metres */
    int flags;              /* SPH_FLAG_* */
} sph_params;

/* One particle record, field for field the reference's FluidParticle
 * (Erosion/fluid_system.h:49-64), plus the carried sediment. */
typedef struct sph_particle {
    int id;
    float position[3];
    float velocity[3];
    float acceleration[3];
    float density;
    float pressure;
    float pressure_force[3];
    float viscosity_force[3];
    float gravity_force[3];
    float surface_force[3];
    float surface_normal[3];
    int neighb_id;
    int32_t sediment; /* fixed-point units, see sph_scene_diag */
} sph_particle;

/* FP64 diagnostics of one scene (the only FP64 on the device). */
typedef struct sph_diag {
    double fluid_mass;     /* n * mass */
    double momentum[3];    /* sum m v */
    double kinetic;        /* sum m |v|^2 / 2 */
    double potential;      /* sum -m (g . x) */
    int64_t sediment_units;  /* sum of carried sediment */
    int64_t terrain_units;   /* sum of terrain deltas */
    int64_t total_units;     /* sediment + terrain: conserved exactly */
    double unit_volume;      /* m^3 per unit */
    int32_t n;               /* particles */
    int32_t nan_particles;   /* particles with a non-finite position */
    uint64_t state_hash;     /* fingerprint of the particle state: the sum (mod 2^64) over
                                particles of a 64-bit mix (splitmix64 finaliser) of the id and
                                the bits of position, velocity and sediment; equal states give
                                equal fingerprints whatever their order in memory */
} sph_diag;

typedef struct sph_system_config {
    int device;               /* CUDA ordinal */
    int64_t particle_capacity; /* initial arena sizes; grown on demand */
    int64_t key_capacity;
    int64_t terrain_capacity;
    int max_scenes;
    int tile;                 /* particles per work tile: 128 or 256 (0 = 256) */
    int graph_steps;          /* steps per captured CUDA graph (0 = no graphs) */
    int variant;              /* kernel variant bits, picked by the autotuner:
                                 1 = density pass over compacted neighbour lists,
                                 4 = relaxed register budget (fewer resident blocks),
                                 8 = the density pass writes each particle's in-range
                                     neighbours (192 slots, 772 B per particle) and the
                                     force pass reads them instead of re-testing the
                                     cells; ignored when the HBM budget has no room,
                                16 = with 8: the force pass's list walk loads ahead,
                                32 = with 8: relaxed register budget of the density pass only,
                                64 = with 8: the density pass loads candidates in pairs,
                               128 = with 8: the force pass gathers one packed 32-byte
                                     record per neighbour (32 more bytes per particle),
                               256 = with 8: cooperative passes, a group of lanes per
                                     particle: the density pass sweeps the particle's
                                     candidates 32 at a time (2048: 16 lanes), the force
                                     pass splits its list over 8 lanes (512: 4, 1024: 16);
                                     with 256, bit 4 relaxes the force pass's registers,
                             32768 = with 8 + 16: the force pass's warps take their work
                                     in 32-particle slices from a counter instead of one
                                     block per tile (65536: the density pass's); same bits,
                            131072 = with 8 + 16: fast arithmetic in both neighbour passes
                                     (grouped products, fused multiply-adds, r^2 for
                                     |r|^2, hardware 1/sqrt); exact in-range test, so the
                                     neighbour sets and NeighbId are unchanged, but not
                                     the reference's rounding (within the 1e-4 bar),
                            262144 = with 8 + 16 + 128 + 131072: the force pass gathers the
                                     neighbours' packed records with TMA (tile::gather4) into
                                     a shared-memory ring fed by a producer warp; same bits
                                     as the other fast-arithmetic forms, slower (not tuned);
                                default 88 (8 + 16 + 64) */
    int64_t hbm_budget;       /* bytes this system may hold (0 = unlimited) */
} sph_system_config;

/* ---- errors and defaults ------------------------------------------------ */
SPH_API const char* sph_last_error(void);
/* Fills the reference's member defaults (fluid_system.h:460-479): g = (0,-9.82,0),
 * deltaT = 0, p0 = 998.29, MASS = 0.02, visc = 3.5, surf_tens = 0.0728, k = 3,
 * cR = 0.5, h = 0.0457, box = [-0.2, 0.2]^3; erosion off. */
SPH_API void sph_params_default(sph_params* p);
SPH_API void sph_system_config_default(sph_system_config* c);

/* ---- system --------------------------------------------------------------- */
SPH_API int sph_system_create(const sph_system_config* cfg, sph_system** out);
SPH_API int sph_system_destroy(sph_system* s);
/* Advance every active scene nsteps (FluidSystemSPH::Run, fluid_system.h:104-183,
 * once per step).  Enqueued on the system's stream; returns without waiting. */
SPH_API int sph_system_step(sph_system* s, int nsteps);
SPH_API int sph_system_sync(sph_system* s);  /* waits for steps and asynchronous readbacks */
/* Device time of nsteps steps measured with CUDA events on the system stream. */
SPH_API int sph_system_time_steps(sph_system* s, int nsteps, float* ms);
/* Device time per stage of one step, averaged over nsteps (stages: keys, scan,
 * scatter, reorder, density, force, terrain, tick); ms must hold 8 floats. */
SPH_API int sph_system_profile_stages(sph_system* s, int nsteps, float* ms);
/* Bytes of device memory the system holds. */
SPH_API int sph_system_memory(sph_system* s, int64_t* bytes);
/* With no live scene, return the arenas' memory and go back to the initial
 * capacities (arenas otherwise only grow); *trimmed = 0 when a scene is live.
 * No counterpart in the reference. */
SPH_API int sph_system_trim(sph_system* s, int* trimmed);

/* Autotuner (no counterpart in the reference).  Times `steps` steps of the
 * system's current scenes under each candidate of particles per work tile
 * (block size 128 or 256), grid cell edge (cell_mult 1 or 0.5, i.e. 27 cells
 * of h or 125 cells of h/2 around a particle) and kernel variant (density
 * pass direct or over compacted lists; neighbour lists handed from the
 * density to the force pass; high-occupancy or relaxed register budget of
 * the neighbour kernels), each trial starting from the same snapshot of
 * every scene's state, then keeps the fastest and restores the state.  One
 * particle per thread (32 per warp) and a re-sort every step are fixed: the
 * exact neighbour sets need the current sort.  In fast mode the cell size
 * changes the order in which neighbours are summed, hence the last bits of
 * the results (within the 1e-4 parity bar). */
typedef struct sph_tune_result {
    int tile;
    float cell_mult;
    int variant;
    float ms_per_step;
    int n_tried;
    int tiles[64];
    float cell_mults[64];
    int variants[64];
    float ms[64];
} sph_tune_result;
SPH_API int sph_system_autotune(sph_system* s, int steps, sph_tune_result* out);

/* ---- scenes (one FluidSystemSPH + Grid each) ------------------------------ */
/* FluidSystemSPH() (fluid_system.h:69-72): a scene with no particles.
 * terrain_w/terrain_d = 0 for no terrain; capacity is a hint. */
SPH_API int sph_scene_create(sph_system* s, const sph_params* p, int capacity, int terrain_w, int terrain_d,
                     int* scene);
SPH_API int sph_scene_destroy(sph_system* s, int scene);
/* Writes through GetMass/GetVisc/GetSurfTen/Getp0/GetGrav (fluid_system.h:261-284)
 * and SetDeltaTime (:216-219) become one parameter upload. */
SPH_API int sph_scene_set_params(sph_system* s, int scene, const sph_params* p);
SPH_API int sph_scene_get_params(sph_system* s, int scene, sph_params* p);
/* Steps the scene still takes in sph_system_step; -1 = unlimited (default). */
SPH_API int sph_scene_set_steps(sph_system* s, int scene, int steps);
SPH_API int sph_scene_get_steps(sph_system* s, int scene, int* steps);
/* Replace all particles: ids 0..n-1, zero sediment.  vel may be NULL. */
SPH_API int sph_scene_set_particles(sph_system* s, int scene, int n, const float* pos3, const float* vel3);
/* Initialize(n) / AddParticles(n) (fluid_system.h:74-102, :232-251): append a
 * ceil(cbrt(n))^3 lattice at spacing 0.025 from (-0.2,-0.05,-0.15)+origin. */
SPH_API int sph_scene_add_lattice(sph_system* s, int scene, int n, const float origin[3], int* added);
SPH_API int sph_scene_count(sph_system* s, int scene, int* n);
/* Positions, velocities, densities and sediment in id order (any may be NULL). */
SPH_API int sph_scene_get_particles(sph_system* s, int scene, float* pos3, float* vel3, float* density,
                            int32_t* sediment);
/* The same readback without waiting (no counterpart in the reference: the
 * front end's per-frame position readback, overlapped with the next steps).
 * It reads the state after all steps enqueued so far; the buffers are
 * complete once sph_system_sync returns and must not be touched before.  The
 * copies overlap later steps only when the buffers are pinned
 * (sph_host_alloc). */
SPH_API int sph_scene_get_particles_async(sph_system* s, int scene, float* pos3, float* vel3, float* density,
                                          int32_t* sediment);
/* Pinned (page-locked) host memory for the asynchronous readback. */
SPH_API int sph_host_alloc(int64_t bytes, void** out);
SPH_API int sph_host_free(void* p);
/* GetParticle(id) (fluid_system.h:286-289).  Force fields are filled when the
 * scene has SPH_FLAG_RECORD, zero otherwise. */
SPH_API int sph_scene_get_particle(sph_system* s, int scene, int id, sph_particle* out);
/* All records in id order (SPH_FLAG_RECORD): 27 floats each, laid out as
 * pos3 vel3 acc3 density pressure fpress3 fvisc3 fgrav3 fsurf3 normal3 pad. */
SPH_API int sph_scene_get_records(sph_system* s, int scene, float* rec27, int* neighb_id);
/* Diagnostics of a scene (no counterpart in the reference): FP64 momentum and
 * energies reduced on the device, the int64 sediment and terrain mass units
 * (their sum is conserved exactly), non-finite positions and the state
 * fingerprint (sph_diag). */
SPH_API int sph_scene_diag(sph_system* s, int scene, sph_diag* out);
/* The same for k scenes in one launch (k <= max_scenes): out[i] for scenes[i]. */
SPH_API int sph_scenes_diag(sph_system* s, int k, const int* scenes, sph_diag* out);

/* ---- terrain (Grid heightfield, grid.h:43-116) ---------------------------- */
/* LoadHeightfield generalised to any size and FP32 metres above the box floor
 * (grid.h:98-102); resets the int64 erosion deltas to zero.  w = d = 0
 * (heights may be NULL) removes the scene's terrain: the step then has no
 * terrain contact and no erosion, as the reference's step, which never reads
 * its Grid. */
SPH_API int sph_scene_set_terrain(sph_system* s, int scene, int w, int d, const float* heights);
/* Seeded fBm value noise (kind 0), ridged fBm (kind 1) or carved valleys
 * (kind 2: amplitude minus the ridged field, sharp valleys cut into a
 * plateau) of the given octaves, amplitude, lacunarity and gain (the
 * repository's own generator). */
SPH_API int sph_scene_gen_terrain(sph_system* s, int scene, uint64_t seed, int octaves, float amplitude,
                          float lacunarity, float gain, int kind);
/* LoadHeightfield (grid.h:98-102): the reference's 512 x 512 8-bit map,
 * x-major (map[512 * x + z]), becomes the scene's 512 x 512 FP32 terrain at
 * metres_per_level per grey level; deltas reset to zero. */
SPH_API int sph_scene_load_heightfield_u8(sph_system* s, int scene, const unsigned char* map512,
                                          float metres_per_level);
/* Current heights (base + delta) and the int64 deltas (either may be NULL). */
SPH_API int sph_scene_get_terrain(sph_system* s, int scene, float* heights, int64_t* delta);
SPH_API int sph_scene_terrain_dims(sph_system* s, int scene, int* w, int* d);
/* Grid::UpdateGrid + genIndices (grid.h:118-176) on the GPU for the
 * reference's 512 x 512 8-bit heightfield (x-major, map[512 * x + z]):
 * verts gets 6 floats (x, y, z, normal) per (x, z) for x < dimx, z < dimz
 * (z-major); indices gets 6 (dimx - 1)(dimz - 1) triangle corners.  Either
 * output may be NULL; *n_indices receives the index count. */
SPH_API int sph_terrain_mesh_u8(const unsigned char* map512, int dimx, int dimy, int dimz, float* verts,
                                unsigned* indices, int64_t index_cap, int64_t* n_indices);
/* The same surface mesh for a scene's current (eroded) heights, in world
 * units: tw * td vertices (x, y, z, normal), z-major, and
 * 6 (tw - 1)(td - 1) indices.  The front end's per-frame terrain redraw. */
SPH_API int sph_scene_terrain_mesh(sph_system* s, int scene, float* verts, unsigned* indices);
/* The same mesh in the units of the reference's Grid, for a front end that
 * draws the eroded terrain where Grid::UpdateGrid (grid.h:138-176) drew the
 * loaded one: vertex (x, H / metres_per_level, z) for vertex indices x < tw,
 * z < td (heights in grey levels, fractional once eroded), the normal the
 * normalised sum of the four cross products of its edge vectors in those
 * units; indices as genIndices (grid.h:118-136). */
SPH_API int sph_scene_terrain_mesh_levels(sph_system* s, int scene, float metres_per_level, float* verts,
                                          unsigned* indices);

/* Grid::collision (Erosion/grid.h:462-805) for n queries at once: the
 * contact of a particle moving from cur to next with velocity vel against
 * the two triangles of each cell of the 8-bit 512 x 512 height map
 * (map[512 * x + z], cell units), including the reference's adjacency walk
 * (findAdjacentCell, grid.h:210-269) and corner cases (grid.h:320-440).
 * Per query: hit 1/0, and on a hit the contact point and normal (zeros
 * otherwise), equal bit for bit to the reference's.  dimx/dimz are the
 * Grid's m_DimX/m_DimZ (2..512).  The reference compiles this routine but
 * never calls it (fluid_system.h:335-340).  Host arrays, 3 floats per query. */
SPH_API int sph_grid_collision_u8(const unsigned char* map512, int dimx, int dimz, int n, const float* cur3,
                                  const float* next3, const float* vel3, float* contact3, float* normal3,
                                  int32_t* hit);

/* ---- checkpoint / restore (no counterpart in the reference) ---------------
 * A scene's whole state in one little-endian binary file: "SPHE", version,
 * the sph_params block, counts, the particle records in device order
 * (position + id, velocity + sediment), NeighbId, step budget, terrain base
 * heights and int64 deltas.  Restoring into a scene (created with any
 * parameters; they are replaced) continues bit for bit like the original. */
SPH_API int sph_scene_save(sph_system* s, int scene, const char* path);
SPH_API int sph_scene_load(sph_system* s, int scene, const char* path);

/* ---- inspection for parity checks ---------------------------------------- */
/* Cell key of each particle and the stable sorted order (ids), as the next
 * step's sort computes them from the current positions. */
SPH_API int sph_scene_debug_sort(sph_system* s, int scene, uint32_t* keys_by_id, int32_t* sorted_ids);
/* In-range neighbour count (|x_i - x_j| <= h, j != i; fluid_system.h:139-142)
 * of each particle, in id order, from the uniform-grid traversal. */
SPH_API int sph_scene_neighbour_counts(sph_system* s, int scene, int32_t* counts_by_id);
/* Entries a neighbour list holds (self included); a particle with more
 * in-range neighbours walks the cells in the force pass instead. */
SPH_API int sph_neighbour_list_capacity(void);
/* Grid dims used by the sort: nx ny nz nkeys. */
SPH_API int sph_scene_grid_dims(sph_system* s, int scene, int* dims4);
/* Counters of the neighbour search the next step would run, from the current
 * positions: out4 = particles, cell rows visited, candidates tested, in-range
 * pairs (self included).  The reference tests n^2 pairs per pass. */
SPH_API int sph_scene_traversal_stats(sph_system* s, int scene, int64_t* out4);

/* ---- seeded scenes, batching and the request server -----------------------
 * No counterpart in the reference (a single interactive scene).  A request
 * describes one erosion scene: a dam-break block of `particles` lattice
 * particles at spacing h/2 placed from `seed` in a cube box, over a
 * `terrain_side`^2 fBm heightmap (6 octaves) seeded with `seed`, run for
 * `steps` steps. */
typedef struct sph_request {
    uint64_t seed;
    int32_t particles;
    int32_t terrain_side;
    int32_t steps;
    float coverage;  /* block volume / box volume above the terrain; 0 = from the seed, in [0.2, 0.5) */
    float amplitude; /* terrain amplitude / box side; 0 = from the seed, in [0.1, 0.4) */
    double arrival_s; /* arrival time in a replayed trace, seconds from the start */
} sph_request;

/* Create the scene a request describes in a system.  `base` gives the
 * physical constants (h, mass, ...); its box is replaced by the recipe's. */
SPH_API int sph_scene_from_request(sph_system* s, const sph_params* base, const sph_request* r, int* scene);

typedef struct sph_server sph_server;

typedef struct sph_server_config {
    int device;
    int tile;                     /* particles per work tile (0 = 256) */
    float cell_mult;              /* grid cell edge / h (0 = 0.5) */
    int chunk_steps;              /* steps per batched launch sequence (CUDA graph), 0 = 16 */
    int64_t hbm_budget;           /* bytes the server may hold (0 = 120 GiB) */
    int64_t max_active_particles; /* admission cap on resident particles (0 = none) */
    int max_scenes;               /* 0 = 4096 */
    sph_params base;              /* physical constants of every scene */
    int policy;                   /* admission order among arrived requests: 0 = arrival,
                                     1 = least work (particles x steps) first */
    int variant;                  /* kernel variant bits of the server's system (0 = the
                                     library default, 88); with a variant that rounds
                                     differently (fast arithmetic, cooperative passes) a
                                     request's result is the same alone and in a mix while
                                     the neighbour lists fit the budget */
} sph_server_config;

typedef struct sph_result {
    int64_t ticket;
    uint64_t seed;
    int32_t particles;
    int32_t steps;
    double arrival_s, admit_s, done_s; /* seconds from the server's start */
    int64_t total_units;               /* sediment + terrain change: 0 when mass is conserved */
    int64_t sediment_units;
    int32_t nan_particles;
    int32_t status;                    /* 0 when served; an error code (SPH_ERR_CAPACITY) when the
                                          request was refused at admission: its scene could not be
                                          created even with nothing else resident */
    double kinetic;
    uint64_t state_hash;               /* sph_diag.state_hash of the final state */
} sph_result;

typedef struct sph_server_stats {
    int64_t completed;
    double wall_s;           /* first arrival to last completion */
    double particle_steps;   /* sum of particles x steps completed */
    double throughput;       /* particle_steps / wall_s */
    double p50_s, p99_s, max_s; /* request latency: completion - arrival */
    int64_t peak_bytes;      /* largest device memory held */
    int32_t peak_active;     /* most scenes resident at once */
    int32_t chunks;          /* batched launch sequences run */
    int64_t peak_particles;  /* most particles resident at once */
    /* host wall time by phase of the serving loop (seconds): admission
     * (scene uploads), preparing queued requests' inputs while a chunk runs
     * on the GPU, waiting for the chunk, retirement (one diagnostic launch
     * for the finished scenes, then their ranges are freed) */
    double admit_s, prepare_s, gpu_wait_s, retire_s;
} sph_server_stats;

SPH_API void sph_server_config_default(sph_server_config* c);
SPH_API int sph_server_create(const sph_server_config* cfg, sph_server** out);
SPH_API int sph_server_destroy(sph_server* s);
/* Queue a request (its arrival_s is ignored: it arrives now).  A request
 * whose scene cannot fit the budget even alone is refused here with
 * SPH_ERR_CAPACITY. */
SPH_API int sph_server_submit(sph_server* s, const sph_request* r, int64_t* ticket);
/* Admit what fits, run one chunk of batched steps, retire finished scenes
 * and copy up to `cap` completed results out; *n_out = number copied,
 * *active = scenes still resident or queued. */
SPH_API int sph_server_poll(sph_server* s, sph_result* out, int cap, int* n_out, int* active);
/* Replay a trace in real time: request i arrives reqs[i].arrival_s seconds
 * after the call starts.  Returns when every request has completed; results
 * are in request order. */
SPH_API int sph_server_run_trace(sph_server* s, const sph_request* reqs, int n, sph_result* results,
                                 sph_server_stats* stats);

/* ---- allocation-free density pass ----------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory themselves or let a library do it: a host application that owns the
 * whole GPU through its own memory pool, a real-time loop that cannot take
 * cudaMalloc's implicit device synchronisation, or a plugin running where
 * allocation is not allowed.  Computes the reference's pass 1 (density and
 * pressure of every particle, fluid_system.h:107-124; no motion) for n
 * particles given as 3n floats in DEVICE memory, writing n densities (and,
 * if pressure_dev is not NULL, n pressures) to DEVICE memory in input order.
 * It runs the same sort and density kernels as a scene step, on `stream`
 * (a cudaStream_t; NULL = the legacy default stream), and returns after the
 * stream has drained.  It allocates nothing: its scratch is one fixed device
 * array of SPH_STATIC_SCRATCH_BYTES that every GPU loading the library holds
 * until the process exits.  Limits: n <= SPH_STATIC_MAX_PARTICLES and a
 * uniform grid of at most SPH_STATIC_MAX_KEYS keys; larger requests return
 * SPH_ERR_CAPACITY; parameters are checked as by sph_scene_create.  The
 * first call on a device resolves the array's device address with that
 * device current.  Every call synchronises its stream before returning, so
 * it must not be called on a stream that is being captured into a CUDA
 * graph: such a call returns SPH_ERR_INVALID without touching the stream.
 * All calls share the array: calls whose work overlaps on the GPU (other
 * streams or host threads) race and must be serialised by the caller. */
#define SPH_STATIC_MAX_PARTICLES 32768
#define SPH_STATIC_MAX_KEYS 262144
#define SPH_STATIC_MAX_TABLE 262144 /* row numbers: ny * nz <= SPH_STATIC_MAX_KEYS */
#define SPH_STATIC_SCRATCH_BYTES 6163200
SPH_API int sph_density_static(const sph_params* p, int n, const float* pos3_dev, float* density_dev,
                               float* pressure_dev, void* stream);

#ifdef __cplusplus
}
#endif
#endif
