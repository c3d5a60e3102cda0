// Host engine of the simulation step: device arenas, scenes, work lists,
// step orchestration and CUDA-graph capture.  Internal to libsph_gb300.so;
// the public surface is include/sph_erosion.h.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sph_erosion.h"
#include "sph_kernels.h"
#include "sph_types.h"

#include <nvtx3/nvToolsExt.h>

namespace sph {

// NVTX range for profilers (ncu --nvtx): stage names of the step, autotuner,
// readbacks and server rounds.  Costs a pointer test without a tool attached.
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void check_cuda(cudaError_t e, const char* what);
#define SPH_CK(x) ::sph::check_cuda((x), #x)

// First-fit allocator of index ranges inside one arena.
class RangeAlloc {
   public:
    void reset(int64_t cap);
    bool alloc(int64_t len, int64_t* off);  // len already rounded by the caller
    void release(int64_t off, int64_t len);
    void grow(int64_t cap);
    int64_t cap() const { return cap_; }
    int64_t used() const { return used_; }

   private:
    std::map<int64_t, int64_t> free_;  // offset -> length
    int64_t cap_ = 0;
    int64_t used_ = 0;
};

// A typed device buffer that can grow while keeping its contents.
template <class T>
struct DevBuf {
    T* p = nullptr;
    int64_t n = 0;
    void resize(int64_t cnt, bool keep, cudaStream_t st);
    void release();
    int64_t bytes() const { return n * (int64_t)sizeof(T); }
};

struct Scene {
    bool live = false;
    sph_params prm{};
    int n = 0;
    int p_cap = 0;
    int64_t p_off = 0;
    int nx = 1, ny = 1, nz = 1, reach = 1, xsub = 1;
    int nkeys = 0, k_cap = 0, nchunks = 0;
    int64_t k_off = 0, c_off = 0, tab_off = 0;
    int tab_len = 0;
    float cell = 0.f, inv_cell = 0.f, lo[3] = {0, 0, 0};
    int tw = 0, td = 0;
    int64_t t_off = 0;
    int steps = -1;  // -1 unlimited, 0 inactive
    SceneDev dev{};
};

// The checks every entry point applies to a parameter block: finite
// positive smoothing radius and box half extents, cell_mult in [0.25, 8].
void validate_params(const sph_params& p);

class System {
   public:
    explicit System(const sph_system_config& cfg);
    ~System();

    int create_scene(const sph_params& p, int capacity, int tw, int td);
    void destroy_scene(int id);
    void set_params(int id, const sph_params& p);
    const sph_params& params(int id) const { return scene(id).prm; }
    void set_steps(int id, int steps);
    int steps(int id) const { return scene(id).steps; }
    void set_particles(int id, int n, const float* pos3, const float* vel3);
    int add_lattice(int id, int n, const float origin[3]);
    int count(int id) const { return scene(id).n; }
    void get_particles(int id, float* pos3, float* vel3, float* density, int32_t* sed);
    void get_particles_async(int id, float* pos3, float* vel3, float* density, int32_t* sed);
    void get_records(int id, float* rec27, int* nbid, int32_t* sed);
    void diag(int id, sph_diag* out);
    void diag_many(const int* ids, int k, sph_diag* out);
    void set_terrain(int id, int w, int d, const float* heights);
    void gen_terrain(int id, uint64_t seed, int octaves, float amp, float lac, float gain, int kind);
    void get_terrain(int id, float* heights, int64_t* delta);
    void terrain_dims(int id, int* w, int* d) const;
    void debug_sort(int id, uint32_t* keys_by_id, int32_t* sorted_ids);
    void neighbour_counts(int id, int32_t* out);
    void traversal_stats(int id, int64_t* out4);
    void save(int id, const char* path);
    void load(int id, const char* path);
    void load_heightfield_u8(int id, const unsigned char* map512, float metres_per_level);
    void grid_dims(int id, int* dims4) const;

    void step(int nsteps);
    void sync();
    bool trim();  // with no live scene: back to the initial arena sizes
    void autotune(int steps, sph_tune_result* out);
    float time_steps(int nsteps);
    void profile_stages(int nsteps, float* ms);
    int64_t memory_bytes() const;
    int num_scenes() const { return (int)scenes_.size(); }
    bool scene_live(int id) const { return id >= 0 && id < (int)scenes_.size() && scenes_[id].live; }
    // Arena bytes of a scene; `lists`: with the optional neighbour lists.
    int64_t scene_bytes(int n, int tw, int td, const sph_params& p, bool lists = true) const;
    cudaStream_t stream() const { return st_; }
    unsigned read_status();
    void check_status();

    // Uniform grid and device descriptor of a scene; they depend on the
    // scene's parameters and ranges only.
    static void geometry(Scene& sc);
    static void fill_dev(Scene& sc);

   private:
    Scene& scene(int id);
    const Scene& scene(int id) const;
    void upload_scene(int id);
    void ensure_particle_cap(Scene& sc, int need);
    void ensure_arena(RangeAlloc& ra, int64_t need, int which);
    void grow_particles(int64_t cap);
    void grow_keys(int64_t cap);
    void grow_terrain(int64_t cap);
    void grow_tables(int64_t cap);
    void grow_chunks(int64_t cap);
    void rebuild_work();
    void ensure_nlist();
    void initial_arenas();
    DevArrays arrays() const;
    LaunchShape shape() const;
    void enqueue_step(const DevArrays& a, const LaunchShape& s, cudaEvent_t* ev);
    void enqueue_sort(const DevArrays& a, const LaunchShape& s);
    void capture_graph();
    void advance_step_mirror(int nsteps);
    void drop_graph();
    void check_budget(int64_t extra) const;
    void upload_terrain_height(Scene& sc);

    sph_system_config cfg_;
    // scene-descriptor uploads from a ring of pinned slots (a slot is reused
    // once the copy that read it has run), so set_params never waits for the
    // stream
    static constexpr int kUploadRing = 64;
    SceneDev* up_dev_ = nullptr;  // pinned, kUploadRing entries
    int* up_steps_ = nullptr;     // pinned, kUploadRing entries
    cudaEvent_t up_ev_[kUploadRing] = {};
    int up_next_ = 0;
    // asynchronous readback: gathers on st_ into one of two staging buffers,
    // device-to-host copies on cst_
    cudaStream_t cst_ = nullptr;
    cudaEvent_t gathered_[2] = {nullptr, nullptr}, copied_[2] = {nullptr, nullptr};
    DevBuf<float> astage_[2];
    int aslot_ = 0;
    int dev_ = 0, nsm_ = 1;
    cudaStream_t st_ = nullptr;
    std::vector<Scene> scenes_;

    RangeAlloc pa_, ka_, ca_, ta_, tba_;
    // particle arena
    DevBuf<float4> pos_, vel_, spos_, svel_, dyn_;
    DevBuf<uint32_t> key_, slot_, perm_;
    DevBuf<int32_t> nbid_, snbid_;
    DevBuf<float> rec_;
    DevBuf<uint32_t> nlist_;  // kNbCap slots per arena particle (variant bit 3)
    DevBuf<int32_t> ncnt_;
    DevBuf<float4> fdat_;     // 2 per arena particle (variant bit 7)
    bool nl_ready_ = false;
    // TMA map over fdat_ (one 32-byte row per particle) for the force
    // pass's gather pipeline (variant bit 18); valid while fmap_ok_
    CUtensorMap fmap_;
    bool fmap_ok_ = false;
    const float4* fmap_base_ = nullptr;
    int64_t fmap_rows_ = 0;
    void ensure_fmap();
    // key arena
    DevBuf<uint32_t> counts_, offsets_;
    DevBuf<uint32_t> chunk_;
    DevBuf<uint32_t> tab_;
    // terrain arena
    DevBuf<float> tbase_, theight_;
    DevBuf<long long> tdelta_;
    // tables and work lists
    DevBuf<SceneDev> dscenes_;
    DevBuf<int> steps_;
    DevBuf<Work> ptiles_, ctiles_, ttiles_;
    DevBuf<int> nwork_;    // [0] particle tiles, [1] chunks, [2] terrain tiles
    DevBuf<int> slist_;
    DevBuf<unsigned> status_;
    DevBuf<int32_t> scratch_i_;
    DevBuf<float> stage_;  // id-order readback staging (8 floats per particle)
    DevBuf<double> diag_part_;
    DevBuf<long long> diag_i_;
    DevBuf<int> diag_nan_;

    int n_ptiles_ = 0, n_ctiles_ = 0, n_ttiles_ = 0;
    bool any_fast_ = false, any_ordered_ = false, any_terrain_ = false, any_limited_ = false,
         any_record_ = false;
    bool work_dirty_ = true;

    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t gexec_ = nullptr;
    bool graph_dirty_ = true;
};

// Host implementation of the seeded fBm generator (sph_terrain.cpp).
void fbm_heights(uint64_t seed, int w, int d, int octaves, float amplitude, float lacunarity, float gain,
                 int kind, float* out, int max_threads = 0);

// Sets the calling thread's sph_last_error() message (sph_capi.cu).
void set_last_error(const std::string& msg);
// Morton-ordered dense row numbers of an ny x nz grid of cell rows:
// tab[z * ny + y] for row (y, z).
void row_table(int ny, int nz, uint32_t* tab);

// Terrain meshes (sph_mesh.cu).
void mesh_u8(const unsigned char* map_host, int dimx, int dimy, int dimz, float* verts, unsigned* idx,
             int64_t idx_cap, int64_t* n_idx);
void mesh_scene(System& sys, int scene, float* verts, unsigned* idx);
int scene_from_request(System& sys, const sph_params& base, const sph_request& r);

}  // namespace sph

// The opaque handle of include/sph_erosion.h.
struct sph_system {
    sph::System* sys;
};

namespace sph {

// Host FP32 constants of a scene (sph_engine.cu): exposed for inspection.
float smax_for(float h);
float coincidence_threshold();

}  // namespace sph
