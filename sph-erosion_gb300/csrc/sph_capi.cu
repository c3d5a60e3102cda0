// extern "C" surface of libsph_gb300.so (declared in include/sph_erosion.h).
// Every entry point catches all C++ exceptions and turns them into a status
// code plus a thread-local message.
#include <cstring>
#include <new>
#include <string>

#include "../../include/sph_erosion.h"
#include "sph_engine.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

template <class F>
int guard(F&& f) {
    try {
        f();
        return SPH_OK;
    } catch (const sph::Error& e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(SPH_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(SPH_ERR_INVALID, e.what());
    } catch (...) {
        return fail(SPH_ERR_INVALID, "unknown error");
    }
}

sph::System& sys(sph_system* s) {
    if (!s || !s->sys) throw sph::Error(SPH_ERR_INVALID, "null system handle");
    return *s->sys;
}

void need(const void* p, const char* what) {
    if (!p) throw sph::Error(SPH_ERR_INVALID, std::string("null ") + what);
}

}  // namespace

extern "C" {

const char* sph_last_error(void) { return g_err.c_str(); }

void sph_params_default(sph_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->gravity[0] = 0.0f;
    p->gravity[1] = -9.82f;
    p->gravity[2] = 0.0f;
    p->dt = 0.0f;
    p->rest_density = 998.29f;
    p->mass = 0.02f;
    p->viscosity = 3.5f;
    p->surface_tension = 0.0728f;
    p->gas_stiffness = 3.0f;
    p->restitution = 0.5f;
    p->smoothing_radius = 0.0457f;
    for (int a = 0; a < 3; ++a) {
        p->box_center[a] = 0.0f;
        p->box_half[a] = 0.2f;
    }
    p->cell_mult = 1.0f;
    p->erosion = 0;
    p->k_capacity = 0.01f;
    p->k_pickup = 5.0f;
    p->k_deposit = 2.0f;
    p->erosion_layer = 0.0457f;
    p->flags = 0;
}

void sph_system_config_default(sph_system_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->device = 0;
    c->particle_capacity = 1 << 16;
    c->key_capacity = 1 << 16;
    c->terrain_capacity = 1 << 12;
    c->max_scenes = 1024;
    c->tile = 256;
    c->graph_steps = 16;
    c->variant = 88;  // neighbour lists, pipelined list walk, paired candidate loads
    c->hbm_budget = 0;
}

int sph_system_create(const sph_system_config* cfg, sph_system** out) {
    return guard([&] {
        need(out, "output handle");
        *out = nullptr;
        sph_system_config c;
        if (cfg)
            c = *cfg;
        else
            sph_system_config_default(&c);
        sph::System* s = new sph::System(c);
        *out = new sph_system{s};
    });
}

int sph_system_destroy(sph_system* s) {
    return guard([&] {
        if (!s) return;
        delete s->sys;
        s->sys = nullptr;
        delete s;
    });
}

int sph_system_step(sph_system* s, int nsteps) { return guard([&] { sys(s).step(nsteps); }); }
int sph_system_sync(sph_system* s) { return guard([&] { sys(s).sync(); }); }

int sph_system_time_steps(sph_system* s, int nsteps, float* ms) {
    return guard([&] {
        need(ms, "ms");
        *ms = sys(s).time_steps(nsteps);
    });
}

int sph_system_profile_stages(sph_system* s, int nsteps, float* ms) {
    return guard([&] {
        need(ms, "ms");
        sys(s).profile_stages(nsteps, ms);
    });
}

int sph_scene_save(sph_system* s, int scene, const char* path) {
    return guard([&] { sys(s).save(scene, path); });
}

int sph_scene_load(sph_system* s, int scene, const char* path) {
    return guard([&] { sys(s).load(scene, path); });
}

int sph_scene_load_heightfield_u8(sph_system* s, int scene, const unsigned char* map512, float metres_per_level) {
    return guard([&] { sys(s).load_heightfield_u8(scene, map512, metres_per_level); });
}

int sph_scene_traversal_stats(sph_system* s, int scene, int64_t* out4) {
    return guard([&] {
        need(out4, "out4");
        sys(s).traversal_stats(scene, out4);
    });
}

int sph_system_autotune(sph_system* s, int steps, sph_tune_result* out) {
    return guard([&] {
        need(out, "out");
        sys(s).autotune(steps, out);
    });
}

int sph_system_memory(sph_system* s, int64_t* bytes) {
    return guard([&] {
        need(bytes, "bytes");
        *bytes = sys(s).memory_bytes();
    });
}

int sph_system_trim(sph_system* s, int* trimmed) {
    return guard([&] {
        const bool t = sys(s).trim();
        if (trimmed) *trimmed = t ? 1 : 0;
    });
}

int sph_scene_create(sph_system* s, const sph_params* p, int capacity, int terrain_w, int terrain_d, int* scene) {
    return guard([&] {
        need(p, "params");
        need(scene, "scene");
        *scene = sys(s).create_scene(*p, capacity, terrain_w, terrain_d);
    });
}

int sph_scene_destroy(sph_system* s, int scene) { return guard([&] { sys(s).destroy_scene(scene); }); }

int sph_scene_set_params(sph_system* s, int scene, const sph_params* p) {
    return guard([&] {
        need(p, "params");
        sys(s).set_params(scene, *p);
    });
}

int sph_scene_get_params(sph_system* s, int scene, sph_params* p) {
    return guard([&] {
        need(p, "params");
        *p = sys(s).params(scene);
    });
}

int sph_scene_set_steps(sph_system* s, int scene, int steps) { return guard([&] { sys(s).set_steps(scene, steps); }); }

int sph_scene_get_steps(sph_system* s, int scene, int* steps) {
    return guard([&] {
        need(steps, "steps");
        *steps = sys(s).steps(scene);
    });
}

int sph_scene_set_particles(sph_system* s, int scene, int n, const float* pos3, const float* vel3) {
    return guard([&] { sys(s).set_particles(scene, n, pos3, vel3); });
}

int sph_scene_add_lattice(sph_system* s, int scene, int n, const float origin[3], int* added) {
    return guard([&] {
        const float zero[3] = {0.f, 0.f, 0.f};
        const int a = sys(s).add_lattice(scene, n, origin ? origin : zero);
        if (added) *added = a;
    });
}

int sph_scene_count(sph_system* s, int scene, int* n) {
    return guard([&] {
        need(n, "n");
        *n = sys(s).count(scene);
    });
}

int sph_scene_get_particles(sph_system* s, int scene, float* pos3, float* vel3, float* density, int32_t* sediment) {
    return guard([&] { sys(s).get_particles(scene, pos3, vel3, density, sediment); });
}

int sph_scene_get_particles_async(sph_system* s, int scene, float* pos3, float* vel3, float* density,
                                  int32_t* sediment) {
    return guard([&] { sys(s).get_particles_async(scene, pos3, vel3, density, sediment); });
}

int sph_host_alloc(int64_t bytes, void** out) {
    return guard([&] {
        need(out, "out");
        *out = nullptr;
        if (bytes <= 0) throw sph::Error(SPH_ERR_INVALID, "bytes must be positive");
        sph::check_cuda(cudaMallocHost(out, (size_t)bytes), "cudaMallocHost");
    });
}

int sph_host_free(void* p) {
    return guard([&] {
        if (p) sph::check_cuda(cudaFreeHost(p), "cudaFreeHost");
    });
}

int sph_scene_get_particle(sph_system* s, int scene, int id, sph_particle* out) {
    return guard([&] {
        need(out, "out");
        sph::System& S = sys(s);
        const int n = S.count(scene);
        if (id < 0 || id >= n) throw sph::Error(SPH_ERR_INVALID, "particle id out of range");
        std::string buf;
        std::vector<float> rec((size_t)n * 27);
        std::vector<int> nb(n);
        std::vector<int32_t> sed(n);
        S.get_records(scene, rec.data(), nb.data(), sed.data());
        const float* r = rec.data() + (size_t)27 * id;
        std::memset(out, 0, sizeof *out);
        out->id = id;
        for (int a = 0; a < 3; ++a) {
            out->position[a] = r[a];
            out->velocity[a] = r[3 + a];
            out->acceleration[a] = r[6 + a];
            out->pressure_force[a] = r[11 + a];
            out->viscosity_force[a] = r[14 + a];
            out->gravity_force[a] = r[17 + a];
            out->surface_force[a] = r[20 + a];
            out->surface_normal[a] = r[23 + a];
        }
        out->density = r[9];
        out->pressure = r[10];
        out->neighb_id = nb[id];
        out->sediment = sed[id];
    });
}

int sph_scene_get_records(sph_system* s, int scene, float* rec27, int* neighb_id) {
    return guard([&] { sys(s).get_records(scene, rec27, neighb_id, nullptr); });
}

int sph_scene_diag(sph_system* s, int scene, sph_diag* out) {
    return guard([&] {
        need(out, "out");
        sys(s).diag(scene, out);
    });
}

int sph_scenes_diag(sph_system* s, int k, const int* scenes, sph_diag* out) {
    return guard([&] {
        if (k < 0) throw sph::Error(SPH_ERR_INVALID, "negative scene count");
        if (k == 0) return;
        need(scenes, "scenes");
        need(out, "out");
        sys(s).diag_many(scenes, k, out);
    });
}

int sph_scene_set_terrain(sph_system* s, int scene, int w, int d, const float* heights) {
    return guard([&] { sys(s).set_terrain(scene, w, d, heights); });
}

int sph_scene_gen_terrain(sph_system* s, int scene, uint64_t seed, int octaves, float amplitude, float lacunarity,
                          float gain, int kind) {
    return guard([&] {
        if (octaves < 1 || octaves > 16) throw sph::Error(SPH_ERR_INVALID, "octaves must be in [1, 16]");
        if (kind < 0 || kind > 2) throw sph::Error(SPH_ERR_INVALID, "kind must be 0, 1 or 2");
        sys(s).gen_terrain(scene, seed, octaves, amplitude, lacunarity, gain, kind);
    });
}

int sph_scene_get_terrain(sph_system* s, int scene, float* heights, int64_t* delta) {
    return guard([&] { sys(s).get_terrain(scene, heights, delta); });
}

int sph_scene_terrain_dims(sph_system* s, int scene, int* w, int* d) {
    return guard([&] {
        need(w, "w");
        need(d, "d");
        sys(s).terrain_dims(scene, w, d);
    });
}

int sph_scene_debug_sort(sph_system* s, int scene, uint32_t* keys_by_id, int32_t* sorted_ids) {
    return guard([&] { sys(s).debug_sort(scene, keys_by_id, sorted_ids); });
}

int sph_scene_neighbour_counts(sph_system* s, int scene, int32_t* counts_by_id) {
    return guard([&] {
        need(counts_by_id, "counts");
        sys(s).neighbour_counts(scene, counts_by_id);
    });
}

int sph_neighbour_list_capacity(void) { return sph::kNbCap; }

int sph_scene_grid_dims(sph_system* s, int scene, int* dims4) {
    return guard([&] {
        need(dims4, "dims");
        sys(s).grid_dims(scene, dims4);
    });
}

}  // extern "C"

namespace sph {
// Lets other translation units report through sph_last_error().
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace sph
