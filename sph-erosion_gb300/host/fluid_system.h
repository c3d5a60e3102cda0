// Drop-in FluidSystemSPH for the reference's front end
// (Erosion/fluid_system.h:66-485), backed by libsph_gb300.so.
//
// Same class, record type and public methods, with the reference's
// semantics: Initialize and AddParticles append a ceil(cbrt(n))^3 lattice at
// spacing 0.025 from (-0.2, -0.05, -0.15) + origin (fluid_system.h:74-102,
// :232-251); Reset re-adds the initial count (:253-259); the Get* pointer
// getters return host members that the next Run uploads, so the ImGui panel's
// live edits (Erosion/main.cpp:278-290) take effect as in the reference; a
// deltaT of 0 pauses the motion (:342).  Run advances one step on the GPU;
// GetParticle returns every FluidParticle field of the last step.  Draw (an
// OpenGL call per particle) is replaced by GetPositions, a host copy of the
// positions for the front end's own instanced draw.
//
// Terrain and erosion (no counterpart in the reference, whose Run never
// reads its Grid): SetTerrain(true) makes Run take the Grid's heightfield,
// the dimX x dimZ block that Grid::UpdateGrid meshes, spread over the box
// floor at metres_per_level per grey level, as the step's terrain (contact
// with the surface); SetErosion(true) also exchanges sediment with it.  Run
// re-uploads the heightfield whenever the Grid's heightfield or dimensions
// change (resetting the erosion), and the Grid then shows the eroded surface
// from UpdateGrid / GetSurfaceParts.  GetDiagnostics reads the FP64 totals
// and the exact sediment + terrain units.
#pragma once
#include <cmath>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "grid.h"
#include "sph_erosion.h"
#include "sph_vec3.h"

struct FluidParticle {
    int Id;
    sph_shim::vec3 Position;
    sph_shim::vec3 Velocity;
    sph_shim::vec3 Acceleration;
    float Density;
    float Pressure;
    sph_shim::vec3 PressureForce;
    sph_shim::vec3 ViscosityForce;
    sph_shim::vec3 GravityForce;
    sph_shim::vec3 SurfaceForce;
    sph_shim::vec3 SurfaceNormal;
    int NeighbId;
};

class FluidSystemSPH {
   public:
    // flags: SPH_FLAG_RECORD keeps every field for GetParticle (the
    // reference's behaviour); add SPH_FLAG_ORDERED to sum neighbours in the
    // reference's order (bit-exact arithmetic, slower).
    explicit FluidSystemSPH(int flags = SPH_FLAG_RECORD) : m_Origin(0.0f, 0.0f, 0.0f), m_flags(flags) {
        sph_system_config cfg;
        sph_system_config_default(&cfg);
        cfg.particle_capacity = 4096;
        cfg.key_capacity = 1 << 16;
        cfg.graph_steps = 0;  // one step per Run
        check(sph_system_create(&cfg, &m_sys));
        sph_params p = params();
        check(sph_scene_create(m_sys, &p, 1024, 0, 0, &m_scene));
    }
    ~FluidSystemSPH() {
        if (m_link) m_link->sys = nullptr;
        if (m_sys) sph_system_destroy(m_sys);
    }
    FluidSystemSPH(const FluidSystemSPH&) = delete;
    FluidSystemSPH& operator=(const FluidSystemSPH&) = delete;

    void Initialize(int nParts) {
        num = nParts;
        init_num = nParts;
        id = 0;
        append_lattice(nParts);
        smoothRadius = h;
    }

    // One simulation step (fluid_system.h:104-183).  With the terrain off
    // (the default) the grid is not read, exactly as in the reference; with
    // it on, the grid's heightfield is the step's terrain.
    void Run(Grid& grid) {
        if (m_terrain && (m_grid_seen != &grid || m_version_seen != grid.HeightfieldVersion())) upload_terrain(grid);
        sph_params p = params();
        check(sph_scene_set_params(m_sys, m_scene, &p));
        check(sph_system_step(m_sys, 1));
    }

    // Terrain contact against the Grid's heightfield from the next Run on;
    // metres_per_level <= 0 keeps the last scale (initially len / 255: the
    // highest grey level reaches half the box's height).  Off removes the
    // terrain (and stops erosion).
    void SetTerrain(bool on, float metres_per_level = 0.0f) {
        if (metres_per_level > 0.0f && metres_per_level != m_mpl) {
            m_mpl = metres_per_level;
            m_grid_seen = nullptr;  // re-upload at the new scale
        }
        if (!on && m_terrain) {
            check(sph_scene_set_terrain(m_sys, m_scene, 0, 0, nullptr));
            if (m_link) m_link->sys = nullptr;
            m_link.reset();
            m_grid_seen = nullptr;
            m_erosion = false;
        }
        m_terrain = on;
    }

    // Sediment exchange with the terrain (turns the terrain on): capacity
    // per m/s of speed, pickup and deposition rates (1/s) and the contact
    // layer above the surface (<= 0: the smoothing radius).
    void SetErosion(bool on, float k_capacity = 0.01f, float k_pickup = 5.0f, float k_deposit = 2.0f,
                    float layer = 0.0f) {
        if (on) SetTerrain(true);
        m_erosion = on;
        m_k_capacity = k_capacity;
        m_k_pickup = k_pickup;
        m_k_deposit = k_deposit;
        m_layer = layer;
    }

    sph_diag GetDiagnostics() {
        sph_diag d;
        check(sph_scene_diag(m_sys, m_scene, &d));
        return d;
    }

    std::vector<float> GetPositions() {
        int n = 0;
        check(sph_scene_count(m_sys, m_scene, &n));
        std::vector<float> pos((size_t)n * 3);
        if (n) check(sph_scene_get_particles(m_sys, m_scene, pos.data(), nullptr, nullptr, nullptr));
        return pos;
    }

    void SetOrigin(const sph_shim::vec3& o) { m_Origin = o; }
    sph_shim::vec3 GetOrigin() const { return m_Origin; }
    void SetDeltaTime(float dt) { deltaT = dt; }
    float GetDeltaTime() const { return deltaT; }

    void PrintCoords() const {
        const std::vector<float> pos = const_cast<FluidSystemSPH*>(this)->GetPositions();
        for (int i = 0; i < num && 3 * (size_t)i + 2 < pos.size(); i++)
            std::cout << "[" << i << "] " << pos[3 * i] << ' ' << pos[3 * i + 1] << ' ' << pos[3 * i + 2] << std::endl;
    }

    void AddParticles(int n) {
        append_lattice(n);
        num += n;
    }

    void Reset() {
        check(sph_scene_set_particles(m_sys, m_scene, 0, nullptr, nullptr));
        num = 0;
        id = 0;
        AddParticles(init_num);
    }

    float* GetMass() { return &MASS; }
    float* GetVisc() { return &visc; }
    float* GetSurfTen() { return &surf_tens; }
    float* Getp0() { return &p0; }
    sph_shim::vec3* GetGrav() { return &g; }

    FluidParticle GetParticle(int pid) {
        sph_particle r;
        check(sph_scene_get_particle(m_sys, m_scene, pid, &r));
        FluidParticle f;
        f.Id = r.id;
        auto v = [](const float* a) { return sph_shim::vec3(a[0], a[1], a[2]); };
        f.Position = v(r.position);
        f.Velocity = v(r.velocity);
        f.Acceleration = v(r.acceleration);
        f.Density = r.density;
        f.Pressure = r.pressure;
        f.PressureForce = v(r.pressure_force);
        f.ViscosityForce = v(r.viscosity_force);
        f.GravityForce = v(r.gravity_force);
        f.SurfaceForce = v(r.surface_force);
        f.SurfaceNormal = v(r.surface_normal);
        f.NeighbId = r.neighb_id;
        return f;
    }

    // Parameters without a setter in the reference (h, k, len): settable here.
    void SetSmoothingRadius(float v) { h = smoothRadius = v; }
    void SetGasStiffness(float v) { k = v; }
    void SetBoxHalf(float v) { len = v; }

   private:
    static void check(int rc) {
        if (rc != SPH_OK) throw std::runtime_error(std::string("sph: ") + sph_last_error());
    }

    sph_params params() const {
        sph_params p;
        sph_params_default(&p);
        p.gravity[0] = g[0];
        p.gravity[1] = g[1];
        p.gravity[2] = g[2];
        p.dt = deltaT;
        p.rest_density = p0;
        p.mass = MASS;
        p.viscosity = visc;
        p.surface_tension = surf_tens;
        p.gas_stiffness = k;
        p.restitution = cR;
        p.smoothing_radius = h;
        for (int a = 0; a < 3; ++a) p.box_half[a] = len;
        p.flags = m_flags;
        p.erosion = m_erosion ? 1 : 0;
        p.k_capacity = m_k_capacity;
        p.k_pickup = m_k_pickup;
        p.k_deposit = m_k_deposit;
        p.erosion_layer = m_layer > 0.0f ? m_layer : h;
        return p;
    }

    void upload_terrain(Grid& grid) {
        const int w = grid.DimX(), d = grid.DimZ();
        if (w < 2 || d < 2 || w > 512 || d > 512)
            throw std::runtime_error("sph: the grid's dimX and dimZ must be in [2, 512] for terrain contact");
        const float mpl = m_mpl > 0.0f ? m_mpl : len / 255.0f;
        const std::vector<float> hts = grid.BlockHeights(mpl);
        check(sph_scene_set_terrain(m_sys, m_scene, w, d, hts.data()));
        if (m_link) m_link->sys = nullptr;
        m_link = std::make_shared<sph_terrain_link>();
        m_link->sys = m_sys;
        m_link->scene = m_scene;
        m_link->metres_per_level = mpl;
        m_link->dimx = w;
        m_link->dimz = d;
        m_link->version = grid.HeightfieldVersion();
        grid.Link(m_link);
        m_grid_seen = &grid;
        m_version_seen = grid.HeightfieldVersion();
    }

    void append_lattice(int n) {
        const float o[3] = {m_Origin[0], m_Origin[1], m_Origin[2]};
        int added = 0;
        check(sph_scene_add_lattice(m_sys, m_scene, n, o, &added));
        id += added;
    }

    // the reference's members and defaults (fluid_system.h:460-479)
    sph_shim::vec3 g = sph_shim::vec3(0.0f, -9.82f, 0.0f);
    float deltaT = 0.0f;
    float p0 = 998.29f;
    float MASS = 0.02f;
    float visc = 3.5f;
    float surf_tens = 0.0728f;
    float k = 3.0f;
    float cR = 0.5f;
    float h = 0.0457f;
    int num = 10;
    int init_num = 0;
    float smoothRadius = 0.0457f;
    float len = 0.2f;
    int id = 0;

    sph_shim::vec3 m_Origin;
    int m_flags;
    // terrain coupling
    bool m_terrain = false, m_erosion = false;
    float m_mpl = 0.0f;
    float m_k_capacity = 0.01f, m_k_pickup = 5.0f, m_k_deposit = 2.0f, m_layer = 0.0f;
    const Grid* m_grid_seen = nullptr;
    uint64_t m_version_seen = 0;
    std::shared_ptr<sph_terrain_link> m_link;
    sph_system* m_sys = nullptr;
    int m_scene = -1;
};
