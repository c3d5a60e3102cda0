// Test infrastructure only (the oracle's "reference" leg).
//
// Builds the reference's own FluidSystemSPH (Erosion/fluid_system.h) and Grid
// (Erosion/grid.h) headless, unmodified, and exposes them through a small C
// ABI so that tests/golden/make_golden.py can record golden vectors and the
// CPU tests can check the C restatement in sph_oracle.c against the real code.
// Nothing in the product links or loads this file.
//
// Harness-side shims (no reference file is edited):
//  * GLEW_NO_GLU: glew.h would otherwise want GL/glu.h.
//  * The two GLEW function pointers that ~Sphere (Erosion/sphere.h:87-95)
//    references are defined as null; they are never called because the
//    system is never drawn, so m_Sphere stays empty.
//  * `using std::abs;` before the include: MSVC (the reference's toolchain)
//    resolves abs(float) in collisionS (Erosion/fluid_system.h:356-370) to the
//    float overload; g++ would otherwise bind int abs(int) and silently turn
//    box collision off.
//  * `#define private public` around the include so that parameters without a
//    setter (h, k, len, ...) and the particle vector can be injected.
// Build with -ffp-contract=off so that no multiply-add is fused.

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cstdio>
#include <vector>
#include <list>
#include <memory>
#include <string>
#include <fstream>
#include <sstream>
#include <iostream>
#include <iomanip>
#include <float.h>
#include <omp.h>

#define GLEW_NO_GLU
#include <GL/glew.h>
#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>

using std::abs;

PFNGLDELETEVERTEXARRAYSPROC __glewDeleteVertexArrays = nullptr;
PFNGLDELETEBUFFERSPROC __glewDeleteBuffers = nullptr;

#define private public
#include "fluid_system.h"
#undef private

namespace {
Grid& dummy_grid() {
    static Grid g(1, 1, 1);
    return g;
}
}  // namespace

extern "C" {

// Field layout of one record returned by ref_get (27 floats):
//  0 pos[3], 3 vel[3], 6 acc[3], 9 density, 10 pressure, 11 fpress[3],
//  14 fvisc[3], 17 fgrav[3], 20 fsurf[3], 23 normal[3], 26 unused.
enum { REF_REC = 27 };

void* ref_new(void) { return new FluidSystemSPH(); }
void ref_free(void* p) { delete static_cast<FluidSystemSPH*>(p); }

void ref_initialize(void* p, int n) { static_cast<FluidSystemSPH*>(p)->Initialize(n); }
void ref_add_particles(void* p, int n) { static_cast<FluidSystemSPH*>(p)->AddParticles(n); }
void ref_reset(void* p) { static_cast<FluidSystemSPH*>(p)->Reset(); }
void ref_set_origin(void* p, float x, float y, float z) {
    static_cast<FluidSystemSPH*>(p)->SetOrigin(glm::vec3(x, y, z));
}

// vals: g.x g.y g.z deltaT p0 MASS visc surf_tens k cR h len
void ref_set_params(void* p, const float* v) {
    FluidSystemSPH* s = static_cast<FluidSystemSPH*>(p);
    s->g = glm::vec3(v[0], v[1], v[2]);
    s->deltaT = v[3];
    s->p0 = v[4];
    s->MASS = v[5];
    s->visc = v[6];
    s->surf_tens = v[7];
    s->k = v[8];
    s->cR = v[9];
    s->h = v[10];
    s->smoothRadius = v[10];
    s->len = v[11];
}

void ref_get_params(void* p, float* v) {
    FluidSystemSPH* s = static_cast<FluidSystemSPH*>(p);
    v[0] = s->g.x; v[1] = s->g.y; v[2] = s->g.z;
    v[3] = s->deltaT; v[4] = s->p0; v[5] = s->MASS; v[6] = s->visc;
    v[7] = s->surf_tens; v[8] = s->k; v[9] = s->cR; v[10] = s->h; v[11] = s->len;
}

// Replace the particle set: Id = index, zero acceleration, NeighbId = -1
// (the reference leaves NeighbId uninitialised until a neighbour is seen).
void ref_set_particles(void* p, int n, const float* pos, const float* vel) {
    FluidSystemSPH* s = static_cast<FluidSystemSPH*>(p);
    s->m_Particles.clear();
    for (int i = 0; i < n; i++) {
        FluidParticle fp;
        std::memset(&fp, 0, sizeof(fp));
        fp.Id = i;
        fp.Position = glm::vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        fp.Velocity = vel ? glm::vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]) : glm::vec3(0.0f);
        fp.Acceleration = glm::vec3(0.0f);
        fp.NeighbId = -1;
        s->m_Particles.push_back(fp);
    }
    s->num = n;
    s->init_num = n;
    s->id = n;
    s->smoothRadius = s->h;
}

int ref_count(void* p) { return (int)static_cast<FluidSystemSPH*>(p)->m_Particles.size(); }

void ref_run(void* p, int nsteps) {
    FluidSystemSPH* s = static_cast<FluidSystemSPH*>(p);
    for (int i = 0; i < nsteps; i++) s->Run(dummy_grid());
}

// rec: n * REF_REC floats; ids / neighb: n ints (may be null)
void ref_get(void* p, float* rec, int* ids, int* neighb) {
    FluidSystemSPH* s = static_cast<FluidSystemSPH*>(p);
    int n = (int)s->m_Particles.size();
    for (int i = 0; i < n; i++) {
        const FluidParticle& fp = s->m_Particles[i];
        float* r = rec + (size_t)REF_REC * i;
        const glm::vec3* v3[] = {&fp.Position, &fp.Velocity, &fp.Acceleration};
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) r[3 * a + c] = (*v3[a])[c];
        r[9] = fp.Density;
        r[10] = fp.Pressure;
        const glm::vec3* f3[] = {&fp.PressureForce, &fp.ViscosityForce, &fp.GravityForce,
                                 &fp.SurfaceForce, &fp.SurfaceNormal};
        for (int a = 0; a < 5; a++)
            for (int c = 0; c < 3; c++) r[11 + 3 * a + c] = (*f3[a])[c];
        r[26] = 0.0f;
        if (ids) ids[i] = fp.Id;
        if (neighb) neighb[i] = fp.NeighbId;
    }
}

// Neighbour count per particle with the reference's own in-range test
// (glm::length(x_i - x_j) <= smoothRadius, j != i; Erosion/fluid_system.h:139-142).
void ref_neighbour_counts(void* p, int* counts) {
    FluidSystemSPH* s = static_cast<FluidSystemSPH*>(p);
    int n = (int)s->m_Particles.size();
    for (int i = 0; i < n; i++) {
        int c = 0;
        for (int j = 0; j < n; j++) {
            float d = glm::length(s->m_Particles[i].Position - s->m_Particles[j].Position);
            if (d <= s->smoothRadius && i != j) c++;
        }
        counts[i] = c;
    }
}

// ---- Grid (Erosion/grid.h) -------------------------------------------------

void* ref_grid_new(int dx, int dy, int dz) { return new Grid(dx, dy, dz); }
// Grid has no destructor in the reference; the harness frees what it can reach.
void ref_grid_free(void* g) {
    Grid* gr = static_cast<Grid*>(g);
    delete[] gr->m_Grid;
    delete[] gr->m_heightfield.map;
    gr->m_Grid = nullptr;
    gr->m_heightfield.map = nullptr;
    delete gr;
}
void ref_grid_load(void* g, const unsigned char* img) {
    static_cast<Grid*>(g)->LoadHeightfield(const_cast<unsigned char*>(img));
}
void ref_grid_update(void* g, int dx, int dy, int dz) { static_cast<Grid*>(g)->UpdateGrid(dx, dy, dz); }
int ref_grid_surface_size(void* g) { return (int)static_cast<Grid*>(g)->GetSurfacePartsSize(); }
int ref_grid_indices_size(void* g) { return (int)static_cast<Grid*>(g)->GetIndicesSize(); }
void ref_grid_surface(void* g, float* out) {
    std::vector<float> v = static_cast<Grid*>(g)->GetSurfaceParts();
    std::memcpy(out, v.data(), v.size() * sizeof(float));
}
void ref_grid_indices(void* g, unsigned* out) {
    std::vector<unsigned> v = static_cast<Grid*>(g)->GetIndices();
    std::memcpy(out, v.data(), v.size() * sizeof(unsigned));
}
int ref_grid_height_at(void* g, int x, int y) { return static_cast<Grid*>(g)->GetHeightfieldAt(x, y); }
int ref_grid_collision(void* g, const float* cur, const float* next, const float* vel, float* cp, float* nrm) {
    glm::vec3 c(cur[0], cur[1], cur[2]), n(next[0], next[1], next[2]), v(vel[0], vel[1], vel[2]);
    glm::vec3 contact(0.0f), norm(0.0f);
    bool hit = static_cast<Grid*>(g)->collision(c, n, v, contact, norm);
    for (int a = 0; a < 3; a++) {
        cp[a] = contact[a];
        nrm[a] = norm[a];
    }
    return hit ? 1 : 0;
}

}  // extern "C"
