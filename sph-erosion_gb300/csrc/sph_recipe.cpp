// Seeded scene recipe: the erosion scene a request describes (seed, particle
// count, terrain side), built identically wherever it is used (the batched
// form, the request server, the tests).
//
// From the seed, a SplitMix64 stream draws, in order:
//   u0 -> coverage f in [0.2, 0.5) (unless given): block volume over the box
//         volume above the highest terrain point;
//   u1 -> amplitude a in [0.1, 0.4) (unless given), as a fraction of the box
//         height (an absolute 0.1-0.4 m would not fit the small boxes);
//   u2, u3 -> the block's x and z placement inside the free floor span.
// The box is a cube of side L = cbrt(n s^3 / (f (1 - a))), s = h/2 the lattice
// spacing, centred at the origin.  The block is a lattice at spacing s, n
// particles in y-slowest order, footprint at most 90% of the box side, one
// spacing above the terrain's maximum height a L.  The terrain is value-noise
// fBm of 6 octaves (lacunarity 2, gain 0.5) seeded with the request seed.
#include "sph_recipe.h"

#include <algorithm>
#include <cmath>

#include "sph_engine.h"

namespace sph {

namespace {
uint64_t mix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}
double unit(uint64_t seed, int k) { return (double)(mix(seed * 0x2545F4914F6CDD1DULL + (uint64_t)k) >> 11) * 0x1p-53; }
}  // namespace

void recipe_geometry(const sph_request& r, float h, RecipeGeometry* g) {
    if (r.particles <= 0) throw Error(SPH_ERR_INVALID, "request needs at least one particle");
    if (r.terrain_side < 2 || r.terrain_side > 8192) throw Error(SPH_ERR_INVALID, "terrain side must be in [2, 8192]");
    const double s = (double)h * 0.5;
    const double f = r.coverage > 0.0f ? (double)r.coverage : 0.2 + 0.3 * unit(r.seed, 0);
    const double a = r.amplitude > 0.0f ? (double)r.amplitude : 0.1 + 0.3 * unit(r.seed, 1);
    if (!(f > 0.0 && f <= 1.0) || !(a > 0.0 && a < 0.9)) throw Error(SPH_ERR_INVALID, "bad coverage or amplitude");
    const double L = std::cbrt((double)r.particles * s * s * s / (f * (1.0 - a)));
    g->side = (float)L;
    g->amplitude = (float)(a * L);
    g->coverage = (float)f;
    const int nmax = std::max(1, (int)std::floor(0.9 * L / s));
    int by = std::max(1, (int)std::lround(0.8 * std::cbrt((double)r.particles)));
    int bx = std::min(nmax, (int)std::ceil(std::sqrt((double)r.particles / by)));
    by = (int)std::ceil((double)r.particles / ((double)bx * bx));
    g->bx = bx;
    g->by = by;
    g->bz = bx;
    const double span = L - s - bx * s;
    g->x0 = (float)(-0.5 * L + 0.5 * s + std::max(0.0, span) * unit(r.seed, 2));
    g->z0 = (float)(-0.5 * L + 0.5 * s + std::max(0.0, span) * unit(r.seed, 3));
    g->y0 = (float)(-0.5 * L + a * L + s);
    g->spacing = (float)s;
}

void recipe_particles(const sph_request& r, const RecipeGeometry& g, float* pos3) {
    int c = 0;
    for (int y = 0; y < g.by && c < r.particles; ++y)
        for (int z = 0; z < g.bz && c < r.particles; ++z)
            for (int x = 0; x < g.bx && c < r.particles; ++x, ++c) {
                pos3[3 * c] = (float)((double)g.x0 + x * (double)g.spacing);
                pos3[3 * c + 1] = (float)((double)g.y0 + y * (double)g.spacing);
                pos3[3 * c + 2] = (float)((double)g.z0 + z * (double)g.spacing);
            }
}

void recipe_params(const sph_params& base, const RecipeGeometry& g, sph_params* p) {
    *p = base;
    for (int a = 0; a < 3; ++a) {
        p->box_center[a] = 0.0f;
        p->box_half[a] = 0.5f * g.side;
    }
}

}  // namespace sph
