// Seeded scene recipes of the batched form and the request server
// (sph_recipe.cpp).
#pragma once
#include "../../include/sph_erosion.h"

namespace sph {

struct RecipeGeometry {
    float side;       // box side (cube centred at the origin)
    float amplitude;  // terrain amplitude, metres
    float coverage;
    int bx, by, bz;   // block lattice dims
    float x0, y0, z0; // first lattice point
    float spacing;
};

void recipe_geometry(const sph_request& r, float h, RecipeGeometry* g);
void recipe_particles(const sph_request& r, const RecipeGeometry& g, float* pos3);
void recipe_params(const sph_params& base, const RecipeGeometry& g, sph_params* p);

}  // namespace sph
