// The vector type of the drop-in headers: glm::vec3 when the front end has
// glm (the reference's own dependency), otherwise a minimal stand-in with
// the members the reference's callers use (x, y, z, operator[]).
#pragma once

#if defined(SPH_SHIM_WITH_GLM) || (defined(__has_include) && __has_include(<glm/glm.hpp>) && \
                                   !defined(SPH_SHIM_NO_GLM))
#include <glm/glm.hpp>
#define SPH_SHIM_HAS_GLM 1
namespace sph_shim {
using vec3 = glm::vec3;
}
#else
namespace sph_shim {
struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
}  // namespace sph_shim
#endif
