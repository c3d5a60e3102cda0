// Terrain surface meshes on the device.
//
// k_mesh_u8 restates Grid::UpdateGrid (Erosion/grid.h:138-176) for the
// reference's 512 x 512 8-bit heightfield: one vertex per (x, z), z-major,
// each followed by the normalised sum of the four cross products of its edge
// vectors to the neighbouring heights, with the reference's operation order
// (explicitly rounded intrinsics, never fused).  The reference bounds the
// z + 1 neighbour by the grid's Y dimension (grid.h:167); that is kept.
// k_mesh_indices emits genIndices (grid.h:118-136): for every cell (z, x)
// with x < dimx - 1 and z < dimz - 1, two triangles, the second one mirrored
// from the opposite corner of the grid, at offset 6 * (z * (dimx - 1) + x).
//
// k_mesh_f32 builds the same kind of mesh for a scene's current (eroded)
// FP32 heights in world units, for the front end to redraw every frame.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "../../include/sph_erosion.h"
#include "sph_engine.h"

namespace sph {

namespace {

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }

struct V3 {
    float x, y, z;
};

// glm::cross (func_geometric.inl:68-79)
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
    return V3{fs(fm(a.y, b.z), fm(b.y, a.z)), fs(fm(a.z, b.x), fm(b.z, a.x)), fs(fm(a.x, b.y), fm(b.x, a.y))};
}

__device__ __forceinline__ V3 add3(V3 a, V3 b) { return V3{fa(a.x, b.x), fa(a.y, b.y), fa(a.z, b.z)}; }

// glm::normalize: v * (1 / sqrt(dot(v, v)))
__device__ __forceinline__ V3 normalize3(V3 v) {
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(fa(fa(fm(v.x, v.x), fm(v.y, v.y)), fm(v.z, v.z))));
    return V3{fm(v.x, inv), fm(v.y, inv), fm(v.z, inv)};
}

constexpr int kSide = 512;  // the reference's hard-coded heightfield side (grid.h:78-80)

__global__ void k_mesh_u8(const unsigned char* __restrict__ map, int dimx, int dimy, int dimz, float* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= dimx * dimz) return;
    const int z = t / dimx, x = t - z * dimx;
    auto H = [&](int hx, int hz) { return (int)map[kSide * hx + hz]; };
    int y = H(x, z);
    if (dimy <= y) y = dimy - 1;
    V3 u{0.f, 0.f, 0.f}, d{0.f, 0.f, 0.f}, r{0.f, 0.f, 0.f}, l{0.f, 0.f, 0.f};
    if (x - 1 >= 0) l = V3{(float)(x - (x - 1)), (float)(y - H(x - 1, z)), 0.0f};
    if (x + 1 < dimx) r = V3{(float)((x + 1) - x), (float)(H(x + 1, z) - y), 0.0f};
    if (z - 1 >= 0) u = V3{0.0f, (float)(y - H(x, z - 1)), (float)(z - (z - 1))};
    if (z + 1 < dimy && z + 1 < kSide) d = V3{0.0f, (float)(H(x, z + 1) - y), (float)((z + 1) - z)};
    const V3 n = normalize3(add3(add3(add3(cross3(u, l), cross3(u, r)), cross3(d, l)), cross3(d, r)));
    float* o = out + (size_t)6 * t;
    o[0] = (float)x;
    o[1] = (float)y;
    o[2] = (float)z;
    o[3] = n.x;
    o[4] = n.y;
    o[5] = n.z;
}

__global__ void k_mesh_indices(int dimx, int dimz, unsigned* __restrict__ idx) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cx = dimx - 1;
    if (t >= cx * (dimz - 1)) return;
    const int z = t / cx, x = t - z * cx;
    const int i = dimx - 1 - x, j = dimz - 1 - z;
    unsigned* o = idx + (size_t)6 * t;
    o[0] = (unsigned)(z * dimx + x);
    o[1] = (unsigned)(z * dimx + (x + 1));
    o[2] = (unsigned)((z + 1) * dimx + x);
    o[3] = (unsigned)(j * dimx + i);
    o[4] = (unsigned)(j * dimx + (i - 1));
    o[5] = (unsigned)((j - 1) * dimx + i);
}

// Mesh of a scene's heights: vertex (xlo + x sx, ylo + H ys, zlo + z sz) and
// the normalised sum of the four cross products of its edge vectors in the
// same units.  World units: ys = 1; the reference Grid's units (one unit per
// vertex along x and z, heights in grey levels): sx = sz = 1, ys = 1 / metres
// per level, origin 0.
__global__ void k_mesh_f32(const float* __restrict__ h, int tw, int td, float xlo, float ylo, float zlo, float sx,
                           float sz, float ys, float* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tw * td) return;
    const int z = t / tw, x = t - z * tw;
    auto H = [&](int q) { return fm(h[q], ys); };
    const float y = H(t);
    V3 u{0.f, 0.f, 0.f}, d{0.f, 0.f, 0.f}, r{0.f, 0.f, 0.f}, l{0.f, 0.f, 0.f};
    if (x > 0) l = V3{sx, fs(y, H(t - 1)), 0.0f};
    if (x + 1 < tw) r = V3{sx, fs(H(t + 1), y), 0.0f};
    if (z > 0) u = V3{0.0f, fs(y, H(t - tw)), sz};
    if (z + 1 < td) d = V3{0.0f, fs(H(t + tw), y), sz};
    const V3 n = normalize3(add3(add3(add3(cross3(u, l), cross3(u, r)), cross3(d, l)), cross3(d, r)));
    float* o = out + (size_t)6 * t;
    o[0] = fa(xlo, fm((float)x, sx));
    o[1] = fa(ylo, y);
    o[2] = fa(zlo, fm((float)z, sz));
    o[3] = n.x;
    o[4] = n.y;
    o[5] = n.z;
}

// Temporary device buffers of one mesh call.
struct Tmp {
    void* p = nullptr;
    explicit Tmp(size_t bytes) {
        if (bytes) check_cuda(cudaMalloc(&p, bytes), "cudaMalloc(mesh)");
    }
    ~Tmp() {
        if (p) cudaFree(p);
    }
};

}  // namespace

void mesh_u8(const unsigned char* map_host, int dimx, int dimy, int dimz, float* verts, unsigned* idx,
             int64_t idx_cap, int64_t* n_idx) {
    if (!map_host || dimx < 1 || dimz < 1 || dimy < 1 || dimx > kSide || dimz > kSide)
        throw Error(SPH_ERR_INVALID, "mesh dims must be in [1, 512] along x and z");
    const int64_t nv = (int64_t)dimx * dimz;
    const int64_t ni = (int64_t)6 * (dimx - 1) * (dimz - 1);
    if (n_idx) *n_idx = ni;
    if (idx && idx_cap < ni) throw Error(SPH_ERR_CAPACITY, "index buffer too small");
    Tmp dmap((size_t)kSide * kSide), dv((size_t)nv * 6 * 4), di((size_t)ni * 4);
    check_cuda(cudaMemcpy(dmap.p, map_host, (size_t)kSide * kSide, cudaMemcpyHostToDevice), "copy map");
    k_mesh_u8<<<(unsigned)((nv + 255) / 256), 256>>>(static_cast<unsigned char*>(dmap.p), dimx, dimy, dimz,
                                                     static_cast<float*>(dv.p));
    if (ni > 0) k_mesh_indices<<<(unsigned)((ni / 6 + 255) / 256), 256>>>(dimx, dimz, static_cast<unsigned*>(di.p));
    check_cuda(cudaGetLastError(), "mesh kernels");
    if (verts) check_cuda(cudaMemcpy(verts, dv.p, (size_t)nv * 24, cudaMemcpyDeviceToHost), "copy verts");
    if (idx && ni > 0) check_cuda(cudaMemcpy(idx, di.p, (size_t)ni * 4, cudaMemcpyDeviceToHost), "copy indices");
}

// metres_per_level = 0: world units; > 0: the reference Grid's units.
void mesh_scene(System& sys, int scene, float* verts, unsigned* idx, float metres_per_level) {
    int tw, td;
    sys.terrain_dims(scene, &tw, &td);
    if (tw < 2) throw Error(SPH_ERR_STATE, "scene has no terrain");
    if (!(metres_per_level >= 0.0f) || !std::isfinite(metres_per_level))
        throw Error(SPH_ERR_INVALID, "metres_per_level must be finite and >= 0");
    const sph_params& p = sys.params(scene);
    const bool grid_units = metres_per_level > 0.0f;
    const float sx = grid_units ? 1.0f : (p.box_half[0] + p.box_half[0]) / (float)(tw - 1);
    const float sz = grid_units ? 1.0f : (p.box_half[2] + p.box_half[2]) / (float)(td - 1);
    const float ys = grid_units ? 1.0f / metres_per_level : 1.0f;
    const float xlo = grid_units ? 0.0f : p.box_center[0] - p.box_half[0];
    const float ylo = grid_units ? 0.0f : p.box_center[1] - p.box_half[1];
    const float zlo = grid_units ? 0.0f : p.box_center[2] - p.box_half[2];
    const int64_t nv = (int64_t)tw * td, ni = (int64_t)6 * (tw - 1) * (td - 1);
    std::vector<float> h((size_t)nv);
    sys.get_terrain(scene, h.data(), nullptr);
    Tmp dh((size_t)nv * 4), dv((size_t)nv * 24), di((size_t)ni * 4);
    check_cuda(cudaMemcpy(dh.p, h.data(), (size_t)nv * 4, cudaMemcpyHostToDevice), "copy heights");
    k_mesh_f32<<<(unsigned)((nv + 255) / 256), 256>>>(static_cast<float*>(dh.p), tw, td, xlo, ylo, zlo, sx, sz, ys,
                                                      static_cast<float*>(dv.p));
    k_mesh_indices<<<(unsigned)((ni / 6 + 255) / 256), 256>>>(tw, td, static_cast<unsigned*>(di.p));
    check_cuda(cudaGetLastError(), "mesh kernels");
    if (verts) check_cuda(cudaMemcpy(verts, dv.p, (size_t)nv * 24, cudaMemcpyDeviceToHost), "copy verts");
    if (idx) check_cuda(cudaMemcpy(idx, di.p, (size_t)ni * 4, cudaMemcpyDeviceToHost), "copy indices");
}

}  // namespace sph

namespace {
template <class F>
int mesh_guard(F&& f) {
    try {
        f();
        return SPH_OK;
    } catch (const sph::Error& e) {
        sph::set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        sph::set_last_error(e.what());
        return SPH_ERR_INVALID;
    }
}
}  // namespace

extern "C" {

SPH_API int sph_terrain_mesh_u8(const unsigned char* map512, int dimx, int dimy, int dimz, float* verts,
                                unsigned* indices, int64_t index_cap, int64_t* n_indices) {
    return mesh_guard([&] { sph::mesh_u8(map512, dimx, dimy, dimz, verts, indices, index_cap, n_indices); });
}

SPH_API int sph_scene_terrain_mesh(sph_system* s, int scene, float* verts, unsigned* indices) {
    return mesh_guard([&] {
        if (!s || !s->sys) throw sph::Error(SPH_ERR_INVALID, "null system handle");
        sph::mesh_scene(*s->sys, scene, verts, indices, 0.0f);
    });
}

SPH_API int sph_scene_terrain_mesh_levels(sph_system* s, int scene, float metres_per_level, float* verts,
                                          unsigned* indices) {
    return mesh_guard([&] {
        if (!s || !s->sys) throw sph::Error(SPH_ERR_INVALID, "null system handle");
        if (!(metres_per_level > 0.0f)) throw sph::Error(SPH_ERR_INVALID, "metres_per_level must be > 0");
        sph::mesh_scene(*s->sys, scene, verts, indices, metres_per_level);
    });
}

}  // extern "C"
