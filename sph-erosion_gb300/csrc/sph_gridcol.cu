// Grid::collision (Erosion/grid.h:178-805) on the GPU: the reference's
// heightfield contact against the two triangles of each cell of its 8-bit
// 512 x 512 map, in integer cell units, with its adjacency walk
// (findAdjacentCell, :210-269), the in-between and corner-case mappings
// (:271-305, :320-440) and the same branch order.  The reference never calls
// it (fluid_system.h:335-340); this port serves front ends that do, as a
// batched query.  Every operation is an explicitly rounded FP32 intrinsic in
// the reference's order, so results equal the reference's bit for bit.
//
// One deliberate departure, where the reference reads outside its map
// (undefined behaviour): a height lookup outside [0, 511] reads 0.
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
struct V2 {
    float x, y;
};

__device__ __forceinline__ V3 sub(V3 a, V3 b) { return V3{fs(a.x, b.x), fs(a.y, b.y), fs(a.z, b.z)}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return V3{fa(a.x, b.x), fa(a.y, b.y), fa(a.z, b.z)}; }
__device__ __forceinline__ V3 scale(float s, V3 v) { return V3{fm(s, v.x), fm(s, v.y), fm(s, v.z)}; }
__device__ __forceinline__ V3 neg(V3 v) { return V3{-v.x, -v.y, -v.z}; }
// glm: tmp = a * b; tmp.x + tmp.y + tmp.z
__device__ __forceinline__ float dot(V3 a, V3 b) { return fa(fa(fm(a.x, b.x), fm(a.y, b.y)), fm(a.z, b.z)); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return V3{fs(fm(a.y, b.z), fm(b.y, a.z)), fs(fm(a.z, b.x), fm(b.z, a.x)), fs(fm(a.x, b.y), fm(b.x, a.y))};
}
// glm::normalize: v * inversesqrt(dot(v, v)), inversesqrt = 1 / sqrt
__device__ __forceinline__ V3 normalize(V3 v) {
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot(v, v)));
    return V3{fm(v.x, inv), fm(v.y, inv), fm(v.z, inv)};
}
__device__ __forceinline__ float length3(V3 v) { return __fsqrt_rn(dot(v, v)); }
__device__ __forceinline__ float length2(V2 v) { return __fsqrt_rn(fa(fm(v.x, v.x), fm(v.y, v.y))); }

struct Tri {
    V3 A, B, C, n;
};

__device__ __forceinline__ Tri make_tri(V3 a, V3 b, V3 c) {
    Tri t{a, b, c, V3{0, 0, 0}};
    t.n = normalize(cross(sub(b, a), sub(c, a)));
    return t;
}

struct Ctx {
    const unsigned char* map;
    int dimx, dimz;
    float det_thr;  // smallest float f with (double)f >= 1e-6
};

__device__ __forceinline__ float height(const Ctx& c, float fx, float fz) {
    const int x = (int)fx, z = (int)fz;  // GetHeightfieldAt(int, int) takes the float indices
    if (x < 0 || x > 511 || z < 0 || z > 511) return 0.0f;
    return (float)c.map[512 * x + z];
}

// getCellTriangles (:195-207): [0] = (C, B, A) "ABC", [1] = (AA, B, C) "AABC"
__device__ __forceinline__ void cell_tris(const Ctx& c, V2 ci, Tri* out) {
    const float x1 = fa(ci.x, 1.0f), y1 = fa(ci.y, 1.0f);
    const V3 A{ci.x, height(c, ci.x, ci.y), ci.y};
    const V3 AA{x1, height(c, x1, y1), y1};
    const V3 B{x1, height(c, x1, ci.y), ci.y};
    const V3 Cc{ci.x, height(c, ci.x, y1), y1};
    out[0] = make_tri(Cc, B, A);
    out[1] = make_tri(AA, B, Cc);
}

// rayIntersectsTriangle (:178-193).  invdet = 1.0 / det is a double quotient
// rounded to float, which equals the correctly rounded float reciprocal.
__device__ __forceinline__ bool ray_hit(const Ctx& c, V3 pos, V3 dir, const Tri& tri, float* t) {
    const V3 E1 = sub(tri.B, tri.A), E2 = sub(tri.C, tri.A);
    const V3 N = cross(E1, E2);
    const float det = -dot(dir, N);
    const float invdet = __frcp_rn(det);
    const V3 AO = sub(pos, tri.A);
    const V3 DAO = cross(AO, dir);
    const float u = fm(dot(E2, DAO), invdet);
    const float v = fm(-dot(E1, DAO), invdet);
    *t = fm(dot(AO, N), invdet);
    return fabsf(det) >= c.det_thr && *t >= 0.0f && u >= 0.0f && v >= 0.0f && fa(u, v) <= 1.0f;
}

// findAdjacentCell (:210-269) with unit cells.
__device__ V2 adjacent_cell(const Ctx& c, V3 pos, V3 dir, V2 ci) {
    float tx, tz;
    const float ox = pos.x, oz = pos.z, dx = dir.x, dz = dir.z;
    if (dx < 0.0f)
        tx = __fdiv_rn(fs(fm(floorf(__fdiv_rn(ox, 1.0f)), 1.0f), ox), dx);
    else if (dx > 0.0f)
        tx = __fdiv_rn(fs(fm(fa(floorf(__fdiv_rn(ox, 1.0f)), 1.0f), 1.0f), ox), dx);
    else
        tx = INFINITY;
    if (dz < 0.0f)
        tz = __fdiv_rn(fs(fm(floorf(__fdiv_rn(oz, 1.0f)), 1.0f), oz), dz);
    else if (dz > 0.0f)
        tz = __fdiv_rn(fs(fm(fa(floorf(__fdiv_rn(oz, 1.0f)), 1.0f), 1.0f), oz), dz);
    else
        tz = INFINITY;
    if (tx < tz) {
        if (dx < 0.0f)
            ci.x = fs(ci.x, 1.0f);
        else if (dx > 0.0f)
            ci.x = fa(ci.x, 1.0f);
    } else {
        if (dz < 0.0f)
            ci.y = fs(ci.y, 1.0f);
        else if (dz > 0.0f)
            ci.y = fa(ci.y, 1.0f);
    }
    if (ci.x < 0.0f || ci.x >= (float)c.dimx || ci.y < 0.0f || ci.y >= (float)c.dimz) ci = V2{-1.0f, -1.0f};
    return ci;
}

__device__ __forceinline__ bool mapped_on(const Ctx& c, const Tri& tri, V3 pos, V3 dir, V3* cp, V3* nrm) {
    float t;
    if (ray_hit(c, pos, dir, tri, &t)) {
        *nrm = dir;
        *cp = add(pos, scale(t, *nrm));
        return true;
    }
    return false;
}

__device__ __forceinline__ bool mapped_between(const Ctx& c, const Tri& t1, const Tri& t2, V3 pos, V3* cp, V3* nrm) {
    float t;
    if (ray_hit(c, pos, normalize(add(t1.n, t2.n)), t1, &t)) {
        *nrm = normalize(add(t1.n, t2.n));
        *cp = add(pos, scale(t, *nrm));
        return true;
    } else if (ray_hit(c, pos, normalize(add(t1.n, t2.n)), t2, &t)) {
        *nrm = normalize(add(t1.n, t2.n));
        *cp = add(pos, scale(t, *nrm));
        return true;
    }
    return false;
}

__device__ __forceinline__ float min3(float a, float b, float c) {
    if (a < b)
        return a < c ? a : c;
    return b < c ? b : c;
}

// Shared tail of both corner cases: the normal of the six triangles' normal
// sum, then the first triangle hit along it.
__device__ bool map_on_fan(const Ctx& c, const Tri* tr, V3 posNext, V3* cp, V3* nrm) {
    V3 n{0.0f, 0.0f, 0.0f};
    for (int k = 0; k < 6; ++k) n = add(n, tr[k].n);
    n = normalize(n);
    for (int k = 0; k < 6; ++k)
        if (mapped_on(c, tr[k], posNext, n, cp, nrm)) return true;
    return false;
}

// cornerCaseABC (:320-378)
__device__ bool corner_abc(const Ctx& c, const Tri& ABC, const Tri& AABC, V3 posCurr, V3 posNext, V2 ci, V3* cp,
                           V3* nrm) {
    const V2 p2{posCurr.x, posCurr.z};
    const V2 o{floorf(posCurr.x), floorf(posCurr.z)};
    const V2 right{fa(o.x, 1.0f), o.y}, down{o.x, fa(o.y, 1.0f)};
    const float dorigin = length2(V2{fs(o.x, p2.x), fs(o.y, p2.y)});
    const float dright = length2(V2{fs(right.x, p2.x), fs(right.y, p2.y)});
    const float ddown = length2(V2{fs(down.x, p2.x), fs(down.y, p2.y)});
    const float dmin = min3(dorigin, dright, ddown);
    Tri tr[6], tmp[2];
    if (dmin == dorigin) {
        tr[0] = ABC;
        cell_tris(c, V2{fs(ci.x, 1.0f), ci.y}, tmp);
        tr[1] = tmp[0];
        tr[2] = tmp[1];
        cell_tris(c, V2{ci.x, fs(ci.y, 1.0f)}, tmp);
        tr[3] = tmp[0];
        tr[4] = tmp[1];
        cell_tris(c, V2{fs(ci.x, 1.0f), fs(ci.y, 1.0f)}, tmp);
        tr[5] = tmp[1];
    } else if (dmin == dright) {
        tr[0] = ABC;
        tr[1] = AABC;
        cell_tris(c, V2{fa(ci.x, 1.0f), ci.y}, tmp);
        tr[2] = tmp[0];
        cell_tris(c, V2{ci.x, fs(ci.y, 1.0f)}, tmp);
        tr[3] = tmp[1];
        cell_tris(c, V2{fa(ci.x, 1.0f), fs(ci.y, 1.0f)}, tmp);
        tr[4] = tmp[0];
        tr[5] = tmp[1];
    } else {
        tr[0] = ABC;
        tr[1] = AABC;
        cell_tris(c, V2{fs(ci.x, 1.0f), ci.y}, tmp);
        tr[2] = tmp[1];
        cell_tris(c, V2{ci.x, fa(ci.y, 1.0f)}, tmp);
        tr[3] = tmp[0];
        cell_tris(c, V2{fs(ci.x, 1.0f), fa(ci.y, 1.0f)}, tmp);
        tr[4] = tmp[0];
        tr[5] = tmp[1];
    }
    return map_on_fan(c, tr, posNext, cp, nrm);
}

// cornerCaseAABC (:380-440)
__device__ bool corner_aabc(const Ctx& c, const Tri& ABC, const Tri& AABC, V3 posCurr, V3 posNext, V2 ci, V3* cp,
                            V3* nrm) {
    const V2 p2{posCurr.x, posCurr.z};
    const V2 o{fa(floorf(posCurr.x), 1.0f), fa(floorf(posCurr.z), 1.0f)};
    const V2 left{fs(o.x, 1.0f), o.y}, up{o.x, fs(o.y, 1.0f)};
    const float dorigin = length2(V2{fs(o.x, p2.x), fs(o.y, p2.y)});
    const float dleft = length2(V2{fs(left.x, p2.x), fs(left.y, p2.y)});
    const float dup = length2(V2{fs(up.x, p2.x), fs(up.y, p2.y)});
    const float dmin = min3(dorigin, dup, dleft);
    Tri tr[6], tmp[2];
    if (dmin == dorigin) {
        tr[0] = AABC;
        cell_tris(c, V2{fa(ci.x, 1.0f), ci.y}, tmp);
        tr[1] = tmp[0];
        tr[2] = tmp[1];
        cell_tris(c, V2{ci.x, fa(ci.y, 1.0f)}, tmp);
        tr[3] = tmp[0];
        tr[4] = tmp[1];
        cell_tris(c, V2{fa(ci.x, 1.0f), fa(ci.y, 1.0f)}, tmp);
        tr[5] = tmp[0];
    } else if (dmin == dup) {
        tr[0] = ABC;
        tr[1] = AABC;
        cell_tris(c, V2{fa(ci.x, 1.0f), ci.y}, tmp);
        tr[2] = tmp[0];
        cell_tris(c, V2{ci.x, fs(ci.y, 1.0f)}, tmp);
        tr[3] = tmp[1];
        cell_tris(c, V2{fa(ci.x, 1.0f), fs(ci.y, 1.0f)}, tmp);
        tr[4] = tmp[0];
        tr[5] = tmp[1];
    } else {
        tr[0] = ABC;
        tr[1] = AABC;
        cell_tris(c, V2{fs(ci.x, 1.0f), ci.y}, tmp);
        tr[2] = tmp[1];
        cell_tris(c, V2{ci.x, fa(ci.y, 1.0f)}, tmp);
        tr[3] = tmp[0];
        cell_tris(c, V2{fs(ci.x, 1.0f), fa(ci.y, 1.0f)}, tmp);
        tr[4] = tmp[0];
        tr[5] = tmp[1];
    }
    return map_on_fan(c, tr, posNext, cp, nrm);
}

constexpr float kFltEps = 1.192092896e-07f;  // FLT_EPSILON

// Grid::collision (:462-805)
__device__ bool collide(const Ctx& c, V3 posCurr, V3 posNext, V3 velNext, V3* contactP, V3* norm) {
    float t;
    const V3 dir = normalize(velNext);
    const V3 dirOpp = neg(dir);
    const V2 ci{floorf(posCurr.x), floorf(posCurr.z)};
    const V2 cn{floorf(posNext.x), floorf(posNext.z)};
    const float mx = (float)(c.dimx - 1), mz = (float)(c.dimz - 1);
    if (ci.x < 0.0f || ci.x >= mx || ci.y < 0.0f || ci.y >= mz || cn.x < 0.0f || cn.x >= mx || cn.y < 0.0f ||
        cn.y >= mz)
        return false;
    if (ci.x == cn.x && ci.y == cn.y) {
        Tri ct[2];
        cell_tris(c, ci, ct);
        const Tri& ABC = ct[0];
        const Tri& AABC = ct[1];
        float dABC = INFINITY, dAABC = INFINITY;
        if (ray_hit(c, posNext, dirOpp, ABC, &t)) dABC = length3(sub(add(posNext, scale(t, dirOpp)), posNext));
        if (ray_hit(c, posNext, dirOpp, AABC, &t)) dAABC = length3(sub(add(posNext, scale(t, dirOpp)), posNext));
        if (dABC < dAABC || (fabsf(fs(dABC, dAABC)) < kFltEps && dABC != INFINITY)) {
            if (ray_hit(c, posNext, ABC.n, ABC, &t)) {
                *norm = ABC.n;
                *contactP = add(posNext, scale(t, *norm));
                return true;
            }
            const V2 adj = adjacent_cell(c, posNext, normalize(add(dir, ABC.n)), ci);
            if (adj.x == -1.0f && adj.y == -1.0f) return false;
            Tri at[2];
            cell_tris(c, adj, at);
            const V2 cd{fs(adj.x, ci.x), fs(adj.y, ci.y)};
            if (cd.x > 0.0f || cd.y > 0.0f) {
                if (mapped_between(c, ABC, AABC, posNext, contactP, norm)) return true;
                if (corner_abc(c, ABC, AABC, posCurr, posNext, ci, contactP, norm)) return true;
            } else {
                if (mapped_between(c, ABC, at[1], posNext, contactP, norm)) return true;
                if (corner_abc(c, ABC, AABC, posCurr, posNext, ci, contactP, norm)) return true;
            }
        } else if (dAABC < dABC) {
            if (ray_hit(c, posNext, AABC.n, AABC, &t)) {
                *norm = AABC.n;
                *contactP = add(posNext, scale(t, *norm));
                return true;
            }
            const V2 adj = adjacent_cell(c, posNext, normalize(add(dir, AABC.n)), ci);
            if (adj.x == -1.0f && adj.y == -1.0f) return false;
            Tri at[2];
            cell_tris(c, adj, at);
            const V2 cd{fs(adj.x, ci.x), fs(adj.y, ci.y)};
            if (cd.x < 0.0f || cd.y < 0.0f) {
                if (mapped_between(c, ABC, AABC, posNext, contactP, norm)) return true;
                if (corner_aabc(c, ABC, AABC, posCurr, posNext, ci, contactP, norm)) return true;
            } else {
                if (mapped_between(c, AABC, at[0], posNext, contactP, norm)) return true;
                if (corner_aabc(c, ABC, AABC, posCurr, posNext, ci, contactP, norm)) return true;
            }
        }
        return false;
    }
    Tri pc[2], pn[2];
    cell_tris(c, ci, pc);
    cell_tris(c, cn, pn);
    const Tri& ABC_pc = pc[0];
    const Tri& AABC_pc = pc[1];
    const Tri& ABC_pn = pn[0];
    const Tri& AABC_pn = pn[1];
    const V2 cd{fs(cn.x, ci.x), fs(cn.y, ci.y)};
    if (cd.x != 0.0f && cd.y != 0.0f) {
        const float s = fa(cd.x, cd.y);
        if (s == -2.0f) {
            if (corner_abc(c, ABC_pc, AABC_pc, posCurr, posNext, ci, contactP, norm)) return true;
        } else if (s == 2.0f) {
            if (corner_aabc(c, ABC_pc, AABC_pc, posCurr, posNext, ci, contactP, norm)) return true;
        } else {
            if (corner_abc(c, ABC_pc, AABC_pc, posCurr, posNext, ci, contactP, norm)) return true;
        }
        return false;
    }
    if (ray_hit(c, posNext, dirOpp, ABC_pc, &t)) {
        if (cd.x == -1.0f || cd.y == -1.0f) {
            if (mapped_between(c, ABC_pc, AABC_pn, posNext, contactP, norm)) return true;
            if (corner_abc(c, ABC_pc, AABC_pc, posCurr, posNext, ci, contactP, norm)) return true;
        } else {
            if (corner_abc(c, ABC_pc, AABC_pc, posCurr, posNext, ci, contactP, norm)) return true;
        }
    } else if (ray_hit(c, posNext, dirOpp, AABC_pc, &t)) {
        if (cd.x == 1.0f || cd.y == 1.0f) {
            if (mapped_between(c, AABC_pc, ABC_pn, posNext, contactP, norm)) return true;
            if (corner_aabc(c, ABC_pc, AABC_pc, posCurr, posNext, ci, contactP, norm)) return true;
        } else {
            if (corner_aabc(c, ABC_pc, AABC_pc, posCurr, posNext, ci, contactP, norm)) return true;
        }
    } else {
        float dA = INFINITY, dAA = INFINITY;
        if (ray_hit(c, posCurr, dir, ABC_pn, &t)) dA = length3(sub(add(posCurr, scale(t, dir)), posCurr));
        if (ray_hit(c, posCurr, dir, AABC_pn, &t)) dAA = length3(sub(add(posCurr, scale(t, dir)), posCurr));
        if (dA < dAA || (fabsf(fs(dA, dAA)) < kFltEps && dA != INFINITY)) {
            if (ray_hit(c, posNext, ABC_pn.n, ABC_pn, &t)) {
                *norm = ABC_pn.n;
                *contactP = add(posNext, scale(t, *norm));
                return true;
            }
            if (cd.x == 1.0f || cd.y == 1.0f) {
                if (mapped_between(c, ABC_pn, AABC_pc, posNext, contactP, norm)) return true;
                if (corner_aabc(c, ABC_pc, AABC_pc, posCurr, posNext, ci, contactP, norm)) return true;
            } else {
                if (corner_abc(c, ABC_pc, AABC_pc, posCurr, posNext, ci, contactP, norm)) return true;
            }
        } else if (dAA < dA) {
            if (ray_hit(c, posNext, AABC_pn.n, AABC_pn, &t)) {
                *norm = AABC_pn.n;
                *contactP = add(posNext, scale(t, *norm));
                return true;
            }
            if (cd.x == -1.0f || cd.y == -1.0f) {
                if (mapped_between(c, AABC_pn, ABC_pc, posNext, contactP, norm)) return true;
                if (corner_abc(c, ABC_pc, AABC_pc, posCurr, posNext, ci, contactP, norm)) return true;
            } else {
                if (corner_aabc(c, ABC_pc, AABC_pc, posCurr, posNext, ci, contactP, norm)) return true;
            }
        }
    }
    return false;
}

__global__ void k_grid_collision(Ctx c, int n, const float* __restrict__ cur, const float* __restrict__ nxt,
                                 const float* __restrict__ vel, float* __restrict__ cp, float* __restrict__ nr,
                                 int32_t* __restrict__ hit) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const V3 a{cur[3 * q], cur[3 * q + 1], cur[3 * q + 2]};
    const V3 b{nxt[3 * q], nxt[3 * q + 1], nxt[3 * q + 2]};
    const V3 v{vel[3 * q], vel[3 * q + 1], vel[3 * q + 2]};
    V3 contact{0.0f, 0.0f, 0.0f}, normal{0.0f, 0.0f, 0.0f};
    const bool h = collide(c, a, b, v, &contact, &normal);
    cp[3 * q] = contact.x;
    cp[3 * q + 1] = contact.y;
    cp[3 * q + 2] = contact.z;
    nr[3 * q] = normal.x;
    nr[3 * q + 1] = normal.y;
    nr[3 * q + 2] = normal.z;
    hit[q] = h ? 1 : 0;
}

float det_threshold() {
    float f = (float)1e-6;
    while ((double)f < 1e-6) f = std::nextafter(f, INFINITY);
    for (;;) {
        const float pv = std::nextafter(f, 0.0f);
        if ((double)pv >= 1e-6)
            f = pv;
        else
            break;
    }
    return f;
}

struct DevMem {
    void* p = nullptr;
    explicit DevMem(size_t b) {
        if (b) check_cuda(cudaMalloc(&p, b), "cudaMalloc(collision)");
    }
    ~DevMem() {
        if (p) cudaFree(p);
    }
};

}  // namespace

void grid_collision_u8(const unsigned char* map512, int dimx, int dimz, int n, const float* cur3, const float* next3,
                       const float* vel3, float* contact3, float* normal3, int32_t* hit) {
    if (!map512 || n < 0 || dimx < 2 || dimz < 2 || dimx > 512 || dimz > 512)
        throw Error(SPH_ERR_INVALID, "grid collision: bad map or dims (2..512)");
    if (n == 0) return;
    if (!cur3 || !next3 || !vel3 || !contact3 || !normal3 || !hit) throw Error(SPH_ERR_INVALID, "null query array");
    const size_t vb = (size_t)n * 12;
    DevMem dmap(512 * 512), dc(vb), dn(vb), dv(vb), dcp(vb), dnr(vb), dh((size_t)n * 4);
    check_cuda(cudaMemcpy(dmap.p, map512, 512 * 512, cudaMemcpyHostToDevice), "copy map");
    check_cuda(cudaMemcpy(dc.p, cur3, vb, cudaMemcpyHostToDevice), "copy");
    check_cuda(cudaMemcpy(dn.p, next3, vb, cudaMemcpyHostToDevice), "copy");
    check_cuda(cudaMemcpy(dv.p, vel3, vb, cudaMemcpyHostToDevice), "copy");
    Ctx c{static_cast<const unsigned char*>(dmap.p), dimx, dimz, det_threshold()};
    k_grid_collision<<<(n + 127) / 128, 128>>>(c, n, static_cast<float*>(dc.p), static_cast<float*>(dn.p),
                                               static_cast<float*>(dv.p), static_cast<float*>(dcp.p),
                                               static_cast<float*>(dnr.p), static_cast<int32_t*>(dh.p));
    check_cuda(cudaGetLastError(), "collision kernel");
    check_cuda(cudaMemcpy(contact3, dcp.p, vb, cudaMemcpyDeviceToHost), "copy");
    check_cuda(cudaMemcpy(normal3, dnr.p, vb, cudaMemcpyDeviceToHost), "copy");
    check_cuda(cudaMemcpy(hit, dh.p, (size_t)n * 4, cudaMemcpyDeviceToHost), "copy");
}

}  // namespace sph

extern "C" SPH_API int sph_grid_collision_u8(const unsigned char* map512, int dimx, int dimz, int n,
                                             const float* cur3, const float* next3, const float* vel3,
                                             float* contact3, float* normal3, int32_t* hit) {
    try {
        sph::grid_collision_u8(map512, dimx, dimz, n, cur3, next3, vel3, contact3, normal3, hit);
        return SPH_OK;
    } catch (const sph::Error& e) {
        sph::set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        sph::set_last_error(e.what());
        return SPH_ERR_INVALID;
    }
}
