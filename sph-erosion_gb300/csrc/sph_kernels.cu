// Hand-written sm_103a kernels of one simulation step, all scenes of a system
// per launch.  Each kernel walks a work list of (scene, tile) items in a
// grid-stride loop; the particle passes are launched with one block per tile,
// so the hardware hands tiles to SMs as they free up.  A scene whose step
// budget is exhausted is skipped.
//
// Stage order per step (the reference's Run, Erosion/fluid_system.h:104-183,
// with its three O(N^2) passes replaced by a uniform grid):
//   keys -> scan -> scatter -> reorder   counting sort into Morton-ordered cell rows along x
//   density                               pass 1 (:107-124)
//   force                                 passes 2 and 3 (:127-178), advance
//                                         (:306-353), box (:355-407), terrain
//                                         contact and erosion exchange
//   terrain                               height snapshot for the next step
//
// Every arithmetic operation of the physics uses an explicitly rounded
// intrinsic (__fmul_rn, __fadd_rn, ...), which the compiler never contracts
// into a fused multiply-add, so each term rounds exactly like the reference's
// scalar FP32 code.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_kernels.h"

namespace sph {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsq(float a) { return __fsqrt_rn(a); }

// x^2 with one rounding (what a correctly rounded powf(x, 2.0f) returns).
__device__ __forceinline__ float pow2(float x) { return __fmul_rn(x, x); }

// x^3 rounded once in all but near-tie cases: x*x = p + e exactly and
// p*x = c + f exactly (TwoProduct with FMA; Ogita, Rump and Oishi, "Accurate
// sum and dot product", SIAM J. Sci. Comput. 2005), then c + (f + e*x).
__device__ __forceinline__ float pow3(float x) {
    float p = __fmul_rn(x, x);
    float e = __fmaf_rn(x, x, -p);
    float c = __fmul_rn(p, x);
    float f = __fmaf_rn(p, x, -c);
    float t = __fmaf_rn(e, x, f);
    return __fadd_rn(c, t);
}

// Squared distance of the reference's glm::length, (dx*dx + dy*dy) + dz*dz.
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return fa(fa(fm(dx, dx), fm(dy, dy)), fm(dz, dz));
}

// Two consecutive float4 (32 bytes at a 32-byte boundary: a packed record,
// or two neighbouring sorted positions) in one 256-bit read-only load, one
// L1 request instead of two.
__device__ __forceinline__ void ld_record(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

__device__ __forceinline__ int cell_coord(float x, float lo, float inv, int n) {
    float t = fm(fs(x, lo), inv);
    if (!(t > 0.0f)) t = 0.0f;  // also maps NaN to 0
    float top = (float)(n - 1);
    if (t > top) t = top;
    return (int)t;
}

struct Cell {
    int cx, cy, cz;
};

__device__ __forceinline__ Cell cell_of(const SceneDev& S, float x, float y, float z) {
    Cell c;
    c.cx = cell_coord(x, S.lo[0], S.inv_cell_x, S.nx);
    c.cy = cell_coord(y, S.lo[1], S.inv_cell, S.ny);
    c.cz = cell_coord(z, S.lo[2], S.inv_cell, S.nz);
    return c;
}

__device__ __forceinline__ uint32_t row_key(const uint32_t* tab, const SceneDev& S, int cy, int cz) {
    return __ldg(tab + S.tab_off + cz * S.ny + cy) * (uint32_t)S.nx;
}

// A particle's position in cell units before flooring and clamping, and its
// cell.
struct Probe {
    Cell c;
    float tx, ty, tz;
    bool finite;
};

__device__ __forceinline__ Probe probe_of(const SceneDev& S, float4 x) {
    Probe q;
    q.tx = fm(fs(x.x, S.lo[0]), S.inv_cell_x);
    q.ty = fm(fs(x.y, S.lo[1]), S.inv_cell);
    q.tz = fm(fs(x.z, S.lo[2]), S.inv_cell);
    q.finite = (q.tx == q.tx) && (q.ty == q.ty) && (q.tz == q.tz);
    q.c = cell_of(S, x.x, x.y, x.z);
    return q;
}

// Distance in cell units from coordinate t to cell k of an axis of n cells.
// The two end cells reach to infinity: positions outside the grid are
// clamped into them.
__device__ __forceinline__ float cell_gap(float t, int k, int n) {
    float g = 0.0f;
    if (k > 0 && t < (float)k) g = (float)k - t;
    if (k < n - 1 && t > (float)(k + 1)) g = t - (float)(k + 1);
    return g;
}

// Cells [xl, xh] of row (y, z) that the h-sphere around the particle can
// reach; false when it reaches none.  Conservative (h enlarged by hcell's
// slack), so only out-of-range candidates are ever dropped and the in-range
// visiting order is the same as for the full (2R+1)^3 block.
__device__ __forceinline__ bool row_span(const SceneDev& S, const Probe& q, int y, int z, int* xl, int* xh) {
    if (!q.finite) return false;  // a NaN position has no neighbour, itself included
    const float gy = cell_gap(q.ty, y, S.ny), gz = cell_gap(q.tz, z, S.nz);
    const float r2 = S.hcell * S.hcell - gy * gy - gz * gz;
    if (!(r2 >= 0.0f)) return false;
    const float r = sqrtf(r2) * (float)S.xsub;  // in x cells
    const float top = (float)(S.nx - 1);
    const float lo = fminf(fmaxf(floorf(q.tx - r), 0.0f), top);
    const float hi = fminf(fmaxf(floorf(q.tx + r), 0.0f), top);
    *xl = (int)lo;
    *xh = (int)hi;
    return true;
}

// Cell rows of the neighbour search.  for_rows(a, S, xi, valid, fn) calls
// fn(st, en) for each of the (2R+1)^2 rows (dz outer, dy inner, both
// ascending) with the particle range [st, en) of the row's cells that the
// h-sphere around xi can reach; a row it cannot reach (or any row when
// valid is false) gives an empty range, so every lane makes the same calls.
// The reach test is conservative (h enlarged by hcell's slack): only
// out-of-range candidates are ever dropped and the in-range visiting order is
// that of the full (2R+1)^3 block.
//
// At reach 1 (cells of h or more) cells along x are half as long as along y
// and z (xsub 2): a row's range is trimmed to the sphere in finer steps at
// no extra row.  For R = 1 and 2 (y/z cells of h and h/2, x reach 2 cells
// either way) the squared gaps of the 5 x cells are computed once per
// particle (registers), so a row costs a few adds and compares; the row loops stay rolled to keep register pressure (and
// so occupancy) where these latency-bound kernels need it.  Other reaches
// take the general path.
template <int R, class Fn>
__device__ __forceinline__ void for_rows_r(const DevArrays& a, const SceneDev& S, float4 xi, bool valid, Fn&& fn) {
    const Probe q = probe_of(S, xi);
    const uint32_t* off = a.offsets + S.k_off;
    const uint32_t* tab = a.tab + S.tab_off;
    const float H2 = S.hcell * S.hcell;
    constexpr int XS = R == 1 ? 2 : 1;  // the scene's xsub at this reach
    constexpr int RX = R * XS;          // reach along x, in x cells
    float gx2[2 * RX + 1];              // squared x-gaps in y/z cell units
#pragma unroll
    for (int d = -RX; d <= RX; ++d) {
        const int k = q.c.cx + d;
        float g2 = INFINITY;
        if (k >= 0 && k < S.nx) {
            const float g = cell_gap(q.tx, k, S.nx) * (1.0f / XS);
            g2 = g * g;
        }
        gx2[d + RX] = g2;
    }
    const bool live = valid && q.finite;
#pragma unroll 1
    for (int dz = -R; dz <= R; ++dz) {
        const int z = q.c.cz + dz;
        const bool zin = live && z >= 0 && z < S.nz;
        float gz2 = INFINITY;
        const uint32_t* tz = tab + (zin ? z : 0) * S.ny;  // row numbers of slab z
        if (zin) {
            const float g = cell_gap(q.tz, z, S.nz);
            gz2 = g * g;
        }
#pragma unroll 1
        for (int dy = -R; dy <= R; ++dy) {
            const int y = q.c.cy + dy;
            uint32_t st = 0, en = 0;
            if (zin && y >= 0 && y < S.ny) {
                const float g = cell_gap(q.ty, y, S.ny);
                const float r2 = H2 - g * g - gz2;
                if (r2 >= 0.0f) {
                    int lo = 0, hi = 0;  // farthest reachable cell on each side
#pragma unroll
                    for (int d = 1; d <= RX; ++d) {
                        if (gx2[RX - d] <= r2) lo = -d;
                        if (gx2[RX + d] <= r2) hi = d;
                    }
                    const uint32_t row = __ldg(tz + y) * (uint32_t)S.nx;
                    st = __ldg(off + row + q.c.cx + lo);
                    en = __ldg(off + row + q.c.cx + hi + 1);
                }
            }
            fn(st, en);
        }
    }
}

template <class Fn>
__device__ __forceinline__ void for_rows_any(const DevArrays& a, const SceneDev& S, float4 xi, bool valid, Fn&& fn) {
    const Probe q = probe_of(S, xi);
    const int R = S.reach;
    const uint32_t* off = a.offsets + S.k_off;
    for (int dz = -R; dz <= R; ++dz) {
        for (int dy = -R; dy <= R; ++dy) {
            const int z = q.c.cz + dz, y = q.c.cy + dy;
            uint32_t st = 0, en = 0;
            int xl, xh;
            if (valid && z >= 0 && z < S.nz && y >= 0 && y < S.ny && row_span(S, q, y, z, &xl, &xh)) {
                const uint32_t row = row_key(a.tab, S, y, z);
                st = __ldg(off + row + xl);
                en = __ldg(off + row + xh + 1);
            }
            fn(st, en);
        }
    }
}

template <class Fn>
__device__ __forceinline__ void for_rows(const DevArrays& a, const SceneDev& S, float4 xi, bool valid, Fn&& fn) {
    if (S.reach == 2)
        for_rows_r<2>(a, S, xi, valid, fn);
    else if (S.reach == 1)
        for_rows_r<1>(a, S, xi, valid, fn);
    else
        for_rows_any(a, S, xi, valid, fn);
}

// Visit every candidate of the trimmed rows around xi: f(j, xj) receives the
// scene-local sorted index and the position.
template <class F>
__device__ __forceinline__ void for_each_candidate(const DevArrays& a, const SceneDev& S, float4 xi, F&& f) {
    const float4* sp = a.spos + S.p_off;
    for_rows(a, S, xi, true, [&](uint32_t st, uint32_t en) {
        for (uint32_t j = st; j < en; ++j) f(j, __ldg(sp + j));
    });
}

// The same visit with the candidates of a row taken two at a time (both
// loads issued before either is tested); the order is unchanged.
template <class F>
__device__ __forceinline__ void for_each_candidate_x2(const DevArrays& a, const SceneDev& S, float4 xi, F&& f) {
    const float4* sp = a.spos + S.p_off;
    for_rows(a, S, xi, true, [&](uint32_t st, uint32_t en) {
        uint32_t j = st;
        for (; j + 1 < en; j += 2) {
            const float4 x0 = __ldg(sp + j), x1 = __ldg(sp + j + 1);
            f(j, x0);
            f(j + 1, x1);
        }
        if (j < en) f(j, __ldg(sp + j));
    });
}

// In-range traversal of the fast path.  Candidates are tested in a tight
// loop and the indices of in-range ones are compacted into a per-thread list
// in shared memory (column threadIdx.x, so lanes touch distinct banks); the
// costly pair terms then run over the list with every lane of the warp busy
// instead of diverging on each candidate.  The visiting order is the
// candidate order, so the sums are the same as a direct traversal.
//
// All lanes of a warp visit the same (dz, dy) cell row at the same time and
// step through it for the longest lane's length, so the list drain is a
// collective step: it runs as soon as any lane's list is full, with all lanes
// draining theirs.  Every lane of the warp must call this function (lanes
// without a particle pass valid = false).
constexpr int kListCap = 32;

template <class F>
__device__ __forceinline__ void for_each_in_range_listed(const DevArrays& a, const SceneDev& S, bool valid,
                                                         float4 xi, uint32_t* list, F&& f) {
    const float4* sp = a.spos + S.p_off;
    uint32_t* my = list + threadIdx.x;
    const int stride = blockDim.x;
    int cnt = 0;
    for_rows(a, S, xi, valid, [&](uint32_t st, uint32_t en) {
        const uint32_t len = en - st;
        const uint32_t maxlen = __reduce_max_sync(kFull, len);
        for (uint32_t t = 0; t < maxlen; ++t) {
            if (t < len) {
                const uint32_t j = st + t;
                const float4 xj = __ldg(sp + j);
                const float s = dist2(fs(xi.x, xj.x), fs(xi.y, xj.y), fs(xi.z, xj.z));
                if (s <= S.smax) my[(cnt++) * stride] = j;
            }
            if (__any_sync(kFull, cnt == kListCap)) {
                for (int q = 0; q < cnt; ++q) f(my[q * stride]);
                cnt = 0;
            }
        }
    });
    for (int q = 0; q < cnt; ++q) f(my[q * stride]);
}

// Ordered (validation) traversal: collect in-range candidates, sort them by
// particle id and visit them in ascending id, which is the reference's
// summation order (all j ascending).
constexpr int kMaxNb = 128;

template <class F>
__device__ __forceinline__ bool for_each_in_range_ordered(const DevArrays& a, const SceneDev& S, float4 xi,
                                                           F&& f) {
    unsigned long long lst[kMaxNb];
    int cnt = 0;
    bool overflow = false;
    for_each_candidate(a, S, xi, [&](uint32_t j, float4 xj) {
        float s = dist2(fs(xi.x, xj.x), fs(xi.y, xj.y), fs(xi.z, xj.z));
        if (s <= S.smax) {
            if (cnt < kMaxNb)
                lst[cnt++] = ((unsigned long long)(uint32_t)__float_as_int(xj.w) << 32) | j;
            else
                overflow = true;
        }
    });
    for (int q = 1; q < cnt; ++q) {
        unsigned long long v = lst[q];
        int r = q - 1;
        while (r >= 0 && lst[r] > v) {
            lst[r + 1] = lst[r];
            --r;
        }
        lst[r + 1] = v;
    }
    const float4* sp = a.spos + S.p_off;
    for (int q = 0; q < cnt; ++q) {
        uint32_t j = (uint32_t)(lst[q] & 0xffffffffu);
        f(j, __ldg(sp + j));
    }
    return !overflow;
}

// kernDefault for an in-range pair (fluid_system.h:410-416), times MASS.
__device__ __forceinline__ float density_term(const SceneDev& S, float len) {
    return fm(S.mass, fm(S.c_poly6, pow3(fs(S.hh, fm(len, len)))));
}

struct ForceAcc {
    float fpx, fpy, fpz;
    float fvx, fvy, fvz;
    float nx, ny, nz;
    float cfl;
    int nb;
    int any;
};

// Terms of passes 2 and 3 for one in-range pair (fluid_system.h:139-171):
// r = x_i - x_j, len = |r|; vj, Aj = P_j/rho_j^2, Bj = m/rho_j.
__device__ __forceinline__ void force_pair(const SceneDev& S, ForceAcc& acc, float rx, float ry, float rz,
                                           float len, float vix, float viy, float viz, float Ai, float4 vj,
                                           float Aj, float Bj, int idj, bool self) {
    // pass 3: colour-field Laplacian, self included (laplDefault, :424-428)
    {
        float ld = fm(fm(-S.c_grad, fs(S.hh, fm(len, len))),
                      fs(fm(fm(3.0f, S.h), S.h), fm(fm(7.0f, len), len)));
        acc.cfl = fa(acc.cfl, fm(Bj, ld));
    }
    if (self) return;
    acc.nb = max(acc.nb, idj);
    acc.any = 1;
    // gradPressure (:430-447)
    float gx, gy, gz;
    const float pw2 = pow2(fs(S.h, len));
    if (len < S.cthr) {
        float t = fm(fm(S.inv_sqrt3, S.c_spiky), pw2);
        gx = -t;
        gy = -t;
        gz = -t;
    } else {
        // glm::normalize: r * (1 / sqrt(dot(r, r))); the correctly rounded
        // reciprocal is the same value as the correctly rounded 1/len
        float inv = __frcp_rn(len);
        gx = -fm(fm(fm(rx, inv), S.c_spiky), pw2);
        gy = -fm(fm(fm(ry, inv), S.c_spiky), pw2);
        gz = -fm(fm(fm(rz, inv), S.c_spiky), pw2);
    }
    const float coef = fm(fa(Ai, Aj), S.mass);
    acc.fpx = fa(acc.fpx, fm(coef, gx));
    acc.fpy = fa(acc.fpy, fm(coef, gy));
    acc.fpz = fa(acc.fpz, fm(coef, gz));
    // laplVisc (:449-453)
    const float lv = fm(S.c_spiky, fs(S.h, len));
    acc.fvx = fa(acc.fvx, fm(fm(fs(vj.x, vix), Bj), lv));
    acc.fvy = fa(acc.fvy, fm(fm(fs(vj.y, viy), Bj), lv));
    acc.fvz = fa(acc.fvz, fm(fm(fs(vj.z, viz), Bj), lv));
    // gradDefault (:418-422)
    const float pw = pow2(fs(S.hh, fm(len, len)));
    acc.nx = fa(acc.nx, fm(Bj, -fm(fm(rx, S.c_grad), pw)));
    acc.ny = fa(acc.ny, fm(Bj, -fm(fm(ry, S.c_grad), pw)));
    acc.nz = fa(acc.nz, fm(Bj, -fm(fm(rz, S.c_grad), pw)));
}

// Fast-arithmetic form of density_term and force_pair (variant bit 17, fast
// mode only): the same kernel terms with the products grouped, fused
// multiply-adds, r^2 in place of |r|^2 and a hardware reciprocal square root
// for 1/|r|.  The in-range test stays exact (s <= smax), so the neighbour sets
// and NeighbId are the reference's; the rounding is not, and the results are
// held to the parity tolerance instead of to bits.
//
// r^2 with two fused multiply-adds, the force pass's fast form (its pairs
// are in range already): like dist2, within 3 units of rounding of the true
// sum of squares.
__device__ __forceinline__ float dist2_fma(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

__device__ __forceinline__ float density_term_fast(const SceneDev& S, float s) {
    const float hs = S.hh - s;
    return (S.mass * S.c_poly6) * (hs * hs * hs);
}

__device__ __forceinline__ void force_pair_fast(const SceneDev& S, ForceAcc& acc, float rx, float ry, float rz,
                                                float s, float vix, float viy, float viz, float Ai, float4 vj,
                                                float Aj, float Bj, int idj, bool self) {
    const float hs = S.hh - s;  // h^2 - r^2
    // pass 3: colour-field Laplacian, self included (laplDefault)
    acc.cfl = fmaf(Bj, (-S.c_grad * hs) * fmaf(-7.0f, s, 3.0f * S.hh), acc.cfl);
    if (self) return;
    acc.nb = max(acc.nb, idj);
    acc.any = 1;
    const float coef = (Ai + Aj) * S.mass;
    if (s < S.cthr * S.cthr) {
        // coincident: gradPressure along normalize(1, 1, 1)
        const float hl = S.h - sqrtf(s);
        const float g = -(S.inv_sqrt3 * S.c_spiky) * (hl * hl) * coef;
        acc.fpx += g;
        acc.fpy += g;
        acc.fpz += g;
        const float bl = Bj * (S.c_spiky * hl);
        acc.fvx = fmaf(vj.x - vix, bl, acc.fvx);
        acc.fvy = fmaf(vj.y - viy, bl, acc.fvy);
        acc.fvz = fmaf(vj.z - viz, bl, acc.fvz);
    } else {
        const float inv = rsqrtf(s);  // 1/|r|
        const float hl = S.h - s * inv;  // h - |r|
        const float g = -(S.c_spiky * coef) * (hl * hl) * inv;  // gradPressure / |r|, times coef
        acc.fpx = fmaf(rx, g, acc.fpx);
        acc.fpy = fmaf(ry, g, acc.fpy);
        acc.fpz = fmaf(rz, g, acc.fpz);
        const float bl = Bj * (S.c_spiky * hl);  // laplVisc times m/rho_j
        acc.fvx = fmaf(vj.x - vix, bl, acc.fvx);
        acc.fvy = fmaf(vj.y - viy, bl, acc.fvy);
        acc.fvz = fmaf(vj.z - viz, bl, acc.fvz);
    }
    const float gn = -(Bj * S.c_grad) * (hs * hs);  // gradDefault / r, times m/rho_j
    acc.nx = fmaf(rx, gn, acc.nx);
    acc.ny = fmaf(ry, gn, acc.ny);
    acc.nz = fmaf(rz, gn, acc.nz);
}

struct TSample {
    float y;
    float nx, ny, nz;
    int vnear;
};

// Heightfield surface at (x, z): bilinear over the vertex grid spanning the
// box floor (the repository's own contact model; the reference's
// Grid::collision is disabled at fluid_system.h:335-340).
__device__ __forceinline__ TSample terrain_at(const SceneDev& S, const float* hs, float x, float z) {
    TSample t;
    float fx = fm(fs(x, S.t_xlo), S.t_isx);
    float fz = fm(fs(z, S.t_zlo), S.t_isz);
    if (!(fx > 0.0f)) fx = 0.0f;
    if (fx > S.t_wmax) fx = S.t_wmax;
    if (!(fz > 0.0f)) fz = 0.0f;
    if (fz > S.t_dmax) fz = S.t_dmax;
    int i0 = (int)fx, j0 = (int)fz;
    if (i0 > S.tw - 2) i0 = S.tw - 2;
    if (j0 > S.td - 2) j0 = S.td - 2;
    const float tx = fs(fx, (float)i0), tz = fs(fz, (float)j0);
    const float* r0 = hs + S.t_off + (size_t)j0 * S.tw + i0;
    const float h00 = __ldg(r0), h10 = __ldg(r0 + 1);
    const float h01 = __ldg(r0 + S.tw), h11 = __ldg(r0 + S.tw + 1);
    const float a0 = fa(h00, fm(tx, fs(h10, h00)));
    const float a1 = fa(h01, fm(tx, fs(h11, h01)));
    const float hgt = fa(a0, fm(tz, fs(a1, a0)));
    t.y = fa(S.t_ylo, hgt);
    const float dx = fm(fa(fs(h10, h00), fm(tz, fs(fs(h11, h01), fs(h10, h00)))), S.t_isx);
    const float dz = fm(fs(a1, a0), S.t_isz);
    const float il = fdv(1.0f, fsq(fa(fa(fm(dx, dx), 1.0f), fm(dz, dz))));
    t.nx = fm(-dx, il);
    t.ny = il;
    t.nz = fm(-dz, il);
    int in = (int)fa(fx, 0.5f), jn = (int)fa(fz, 0.5f);
    if (in > S.tw - 1) in = S.tw - 1;
    if (jn > S.td - 1) jn = S.td - 1;
    t.vnear = jn * S.tw + in;
    return t;
}

// collisionS (fluid_system.h:355-407) for a box with centre c, half extents
// l and axis weights w (exactly 1 for the reference's cube).
__device__ __forceinline__ bool box_collide(const SceneDev& S, float px, float py, float pz, float* cp,
                                            float* nrm) {
    const float q[3] = {fs(px, S.box_c[0]), fs(py, S.box_c[1]), fs(pz, S.box_c[2])};
    const float aq[3] = {fabsf(q[0]), fabsf(q[1]), fabsf(q[2])};
    if (aq[0] < S.box_l[0] && aq[1] < S.box_l[1] && aq[2] < S.box_l[2]) return false;
    const float m0 = fm(aq[0], S.box_w[0]), m1 = fm(aq[1], S.box_w[1]), m2 = fm(aq[2], S.box_w[2]);
    int ax = 0;
    float maxp = m0;
    if (maxp < m1) {
        ax = 1;
        maxp = m1;
    }
    if (maxp < m2) ax = 2;
    cp[0] = px;
    cp[1] = py;
    cp[2] = pz;
    nrm[0] = nrm[1] = nrm[2] = 0.0f;
    float v, s;
    if (q[ax] < -S.box_l[ax]) {
        v = fs(S.box_c[ax], S.box_l[ax]);
        s = 1.0f;
    } else {
        v = fa(S.box_c[ax], S.box_l[ax]);
        s = -1.0f;
    }
    cp[ax] = v;
    nrm[ax] = s;
    return true;
}

__device__ __forceinline__ float len3(float x, float y, float z) { return fsq(dist2(x, y, z)); }

// ---------------------------------------------------------------------------
// Runs of equal values among the valid lanes of a warp (the valid lanes are a
// prefix, `mask`): the first lane of each run adds the run's length to
// counter[v] and every lane gets old value + its position in the run.  The
// state arrives in the previous step's sorted order, so particles of one cell
// are mostly adjacent and one atomic serves each cell.  Split in three phases
// so that several independent runs can have their atomics in flight at once.
struct Run {
    bool start;
    int leader;
    uint32_t len;
};

__device__ __forceinline__ Run run_of(uint32_t v, unsigned mask, int lane) {
    const uint32_t prev = __shfl_up_sync(mask, v, 1);
    Run r;
    r.start = lane == 0 || prev != v;
    const unsigned starts = __ballot_sync(mask, r.start);
    const unsigned upto = (2u << lane) - 1u;  // lanes 0..lane (all lanes for lane 31)
    r.leader = 31 - __clz(starts & upto);
    const unsigned above = starts & ~upto;
    const int end = above ? __ffs(above) - 1 : 32 - __clz(mask);
    r.len = (uint32_t)(end - lane);
    return r;
}

// keys: cell key of each particle, its slot within the cell (run-aggregated
// atomics) and the per-chunk totals that the scan needs.  Each block takes
// kKeyTiles consecutive work items, with their loads, then their atomics,
// then their shuffles issued together.
constexpr int kKeyTiles = 4;

__global__ void __launch_bounds__(kMaxTile) k_keys(DevArrays a) {
    const int nwork = *a.n_ptiles;
    const int lane = threadIdx.x & 31;
    for (int w0 = blockIdx.x * kKeyTiles; w0 < nwork; w0 += gridDim.x * kKeyTiles) {
        bool valid[kKeyTiles];
        int idx[kKeyTiles];
        uint32_t k[kKeyTiles], gk[kKeyTiles], ck[kKeyTiles];
        float4 x[kKeyTiles];
#pragma unroll
        for (int u = 0; u < kKeyTiles; ++u) {
            valid[u] = false;
            idx[u] = 0;
            const int w = w0 + u;
            if (w < nwork) {
                const Work wk = a.ptiles[w];
                if (a.steps_left[wk.scene] != 0) {
                    const SceneDev& S = a.scenes[wk.scene];
                    idx[u] = wk.start + threadIdx.x;
                    valid[u] = idx[u] < S.p_off + S.n;
                    if (valid[u]) x[u] = a.pos[idx[u]];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kKeyTiles; ++u) {
            if (!valid[u]) continue;
            const SceneDev& S = a.scenes[a.ptiles[w0 + u].scene];
            const Cell c = cell_of(S, x[u].x, x[u].y, x[u].z);
            k[u] = row_key(a.tab, S, c.cy, c.cz) + (uint32_t)c.cx;
            gk[u] = (uint32_t)S.k_off + k[u];
            ck[u] = (uint32_t)S.c_off + (k[u] >> kChunkBits);
        }
        Run rk[kKeyTiles];
        uint32_t base[kKeyTiles];
#pragma unroll
        for (int u = 0; u < kKeyTiles; ++u) {
            const unsigned mask = __ballot_sync(kFull, valid[u]);
            base[u] = 0;
            if (!valid[u]) continue;
            rk[u] = run_of(gk[u], mask, lane);
            const Run rc = run_of(ck[u], mask, lane);
            if (rk[u].start) base[u] = atomicAdd(a.counts + gk[u], rk[u].len);
            if (rc.start) atomicAdd(a.chunk_sum + ck[u], rc.len);
        }
#pragma unroll
        for (int u = 0; u < kKeyTiles; ++u) {
            const unsigned mask = __ballot_sync(kFull, valid[u]);
            if (!valid[u]) continue;
            const uint32_t b = __shfl_sync(mask, base[u], rk[u].leader);
            a.key[idx[u]] = k[u];
            a.slot[idx[u]] = b + (uint32_t)(lane - rk[u].leader);
        }
    }
}

template <int NT>
__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    uint32_t t = 0;
#pragma unroll
    for (int q = 0; q < NT / 32; ++q) t += sh[q];
    return t;
}

template <int NT>
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t u = __shfl_up_sync(kFull, inc, o);
        if (lane >= o) inc += u;
    }
    __syncthreads();
    if (lane == 31) sh[wid] = inc;
    __syncthreads();
    uint32_t before = 0;
#pragma unroll
    for (int q = 0; q < NT / 32; ++q)
        if (q < wid) before += sh[q];
    return before + inc - v;
}

// scan: exclusive prefix of the per-key counts within each scene, one chunk
// of kChunk keys per work item.  The chunk's offset is the sum of the earlier
// chunk totals of its scene, so no block waits on another.  Counts are
// cleared for the next step.
__global__ void __launch_bounds__(kScanThreads) k_scan(DevArrays a) {
    __shared__ uint32_t sh[kScanThreads / 32];
    const int nwork = *a.n_ctiles;
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const Work wk = a.ctiles[w];
        if (a.steps_left[wk.scene] == 0) continue;
        const SceneDev& S = a.scenes[wk.scene];
        const int c = wk.start;
        uint32_t pre = 0;
        for (int j = threadIdx.x; j < c; j += kScanThreads) pre += a.chunk_sum[S.c_off + j];
        pre = block_sum<kScanThreads>(pre, sh);
        const size_t base = (size_t)S.k_off + (size_t)c * kChunk + (size_t)threadIdx.x * 16;
        uint4* cp = reinterpret_cast<uint4*>(a.counts + base);
        uint32_t v[16];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint4 t = cp[q];
            v[4 * q] = t.x;
            v[4 * q + 1] = t.y;
            v[4 * q + 2] = t.z;
            v[4 * q + 3] = t.w;
        }
        uint32_t run = 0;
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            uint32_t t = v[q];
            v[q] = run;
            run += t;
        }
        const uint32_t add = pre + block_exclusive<kScanThreads>(run, sh);
        uint4* op = reinterpret_cast<uint4*>(a.offsets + base);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            op[q] = make_uint4(v[4 * q] + add, v[4 * q + 1] + add, v[4 * q + 2] + add, v[4 * q + 3] + add);
            cp[q] = make_uint4(0u, 0u, 0u, 0u);
        }
        __syncthreads();
    }
}

// scatter: place each particle's index at its cell's offset + slot, and clear
// the chunk totals (the scan that read them has finished).
__global__ void __launch_bounds__(kMaxTile) k_scatter(DevArrays a) {
    const int nwork = *a.n_ptiles;
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const Work wk = a.ptiles[w];
        if (a.steps_left[wk.scene] == 0) continue;
        const SceneDev& S = a.scenes[wk.scene];
        const int i = wk.start + threadIdx.x;
        if (i < S.p_off + S.n) {
            const uint32_t dst = a.offsets[S.k_off + a.key[i]] + a.slot[i];
            if (dst < (uint32_t)S.n)
                a.perm[S.p_off + dst] = (uint32_t)i;
            else
                atomicOr(a.status, 2u);  // inconsistent counts: never write out of range
        }
        const int t = (wk.start - S.p_off) / (int)blockDim.x;
        const int ntiles = (S.n + (int)blockDim.x - 1) / (int)blockDim.x;
        for (int j = t * (int)blockDim.x + (int)threadIdx.x; j < S.nchunks; j += ntiles * (int)blockDim.x)
            a.chunk_sum[S.c_off + j] = 0u;
    }
}

// reorder: make the order within each cell stable (ascending previous index,
// so results never depend on atomic arrival order) and gather the state into
// the sorted arrays.
__global__ void __launch_bounds__(kMaxTile) k_reorder(DevArrays a) {
    const int nwork = *a.n_ptiles;
    if (a.ctr && blockIdx.x == 0 && threadIdx.x < 2) a.ctr[threadIdx.x] = 0u;  // for this step's neighbour kernels
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const Work wk = a.ptiles[w];
        if (a.steps_left[wk.scene] == 0) continue;
        const SceneDev& S = a.scenes[wk.scene];
        const int p = wk.start + threadIdx.x;
        if (p >= S.p_off + S.n) continue;
        const uint32_t i = a.perm[p];
        if (i < (uint32_t)S.p_off || i >= (uint32_t)(S.p_off + S.n)) {
            atomicOr(a.status, 2u);
            continue;
        }
        const uint32_t k = a.key[i];
        const uint32_t st = a.offsets[S.k_off + k];
        const uint32_t en = min(a.offsets[S.k_off + k + 1], (uint32_t)S.n);
        const uint32_t* cell = a.perm + S.p_off;
        uint32_t r = 0;
        for (uint32_t q = st; q < en; ++q) r += (cell[q] < i) ? 1u : 0u;
        if (st + r >= (uint32_t)S.n) {
            atomicOr(a.status, 2u);
            continue;
        }
        const int dst = S.p_off + (int)(st + r);
        a.spos[dst] = a.pos[i];
        a.svel[dst] = a.vel[i];
        if (S.flags & kFlagRecord) a.snbid[dst] = a.nbid[i];
    }
}

// Work slices of the neighbour kernels.  Static: block b takes the tiles b,
// b + gridDim.x, ..., and its thread t the tile's lane t.  Dynamic (DYN):
// every warp takes the next 32-lane slice of any tile from a counter, so no
// warp slot waits for the slowest warp of its block.  Which warp computes a
// particle changes nothing in what it computes.
template <bool DYN>
__device__ __forceinline__ int next_slice(unsigned* ctr, int cur) {
    if (!DYN) return cur + (int)gridDim.x;
    int t = 0;
    if ((threadIdx.x & 31) == 0) t = (int)atomicAdd(ctr, 1u);
    return __shfl_sync(kFull, t, 0);
}

template <bool DYN>
__device__ __forceinline__ int first_slice(unsigned* ctr) {
    return DYN ? next_slice<true>(ctr, 0) : (int)blockIdx.x;
}

// density: pass 1 (fluid_system.h:107-124), then the per-particle factors the
// force pass reuses: P/rho^2 and m/rho.
// LISTED: the in-range pairs are compacted (for_each_in_range_listed) instead
// of evaluated inside the candidate loop; which one is faster depends on the
// neighbour density, so the autotuner picks it.
template <bool ORDERED, bool LISTED, int MINB, bool NL = false, bool X2 = false, bool PACK = false,
          bool DYN = false, bool FM = false>
__global__ void __launch_bounds__(kMaxTile, MINB) k_density(DevArrays a) {
    extern __shared__ uint32_t list[];
    const int nwork = *a.n_ptiles;
    const int spt = DYN ? a.tile / 32 : 1;  // slices per tile
    for (int sl = first_slice<DYN>(a.ctr); sl < nwork * spt; sl = next_slice<DYN>(a.ctr, sl)) {
        const int w = DYN ? sl / spt : sl;
        const int li = DYN ? (sl % spt) * 32 + (int)(threadIdx.x & 31) : (int)threadIdx.x;  // lane within the tile
        const int stride = DYN ? a.tile : (int)blockDim.x;
        const Work wk = a.ptiles[w];
        if (a.steps_left[wk.scene] == 0) continue;
        const SceneDev S = a.scenes[wk.scene];  // by value: the list stores cannot alias it
        if (((S.flags & kFlagOrdered) != 0) != ORDERED) continue;
        const int p = wk.start + li;
        const bool valid = p < S.p_off + S.n;
        if ((ORDERED || !LISTED) && !valid) continue;
        const float4 xi = a.spos[valid ? p : S.p_off];
        float rho = 0.0f;
        if (ORDERED) {
            auto term = [&](uint32_t, float4 xj) {
                float s = dist2(fs(xi.x, xj.x), fs(xi.y, xj.y), fs(xi.z, xj.z));
                if (s <= S.smax) rho = fa(rho, density_term(S, fsq(s)));
            };
            if (!for_each_in_range_ordered(a, S, xi, term)) atomicOr(a.status, 1u);
        } else if (LISTED) {
            const float4* sp = a.spos + S.p_off;
            for_each_in_range_listed(a, S, valid, xi, list, [&](uint32_t j) {
                const float4 xj = __ldg(sp + j);
                const float s = dist2(fs(xi.x, xj.x), fs(xi.y, xj.y), fs(xi.z, xj.z));
                rho = fa(rho, density_term(S, fsq(s)));
            });
            if (!valid) continue;
        } else {
            // NL: the in-range candidates, in visiting order, also go to the
            // particle's neighbour list for the force pass
            uint32_t* nl = a.nlist + (size_t)wk.start * kNbCap + li;
            int cnt = 0;
            auto visit = [&](uint32_t j, float4 xj) {
                const float s = dist2(fs(xi.x, xj.x), fs(xi.y, xj.y), fs(xi.z, xj.z));
                if (s <= S.smax) {
                    if (FM)
                        rho += density_term_fast(S, s);
                    else
                        rho = fa(rho, density_term(S, fsq(s)));
                    if (NL) {
                        if (cnt < kNbCap) nl[(size_t)cnt * stride] = j;
                        ++cnt;
                    }
                }
            };
            if (X2) {
                for_each_candidate_x2(a, S, xi, visit);
            } else {
                for_each_candidate(a, S, xi, visit);
            }
            if (NL) a.ncnt[p] = cnt;
        }
        const float P = fm(S.k, fs(rho, S.p0));
        const float Ai = fdv(P, fm(rho, rho)), Bi = fdv(S.mass, rho);
        a.dyn[p] = make_float4(rho, Ai, Bi, P);
        if (PACK) {
            const float4 vi = a.svel[p];
            a.fdat[2 * (size_t)p] = make_float4(xi.x, xi.y, xi.z, Ai);
            a.fdat[2 * (size_t)p + 1] = make_float4(vi.x, vi.y, vi.z, Bi);
        }
    }
}

// Pass-2 results (fluid_system.h:151-154), pass 3 (:163, :177) and advance
// (:306-353) with the terrain contact, the box collision and the erosion
// exchange, from a particle's neighbour sums; only a writer stores the state
// and the record and adds the exchange to the terrain.
__device__ __forceinline__ void integrate_and_store(const DevArrays& a, const SceneDev& S, int p, float4 xi, float4 vi,
                                                    float rho, const ForceAcc& acc, bool writer) {
    // pass-2 results (:151-154) and pass 3 (:163, :177)
    const float Fpx = -fm(acc.fpx, rho), Fpy = -fm(acc.fpy, rho), Fpz = -fm(acc.fpz, rho);
    const float Fvx = fm(acc.fvx, S.visc), Fvy = fm(acc.fvy, S.visc), Fvz = fm(acc.fvz, S.visc);
    const float Fgx = fm(rho, S.g[0]), Fgy = fm(rho, S.g[1]), Fgz = fm(rho, S.g[2]);
    const float nsig = fm(-S.sigma, acc.cfl);
    const float Fsx = fm(nsig, acc.nx), Fsy = fm(nsig, acc.ny), Fsz = fm(nsig, acc.nz);
    // advance (:318-331)
    const float Fx = fa(fa(Fpx, Fvx), fa(Fgx, Fsx));
    const float Fy = fa(fa(Fpy, Fvy), fa(Fgy, Fsy));
    const float Fz = fa(fa(Fpz, Fvz), fa(Fgz, Fsz));
    const float ax = fdv(Fx, rho), ay = fdv(Fy, rho), az = fdv(Fz, rho);
    const float dt = S.dt;
    float vx = fa(vi.x, fm(ax, dt)), vy = fa(vi.y, fm(ay, dt)), vz = fa(vi.z, fm(az, dt));
    float px = fa(xi.x, fm(vx, dt)), py = fa(xi.y, fm(vy, dt)), pz = fa(xi.z, fm(vz, dt));

    const bool has_t = (S.flags & kFlagTerrain) != 0;
    TSample ts;
    if (has_t) {
        ts = terrain_at(S, a.theight, px, pz);
        if (py < ts.y && dt != 0.0f) {
            const float d = fs(ts.y, py);
            const float vdn = fa(fa(fm(vx, ts.nx), fm(vy, ts.ny)), fm(vz, ts.nz));
            if (vdn < 0.0f) {
                const float sp = len3(vx, vy, vz);
                const float f = fa(1.0f, sp > 0.0f ? fdv(fm(S.cr, d), fm(dt, sp)) : 0.0f);
                vx = fs(vx, fm(fm(ts.nx, f), vdn));
                vy = fs(vy, fm(fm(ts.ny, f), vdn));
                vz = fs(vz, fm(fm(ts.nz, f), vdn));
            }
            py = ts.y;
        }
    }
    bool moved = false;
    {
        float cp[3], nr[3];
        if (box_collide(S, px, py, pz, cp, nr) && dt != 0.0f) {
            const float d = len3(fs(px, cp[0]), fs(py, cp[1]), fs(pz, cp[2]));
            const float f = fa(1.0f, fdv(fm(0.5f, d), fm(dt, len3(vx, vy, vz))));
            const float vdn = fa(fa(fm(vx, nr[0]), fm(vy, nr[1])), fm(vz, nr[2]));
            vx = fs(vx, fm(fm(nr[0], f), vdn));
            vy = fs(vy, fm(fm(nr[1], f), vdn));
            vz = fs(vz, fm(fm(nr[2], f), vdn));
            moved = px != cp[0] || pz != cp[2];
            px = cp[0];
            py = cp[1];
            pz = cp[2];
        }
    }
    int sed = __float_as_int(vi.w);
    if (has_t && (S.flags & kFlagErosion)) {
        // the exchange uses the surface under the particle's final
        // position: a wall that moved it in x or z moved it to another
        // sample of the terrain
        if (moved) ts = terrain_at(S, a.theight, px, pz);
        const float e = fs(py, ts.y);
        if (e <= S.layer) {
            float capf = fm(S.k_capacity, len3(vx, vy, vz));
            if (capf > 1.0f) capf = 1.0f;
            const float cap = fm(capf, 1073741824.0f);
            const float s = __int2float_rn(sed);
            const float q = (s < cap) ? fm(fm(S.k_pick, dt), fs(cap, s)) : -fm(fm(S.k_dep, dt), fs(s, cap));
            if (q == q) {
                long long Q = __float2ll_rn(q);
                if ((long long)sed + Q < 0) Q = -(long long)sed;
                if ((long long)sed + Q > 1073741824LL) Q = 1073741824LL - (long long)sed;
                if (Q != 0) {
                    sed += (int)Q;
                    if (writer)
                        atomicAdd(reinterpret_cast<unsigned long long*>(a.tdelta + S.t_off + ts.vnear),
                                  (unsigned long long)(-Q));
                }
            }
        }
    }
    if (!writer) return;
    a.pos[p] = make_float4(px, py, pz, xi.w);
    a.vel[p] = make_float4(vx, vy, vz, __int_as_float(sed));
    if (S.flags & kFlagRecord) {
        float* r = a.rec + (size_t)p * kRecFloats;
        r[0] = ax; r[1] = ay; r[2] = az;
        r[3] = Fpx; r[4] = Fpy; r[5] = Fpz;
        r[6] = Fvx; r[7] = Fvy; r[8] = Fvz;
        r[9] = Fgx; r[10] = Fgy; r[11] = Fgz;
        r[12] = Fsx; r[13] = Fsy; r[14] = Fsz;
        r[15] = acc.nx; r[16] = acc.ny; r[17] = acc.nz;
        a.nbid[p] = acc.any ? acc.nb : a.snbid[p];
    }
}

// force: passes 2 and 3 (fluid_system.h:127-178) and advance (:306-353) with
// the terrain contact, the box collision and the erosion exchange.
// NL: the in-range neighbours come from the lists the density pass wrote
// (same order as the traversal, so the same sums); a particle whose list
// overflowed walks its cells instead.  NL = 2
// software-pipelines the list walk: list entries two ahead and the
// neighbour's state one ahead are loaded before the current pair is summed.
template <bool ORDERED, int MINB, int NL = 0, bool DYN = false, bool FM = false>
__global__ void __launch_bounds__(kMaxTile, MINB) k_force(DevArrays a) {
    extern __shared__ uint32_t list[];
    const int nwork = *a.n_ptiles;
    const int spt = DYN ? a.tile / 32 : 1;  // slices per tile
    for (int sl = first_slice<DYN>(a.ctr + 1); sl < nwork * spt; sl = next_slice<DYN>(a.ctr + 1, sl)) {
        const int w = DYN ? sl / spt : sl;
        const int li = DYN ? (sl % spt) * 32 + (int)(threadIdx.x & 31) : (int)threadIdx.x;  // lane within the tile
        const int lstride = DYN ? a.tile : (int)blockDim.x;
        const Work wk = a.ptiles[w];
        if (a.steps_left[wk.scene] == 0) continue;
        const SceneDev& S = a.scenes[wk.scene];
        if (((S.flags & kFlagOrdered) != 0) != ORDERED) continue;
        const int p0 = wk.start + li;
        const bool valid = p0 < S.p_off + S.n;
        if (ORDERED && !valid) continue;
        const int p = valid ? p0 : S.p_off;
        const int pl = p - S.p_off;
        const float4 xi = a.spos[p];
        const float4 vi = a.svel[p];
        const float4 di = a.dyn[p];
        const float rho = di.x, Ai = di.y;
        ForceAcc acc = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, -1, 0};
        const float4* sp = a.spos + S.p_off;
        const float4* sv = a.svel + S.p_off;
        const float4* sd = a.dyn + S.p_off;
        auto pair_with = [&](uint32_t j, float4 xj, float4 vj, float4 dj) {
            const float rx = fs(xi.x, xj.x), ry = fs(xi.y, xj.y), rz = fs(xi.z, xj.z);
            const float s = FM ? dist2_fma(rx, ry, rz) : dist2(rx, ry, rz);
            if (FM)
                force_pair_fast(S, acc, rx, ry, rz, s, vi.x, vi.y, vi.z, Ai, vj, dj.y, dj.z, __float_as_int(xj.w),
                                (int)j == pl);
            else
                force_pair(S, acc, rx, ry, rz, fsq(s), vi.x, vi.y, vi.z, Ai, vj, dj.y, dj.z, __float_as_int(xj.w),
                           (int)j == pl);
        };
        auto pair = [&](uint32_t j, float4 xj) { pair_with(j, xj, __ldg(sv + j), __ldg(sd + j)); };
        if (ORDERED) {
            // the ordered list holds only in-range candidates
            if (!for_each_in_range_ordered(a, S, xi, pair)) atomicOr(a.status, 1u);
        } else {
            const int cnt = (NL && valid) ? a.ncnt[p] : 0;
            if (!NL) {
                for_each_in_range_listed(a, S, valid, xi, list, [&](uint32_t j) { pair(j, __ldg(sp + j)); });
            } else if (cnt > kNbCap) {
                // the list overflowed: this lane walks its cells (same order)
                for_each_candidate(a, S, xi, [&](uint32_t j, float4 xj) {
                    if (dist2(fs(xi.x, xj.x), fs(xi.y, xj.y), fs(xi.z, xj.z)) <= S.smax) pair(j, xj);
                });
            } else if (NL == 1) {
                const uint32_t* nl = a.nlist + (size_t)wk.start * kNbCap + li;
                for (int q = 0; q < cnt; ++q) {
                    const uint32_t j = __ldg(nl + (size_t)q * lstride);
                    pair(j, __ldg(sp + j));
                }
            } else if (NL == 2) {
                const uint32_t* nl = a.nlist + (size_t)wk.start * kNbCap + li;
                const int stride = lstride;
                uint32_t j0 = cnt > 0 ? __ldg(nl) : 0u;
                uint32_t j1 = cnt > 1 ? __ldg(nl + stride) : 0u;
                float4 x0 = make_float4(0.f, 0.f, 0.f, 0.f), v0 = x0, d0 = x0;
                if (cnt > 0) {
                    x0 = __ldg(sp + j0);
                    v0 = __ldg(sv + j0);
                    d0 = __ldg(sd + j0);
                }
                nl += 2 * stride;
                for (int q = 0; q < cnt; ++q, nl += stride) {
                    const uint32_t j2 = (q + 2 < cnt) ? __ldg(nl) : 0u;
                    float4 x1 = x0, v1 = v0, d1 = d0;
                    if (q + 1 < cnt) {
                        x1 = __ldg(sp + j1);
                        v1 = __ldg(sv + j1);
                        d1 = __ldg(sd + j1);
                    }
                    pair_with(j0, x0, v0, d0);
                    j0 = j1;
                    j1 = j2;
                    x0 = x1;
                    v0 = v1;
                    d0 = d1;
                }
            } else {
                // NL == 3: the same walk over the packed 32-byte records (one
                // sector per neighbour); the id is read only in record mode
                const uint32_t* nl = a.nlist + (size_t)wk.start * kNbCap + li;
                const int stride = lstride;
                const float4* fd = a.fdat + 2 * (size_t)S.p_off;
                const bool rec = (S.flags & kFlagRecord) != 0;
                uint32_t j0 = cnt > 0 ? __ldg(nl) : 0u;
                uint32_t j1 = cnt > 1 ? __ldg(nl + stride) : 0u;
                float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), b0 = a0;
                if (cnt > 0) ld_record(fd + 2 * j0, a0, b0);
                nl += 2 * stride;
                for (int q = 0; q < cnt; ++q, nl += stride) {
                    const uint32_t j2 = (q + 2 < cnt) ? __ldg(nl) : 0u;
                    float4 a1 = a0, b1 = b0;
                    if (q + 1 < cnt) ld_record(fd + 2 * j1, a1, b1);
                    const int idj = rec ? __float_as_int(__ldg(&sp[j0].w)) : 0;
                    const float rx = fs(xi.x, a0.x), ry = fs(xi.y, a0.y), rz = fs(xi.z, a0.z);
                    if (FM)
                        force_pair_fast(S, acc, rx, ry, rz, dist2_fma(rx, ry, rz), vi.x, vi.y, vi.z, Ai, b0, a0.w, b0.w,
                                        idj, (int)j0 == pl);
                    else
                        force_pair(S, acc, rx, ry, rz, fsq(dist2(rx, ry, rz)), vi.x, vi.y, vi.z, Ai, b0, a0.w, b0.w,
                                   idj, (int)j0 == pl);
                    j0 = j1;
                    j1 = j2;
                    a0 = a1;
                    b0 = b1;
                }
            }
            if (!valid) continue;
        }
        integrate_and_store(a, S, p, xi, vi, rho, acc, true);
    }
}

// ---------------------------------------------------------------------------
// Cooperative neighbour passes (variant bit 8): a group of G lanes shares one
// particle.  The lists the density pass hands to the force pass are
// particle-major here (particle p's entries at p * kNbCap + q), which both
// passes read and write in contiguous runs.

// Range [st, en) of stencil row r of the particle at probe q: rows in the
// order of for_rows (dz outer, dy inner, both ascending), trimmed the same
// way, so a particle's candidates come in the same order.  gx2 holds the
// squared x-gaps, in y/z cell units, of the x cells cx - 2 .. cx + 2 (R = 1
// with xsub 2, R = 2 with xsub 1; unused for R = 0, the general reach).
template <int R>
__device__ __forceinline__ void stencil_row(const DevArrays& a, const SceneDev& S, const Probe& q, const float* gx2,
                                            int r, uint32_t& st, uint32_t& en) {
    st = en = 0;
    const int side = R > 0 ? 2 * R + 1 : 2 * S.reach + 1;
    const int reach = R > 0 ? R : S.reach;
    const int dz = r / side - reach, dy = r % side - reach;
    const int z = q.c.cz + dz, y = q.c.cy + dy;
    if (!q.finite || z < 0 || z >= S.nz || y < 0 || y >= S.ny) return;
    const uint32_t* off = a.offsets + S.k_off;
    if (R > 0) {
        const float gz = cell_gap(q.tz, z, S.nz), gy = cell_gap(q.ty, y, S.ny);
        const float r2 = S.hcell * S.hcell - gy * gy - gz * gz;
        if (!(r2 >= 0.0f)) return;
        int lo = 0, hi = 0;
        constexpr int RX = (R > 0 ? R : 1) * (R == 1 ? 2 : 1);
#pragma unroll
        for (int d = 1; d <= RX; ++d) {
            if (gx2[RX - d] <= r2) lo = -d;
            if (gx2[RX + d] <= r2) hi = d;
        }
        const uint32_t row = row_key(a.tab, S, y, z);
        st = __ldg(off + row + q.c.cx + lo);
        en = __ldg(off + row + q.c.cx + hi + 1);
    } else {
        int xl, xh;
        if (!row_span(S, q, y, z, &xl, &xh)) return;
        const uint32_t row = row_key(a.tab, S, y, z);
        st = __ldg(off + row + xl);
        en = __ldg(off + row + xh + 1);
    }
}

// Group geometry of G lanes per particle (G a power of two, 4..32).
template <int G>
struct Group {
    int gl;         // lane within the group
    int gbase;      // first lane of the group within the warp
    unsigned mask;  // the group's lanes
    __device__ __forceinline__ Group() {
        const int lane = threadIdx.x & 31;
        gl = lane & (G - 1);
        gbase = lane & ~(G - 1);
        mask = G == 32 ? kFull : (((1u << G) - 1u) << gbase);
    }
};

// Sum over the group, the same bits in every lane (each butterfly step adds
// two equal-rounded operands in either order), in a fixed order.
template <int G>
__device__ __forceinline__ float group_sum(float v, unsigned mask) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v = fa(v, __shfl_xor_sync(mask, v, o, G));
    return v;
}

// density, cooperative: the group walks the particle's candidates as one
// stream (row after row, ascending index within a row) in windows of G, one
// candidate per lane, so neighbouring lanes load neighbouring particles.
// Each lane sums its candidates' terms in stream order; the group's partial
// sums are combined by group_sum.  In-range candidates are appended to the
// particle's list in stream order (ballot + prefix count).
template <int G, int R, bool PACK>
__device__ __forceinline__ void density_coop_particle(const DevArrays& a, const SceneDev& S, int p, int* soff,
                                                      const Group<G>& g) {
    const float4 xi = a.spos[p];
    const Probe q = probe_of(S, xi);
    constexpr int XS = R == 1 ? 2 : 1;  // the scene's xsub at this reach
    constexpr int RX = (R > 0 ? R : 1) * XS;
    float gx2[2 * RX + 1];  // squared x-gaps in y/z cell units
    if (R > 0) {
#pragma unroll
        for (int d = -RX; d <= RX; ++d) {
            const int k = q.c.cx + d;
            float g2 = INFINITY;
            if (k >= 0 && k < S.nx) {
                const float gg = cell_gap(q.tx, k, S.nx) * (1.0f / XS);
                g2 = gg * gg;
            }
            gx2[d + RX] = g2;
        }
    }
    const float4* sp = a.spos + S.p_off;
    uint32_t* nl = a.nlist + (size_t)p * kNbCap;
    const int side = R > 0 ? 2 * R + 1 : 2 * S.reach + 1;
    const int nrows = side * side;
    float rho = 0.0f;
    int cnt = 0;
    const unsigned below = (1u << g.gl) - 1u;
    for (int rb = 0; rb < nrows; rb += G) {
        uint32_t st = 0, en = 0;
        if (rb + g.gl < nrows) stencil_row<R>(a, S, q, gx2, rb + g.gl, st, en);
        const int len = (int)(en - st);
        int inc = len;
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            const int v = __shfl_up_sync(g.mask, inc, o, G);
            if (g.gl >= o) inc += v;
        }
        const int pre = inc - len;
        const int total = __shfl_sync(g.mask, inc, G - 1, G);
        int carry = 0;
        for (int wb = 0; wb < total; wb += G) {
            // the rows that start in this window record where their
            // candidates sit: candidate t of the stream is particle t + off
            const bool starts = len > 0 && pre >= wb && pre < wb + G;
            if (starts) soff[pre - wb] = (int)st - pre;
            const unsigned m = __reduce_or_sync(g.mask, starts ? (1u << (pre - wb)) : 0u);
            __syncwarp(g.mask);
            const unsigned upto = m & ((2u << g.gl) - 1u);
            const int off = upto ? soff[31 - __clz(upto)] : carry;
            carry = m ? soff[31 - __clz(m)] : carry;
            __syncwarp(g.mask);
            const int t = wb + g.gl;
            bool in = false;
            uint32_t j = 0;
            float s = 0.0f;
            if (t < total) {
                j = (uint32_t)(t + off);
                const float4 xj = __ldg(sp + j);
                s = dist2(fs(xi.x, xj.x), fs(xi.y, xj.y), fs(xi.z, xj.z));
                in = s <= S.smax;
            }
            if (in) rho = fa(rho, density_term(S, fsq(s)));
            const unsigned b = (__ballot_sync(g.mask, in) & g.mask) >> g.gbase;
            const int at = cnt + __popc(b & below);
            if (in && at < kNbCap) nl[at] = j;
            cnt += __popc(b);
        }
    }
    rho = group_sum<G>(rho, g.mask);
    if (g.gl == 0) {
        const float P = fm(S.k, fs(rho, S.p0));
        const float Ai = fdv(P, fm(rho, rho)), Bi = fdv(S.mass, rho);
        a.dyn[p] = make_float4(rho, Ai, Bi, P);
        a.ncnt[p] = cnt;
        if (PACK) {
            const float4 vi = a.svel[p];
            a.fdat[2 * (size_t)p] = make_float4(xi.x, xi.y, xi.z, Ai);
            a.fdat[2 * (size_t)p + 1] = make_float4(vi.x, vi.y, vi.z, Bi);
        }
    }
}

template <int G, bool PACK>
__global__ void __launch_bounds__(256) k_density_coop(DevArrays a) {
    __shared__ int s_off[256];
    const Group<G> g;
    int* soff = s_off + (threadIdx.x & ~(G - 1));
    const int group = threadIdx.x / G, ngroups = blockDim.x / G;
    const int nwork = *a.n_ptiles;
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const Work wk = a.ptiles[w];
        if (a.steps_left[wk.scene] == 0) continue;
        const SceneDev& S = a.scenes[wk.scene];
        if (S.flags & kFlagOrdered) continue;
        const int end = min(wk.start + (int)blockDim.x, S.p_off + S.n);
        for (int p = wk.start + group; p < end; p += ngroups) {
            if (S.reach == 2)
                density_coop_particle<G, 2, PACK>(a, S, p, soff, g);
            else if (S.reach == 1)
                density_coop_particle<G, 1, PACK>(a, S, p, soff, g);
            else
                density_coop_particle<G, 0, PACK>(a, S, p, soff, g);
        }
    }
}

// force, cooperative: the group splits the particle's list (lane gl takes
// entries gl, gl + G, ...), each lane sums its pairs' terms in list order,
// the group combines them with group_sum, and every lane of the group then
// holds the particle's sums; the integration, contacts and erosion are
// computed alike in every lane and written by lane 0.  A particle whose list
// overflowed has the group split its cell rows instead (row r to lane r mod G).
template <int G, bool PACK, int MINB>
__global__ void __launch_bounds__(256, MINB) k_force_coop(DevArrays a) {
    const Group<G> g;
    const int group = threadIdx.x / G, ngroups = blockDim.x / G;
    const int nwork = *a.n_ptiles;
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const Work wk = a.ptiles[w];
        if (a.steps_left[wk.scene] == 0) continue;
        const SceneDev& S = a.scenes[wk.scene];
        if (S.flags & kFlagOrdered) continue;
        const int end = min(wk.start + (int)blockDim.x, S.p_off + S.n);
        for (int p = wk.start + group; p < end; p += ngroups) {
            const int pl = p - S.p_off;
            const float4 xi = a.spos[p];
            const float4 vi = a.svel[p];
            const float4 di = a.dyn[p];
            const float rho = di.x, Ai = di.y;
            ForceAcc acc = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, -1, 0};
            const float4* sp = a.spos + S.p_off;
            const float4* sv = a.svel + S.p_off;
            const float4* sd = a.dyn + S.p_off;
            const bool rec = (S.flags & kFlagRecord) != 0;
            auto pair = [&](uint32_t j, float4 xj, float4 vj, float Aj, float Bj, int idj) {
                const float rx = fs(xi.x, xj.x), ry = fs(xi.y, xj.y), rz = fs(xi.z, xj.z);
                force_pair(S, acc, rx, ry, rz, fsq(dist2(rx, ry, rz)), vi.x, vi.y, vi.z, Ai, vj, Aj, Bj, idj,
                           (int)j == pl);
            };
            const int cnt = a.ncnt[p];
            if (cnt <= kNbCap) {
                const uint32_t* nl = a.nlist + (size_t)p * kNbCap;
                int qn = g.gl;
                uint32_t j0 = qn < cnt ? __ldg(nl + qn) : 0u;
                for (int qq = g.gl; qq < cnt; qq += G) {
                    qn += G;
                    const uint32_t j1 = qn < cnt ? __ldg(nl + qn) : 0u;  // next entry, loaded ahead
                    if (PACK) {
                        const float4* fd = a.fdat + 2 * (size_t)S.p_off;
                        const float4 r0 = __ldg(fd + 2 * j0), r1 = __ldg(fd + 2 * j0 + 1);
                        const int idj = rec ? __float_as_int(__ldg(&sp[j0].w)) : 0;
                        pair(j0, r0, r1, r0.w, r1.w, idj);
                    } else {
                        const float4 xj = __ldg(sp + j0), vj = __ldg(sv + j0), dj = __ldg(sd + j0);
                        pair(j0, xj, vj, dj.y, dj.z, __float_as_int(xj.w));
                    }
                    j0 = j1;
                }
            } else {
                int r = 0;
                for_rows(a, S, xi, true, [&](uint32_t st, uint32_t en) {
                    if ((r++ & (G - 1)) != g.gl) return;
                    for (uint32_t j = st; j < en; ++j) {
                        const float4 xj = __ldg(sp + j);
                        if (dist2(fs(xi.x, xj.x), fs(xi.y, xj.y), fs(xi.z, xj.z)) <= S.smax) {
                            const float4 vj = __ldg(sv + j), dj = __ldg(sd + j);
                            pair(j, xj, vj, dj.y, dj.z, __float_as_int(xj.w));
                        }
                    }
                });
            }
            acc.fpx = group_sum<G>(acc.fpx, g.mask);
            acc.fpy = group_sum<G>(acc.fpy, g.mask);
            acc.fpz = group_sum<G>(acc.fpz, g.mask);
            acc.fvx = group_sum<G>(acc.fvx, g.mask);
            acc.fvy = group_sum<G>(acc.fvy, g.mask);
            acc.fvz = group_sum<G>(acc.fvz, g.mask);
            acc.nx = group_sum<G>(acc.nx, g.mask);
            acc.ny = group_sum<G>(acc.ny, g.mask);
            acc.nz = group_sum<G>(acc.nz, g.mask);
            acc.cfl = group_sum<G>(acc.cfl, g.mask);
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) {
                acc.nb = max(acc.nb, __shfl_xor_sync(g.mask, acc.nb, o, G));
                acc.any |= __shfl_xor_sync(g.mask, acc.any, o, G);
            }
            integrate_and_store(a, S, p, xi, vi, rho, acc, g.gl == 0);
        }
    }
}

// ---------------------------------------------------------------------------
// Force pass with a TMA gather pipeline (variant bit 18, with lists, packed
// records and fast arithmetic).  Each block holds T consumer threads (one
// particle of the tile each) and one producer warp.  For list slot q the
// producer reads the T list entries (16-byte loads), keeps them in an index
// ring in shared memory and issues TMA tile::gather4 copies of the T packed
// records (rows of a 2-D tensor map over fdat, one row high) into a ring of
// stages in shared memory; each stage's copies complete on its `full`
// mbarrier, and the consumer warps release the stage through its `empty`
// mbarrier.  The consumers then sum the same pairs in the same order as the
// per-lane fast-arithmetic pass (the same bits), but their neighbour records
// come from shared memory and hold no registers while in flight.  Every wait
// is bounded by a clock limit; a wait that runs out sets status bit 2 and
// ends the block's work.
constexpr int kTmaRingBytes = 32768;  // record ring; stages = kTmaRingBytes / (T * 32)
constexpr long long kWaitLimit = 4000000000LL;  // clock cycles (about 2 s)

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Waits until the phase of parity `parity` has completed; false when the
// clock limit runs out first.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    const long long t0 = clock64();
    for (;;) {
        unsigned done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > kWaitLimit) return false;
    }
}

// Four rows (record indices) of the tensor map into 128 contiguous bytes of
// shared memory; rows outside the tensor read as zeros.
__device__ __forceinline__ void tma_gather4(void* dst, const CUtensorMap* map, int r0, int r1, int r2, int r3,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
        "%3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(smem_u32(bar))
        : "memory");
}

template <int MINB>
__global__ void __launch_bounds__(kMaxTile + 32, MINB) k_force_tma(DevArrays a, const __grid_constant__ CUtensorMap fmap) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ int s_m;
    const int T = (int)blockDim.x - 32;  // consumers: 128 or 256
    const int D = kTmaRingBytes / (T * 32);
    unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);  // TMA wants 128-B rows
    float4* ring = reinterpret_cast<float4*>(smem);  // stage s, lane l: ring[2 * (s * T + l) + {0, 1}]
    uint32_t* jring = reinterpret_cast<uint32_t*>(smem + kTmaRingBytes);  // stage s, lane l: jring[s * T + l]
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + kTmaRingBytes + (size_t)D * T * 4);
    uint64_t* empty = full + D;
    const int tid = threadIdx.x, lane = tid & 31;
    const bool producer = tid >= T;
    if (tid == 0) {
        for (int q = 0; q < D; ++q) {
            mbar_init(full + q, 1);
            mbar_init(empty + q, (unsigned)(T / 32));
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    unsigned it = 0;  // ring slots this block has used
    bool ok = true;
    const int nwork = *a.n_ptiles;
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const Work wk = a.ptiles[w];
        if (a.steps_left[wk.scene] == 0) continue;
        const SceneDev& S = a.scenes[wk.scene];
        if (S.flags & kFlagOrdered) continue;
        const int end = S.p_off + S.n;
        if (producer) {
            int m = 0;
            for (int l = lane; l < T; l += 32) {
                const int p = wk.start + l;
                if (p < end) m = max(m, min(a.ncnt[p], kNbCap));
            }
            for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(kFull, m, o));
            if (lane == 0) s_m = ok ? m : 0;
        }
        __syncthreads();
        const int M = s_m;  // list slots in use in this tile
        if (producer) {
            const uint32_t* nl = a.nlist + (size_t)wk.start * kNbCap;
            const int per = T / 32;  // consumer lanes per producer lane
            for (int q = 0; q < M && ok; ++q) {
                const unsigned i2 = it + (unsigned)q, st = i2 % (unsigned)D, ph = (i2 / (unsigned)D) & 1u;
                if (i2 >= (unsigned)D && !mbar_wait(empty + st, ph ^ 1u)) {
                    ok = false;
                    break;
                }
                const uint32_t* e = nl + (size_t)q * T + per * lane;
                uint4 jj[2];
                for (int g = 0; g < per; g += 4) {
                    jj[g / 4] = *reinterpret_cast<const uint4*>(e + g);
                    *reinterpret_cast<uint4*>(jring + (size_t)st * T + per * lane + g) = jj[g / 4];
                }
                __syncwarp();
                if (lane == 0) mbar_arrive_expect_tx(full + st, (unsigned)(T * 32));
                for (int g = 0; g < per; g += 4) {
                    const uint4 v = jj[g / 4];
                    tma_gather4(ring + 2 * ((size_t)st * T + per * lane + g), &fmap, S.p_off + (int)v.x,
                                S.p_off + (int)v.y, S.p_off + (int)v.z, S.p_off + (int)v.w, full + st);
                }
            }
        } else {
            const int p0 = wk.start + tid;
            const bool valid = p0 < end;
            const int p = valid ? p0 : S.p_off;
            const int pl = p - S.p_off;
            const float4 xi = a.spos[p];
            const float4 vi = a.svel[p];
            const float4 di = a.dyn[p];
            const float rho = di.x, Ai = di.y;
            const int cnt = valid ? a.ncnt[p] : 0;
            const bool listed = cnt <= kNbCap;
            const bool rec = (S.flags & kFlagRecord) != 0;
            const float4* sp = a.spos + S.p_off;
            ForceAcc acc = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, -1, 0};
            for (int q = 0; q < M; ++q) {
                const unsigned i2 = it + (unsigned)q, st = i2 % (unsigned)D, ph = (i2 / (unsigned)D) & 1u;
                if (ok && !mbar_wait(full + st, ph)) ok = false;
                if (ok && listed && q < cnt) {
                    const float4 r0 = ring[2 * ((size_t)st * T + tid)], r1 = ring[2 * ((size_t)st * T + tid) + 1];
                    const uint32_t j = jring[(size_t)st * T + tid];
                    const int idj = rec ? __float_as_int(__ldg(&sp[j].w)) : 0;
                    const float rx = fs(xi.x, r0.x), ry = fs(xi.y, r0.y), rz = fs(xi.z, r0.z);
                    force_pair_fast(S, acc, rx, ry, rz, dist2_fma(rx, ry, rz), vi.x, vi.y, vi.z, Ai, r1, r0.w, r1.w, idj,
                                    (int)j == pl);
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(empty + st);
            }
            if (valid && !listed) {
                // the list overflowed: this lane walks its cells (same order)
                const float4* sv = a.svel + S.p_off;
                const float4* sd = a.dyn + S.p_off;
                for_each_candidate(a, S, xi, [&](uint32_t j, float4 xj) {
                    const float rx = fs(xi.x, xj.x), ry = fs(xi.y, xj.y), rz = fs(xi.z, xj.z);
                    if (dist2(rx, ry, rz) <= S.smax) {
                        const float4 vj = __ldg(sv + j), dj = __ldg(sd + j);
                        force_pair_fast(S, acc, rx, ry, rz, dist2_fma(rx, ry, rz), vi.x, vi.y, vi.z, Ai, vj, dj.y, dj.z,
                                        __float_as_int(xj.w), (int)j == pl);
                    }
                });
            }
            if (valid) integrate_and_store(a, S, p, xi, vi, rho, acc, true);
        }
        it += (unsigned)M;
        __syncthreads();
    }
    if (!ok) atomicOr(a.status, 4u);
}

size_t force_tma_smem(int tile) {
    const int D = kTmaRingBytes / (tile * 32);
    return 128 + kTmaRingBytes + (size_t)D * tile * 4 + 2 * (size_t)D * 8;
}

// terrain: height snapshot = base + delta * unit, read by the next step.
// Four vertices per thread: a tile of T vertices takes T / 4 threads, each
// with 16-byte loads and stores (a scene's vertices start on a 512-vertex
// boundary, so every thread's first vertex is 4-aligned).
__global__ void __launch_bounds__(kMaxTile / 4) k_terrain(DevArrays a) {
    const int nwork = *a.n_ttiles;
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const Work wk = a.ttiles[w];
        if (a.steps_left[wk.scene] == 0) continue;
        const SceneDev& S = a.scenes[wk.scene];
        const int t = wk.start + 4 * (int)threadIdx.x;
        const int end = S.t_off + S.tw * S.td;
        const float u = S.height_unit;
        if (t + 3 < end) {
            const float4 b = *reinterpret_cast<const float4*>(a.tbase + t);
            const longlong2 d0 = *reinterpret_cast<const longlong2*>(a.tdelta + t);
            const longlong2 d1 = *reinterpret_cast<const longlong2*>(a.tdelta + t + 2);
            *reinterpret_cast<float4*>(a.theight + t) =
                make_float4(fa(b.x, fm(__ll2float_rn(d0.x), u)), fa(b.y, fm(__ll2float_rn(d0.y), u)),
                            fa(b.z, fm(__ll2float_rn(d1.x), u)), fa(b.w, fm(__ll2float_rn(d1.y), u)));
        } else {
            for (int k = t; k < end && k < t + 4; ++k) a.theight[k] = fa(a.tbase[k], fm(__ll2float_rn(a.tdelta[k]), u));
        }
    }
}

__global__ void k_tick(int* steps_left, int nscenes) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nscenes && steps_left[s] > 0) steps_left[s] -= 1;
}

__global__ void __launch_bounds__(kMaxTile) k_neighbour_counts(DevArrays a, int32_t* out) {
    const int nwork = *a.n_ptiles;
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const Work wk = a.ptiles[w];
        const SceneDev& S = a.scenes[wk.scene];
        const int p = wk.start + threadIdx.x;
        if (p >= S.p_off + S.n) continue;
        const float4 xi = a.spos[p];
        const int pl = p - S.p_off;
        int cnt = 0;
        for_each_candidate(a, S, xi, [&](uint32_t j, float4 xj) {
            float s = dist2(fs(xi.x, xj.x), fs(xi.y, xj.y), fs(xi.z, xj.z));
            if (s <= S.smax && (int)j != pl) ++cnt;
        });
        const int id = __float_as_int(xi.w);
        if (id >= 0 && id < S.n) out[S.p_off + id] = cnt;
    }
}

// splitmix64's finaliser (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014).
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ unsigned long long pair64(float lo, float hi) {
    return (unsigned long long)(uint32_t)__float_as_int(lo) |
           ((unsigned long long)(uint32_t)__float_as_int(hi) << 32);
}

// FP64 diagnostics: kDiagBlocks blocks per listed scene write fixed-order
// partial sums of momentum and energies (so the result is reproducible);
// integer totals use int64 atomics, which are exact in any order: sediment
// and terrain units, non-finite positions and the state fingerprint (sum of
// a mix of each particle's id and state bits, so any order of the particles
// in memory gives the same value).  isums holds three values per listed
// scene.
__global__ void __launch_bounds__(256) k_diag(DevArrays a, double* partial, long long* isums, int* nan_count) {
    __shared__ double sh[kDiagDoubles][8];
    const int li = blockIdx.x / kDiagBlocks, b = blockIdx.x % kDiagBlocks;
    const int sidx = a.scene_list[li];
    const SceneDev& S = a.scenes[sidx];
    double acc[kDiagDoubles] = {0, 0, 0, 0, 0, 0, 0, 0};
    long long sed = 0, ter = 0;
    unsigned long long fp = 0;
    int nan = 0;
    const double m = (double)S.mass;
    for (int q = b * 256 + threadIdx.x; q < S.n; q += kDiagBlocks * 256) {
        const float4 x = a.pos[S.p_off + q];
        const float4 v = a.vel[S.p_off + q];
        unsigned long long h = mix64(0x9e3779b97f4a7c15ULL * (unsigned long long)(uint32_t)(__float_as_int(x.w) + 1));
        h = mix64(h ^ pair64(x.x, x.y));
        h = mix64(h ^ pair64(x.z, v.x));
        h = mix64(h ^ pair64(v.y, v.z));
        h = mix64(h ^ (unsigned long long)(uint32_t)__float_as_int(v.w));
        fp += h;
        const double vx = v.x, vy = v.y, vz = v.z;
        acc[0] += m * vx;
        acc[1] += m * vy;
        acc[2] += m * vz;
        acc[3] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        acc[4] += -m * ((double)S.g[0] * x.x + (double)S.g[1] * x.y + (double)S.g[2] * x.z);
        sed += (long long)__float_as_int(v.w);
        if (!isfinite(x.x) || !isfinite(x.y) || !isfinite(x.z)) ++nan;
    }
    if (S.flags & kFlagTerrain)
        for (int t = b * 256 + threadIdx.x; t < S.tw * S.td; t += kDiagBlocks * 256) ter += a.tdelta[S.t_off + t];
    for (int c = 0; c < kDiagDoubles; ++c) {
        double v = acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
        if ((threadIdx.x & 31) == 0) sh[c][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < kDiagDoubles) {
        double v = 0.0;
        for (int q = 0; q < 8; ++q) v += sh[threadIdx.x][q];
        partial[(size_t)blockIdx.x * kDiagDoubles + threadIdx.x] = v;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sed += __shfl_down_sync(kFull, sed, o);
        ter += __shfl_down_sync(kFull, ter, o);
        fp += __shfl_down_sync(kFull, fp, o);
        nan += __shfl_down_sync(kFull, nan, o);
    }
    if ((threadIdx.x & 31) == 0) {
        unsigned long long* u = reinterpret_cast<unsigned long long*>(isums + 3 * li);
        if (sed) atomicAdd(u, (unsigned long long)sed);
        if (ter) atomicAdd(u + 1, (unsigned long long)ter);
        if (fp) atomicAdd(u + 2, fp);
        if (nan) atomicAdd(nan_count + li, nan);
    }
}

}  // namespace

void launch_keys(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    k_keys<<<(s.grid_p + kKeyTiles - 1) / kKeyTiles, s.tile, 0, st>>>(a);
}
void launch_scan(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    k_scan<<<s.grid_c, kScanThreads, 0, st>>>(a);
}
void launch_scatter(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    k_scatter<<<s.grid_p, s.tile, 0, st>>>(a);
}
void launch_reorder(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    k_reorder<<<s.grid_p, s.tile, 0, st>>>(a);
}
namespace {
// Traversal counters of one scene: [rows visited, candidates tested,
// in-range pairs (self included)], summed with int64 atomics.
__global__ void __launch_bounds__(256) k_traversal_stats(DevArrays a, int scene, unsigned long long* out) {
    const SceneDev& S = a.scenes[scene];
    unsigned long long rows = 0, cand = 0, hits = 0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S.n; p += gridDim.x * blockDim.x) {
        const float4 xi = a.spos[S.p_off + p];
        const Probe q = probe_of(S, xi);
        const int R = S.reach;
        for (int dz = -R; dz <= R; ++dz)
            for (int dy = -R; dy <= R; ++dy) {
                const int z = q.c.cz + dz, y = q.c.cy + dy;
                int xl, xh;
                if (z < 0 || z >= S.nz || y < 0 || y >= S.ny || !row_span(S, q, y, z, &xl, &xh)) continue;
                const uint32_t row = row_key(a.tab, S, y, z);
                const uint32_t st = a.offsets[S.k_off + row + xl], en = a.offsets[S.k_off + row + xh + 1];
                ++rows;
                for (uint32_t j = st; j < en; ++j) {
                    const float4 xj = a.spos[S.p_off + j];
                    ++cand;
                    hits += dist2(fs(xi.x, xj.x), fs(xi.y, xj.y), fs(xi.z, xj.z)) <= S.smax;
                }
            }
    }
    for (int o = 16; o > 0; o >>= 1) {
        rows += __shfl_down_sync(kFull, rows, o);
        cand += __shfl_down_sync(kFull, cand, o);
        hits += __shfl_down_sync(kFull, hits, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out, rows);
        atomicAdd(out + 1, cand);
        atomicAdd(out + 2, hits);
    }
}

__global__ void k_gather_by_id(const float4* __restrict__ pos, const float4* __restrict__ vel,
                               const float4* __restrict__ dyn, int p_off, int n, float* __restrict__ pos3,
                               float* __restrict__ vel3, float* __restrict__ dens, int32_t* __restrict__ sed) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float4 x = pos[p_off + p];
    const int id = __float_as_int(x.w);
    if (id < 0 || id >= n) return;
    if (pos3) {
        pos3[3 * id] = x.x;
        pos3[3 * id + 1] = x.y;
        pos3[3 * id + 2] = x.z;
    }
    if (vel3 || sed) {
        const float4 v = vel[p_off + p];
        if (vel3) {
            vel3[3 * id] = v.x;
            vel3[3 * id + 1] = v.y;
            vel3[3 * id + 2] = v.z;
        }
        if (sed) sed[id] = __float_as_int(v.w);
    }
    if (dens) dens[id] = dyn[p_off + p].x;
}
}  // namespace

void launch_traversal_stats(const DevArrays& a, int scene, unsigned long long* out, cudaStream_t st) {
    k_traversal_stats<<<304, 256, 0, st>>>(a, scene, out);
}

void launch_gather_by_id(const float4* pos, const float4* vel, const float4* dyn, int p_off, int n, float* pos3,
                         float* vel3, float* dens, int32_t* sed, cudaStream_t st) {
    if (n > 0) k_gather_by_id<<<(n + 255) / 256, 256, 0, st>>>(pos, vel, dyn, p_off, n, pos3, vel3, dens, sed);
}

void configure_kernels() {
    const int bytes = kListCap * kMaxTile * (int)sizeof(uint32_t);
    cudaFuncSetAttribute(k_density<false, true, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_density<false, true, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_force<false, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_force<false, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

static size_t list_bytes(const LaunchShape& s) { return (size_t)kListCap * s.tile * sizeof(uint32_t); }

// Variant bit 2 relaxes the register budget of the two neighbour kernels
// (fewer resident blocks, no spills) against the default high occupancy.
// Bit 3 hands the in-range neighbour lists from the density pass to the force
// pass (takes precedence over bit 0); bit 4 with it pipelines the force
// pass's list walk; bit 5 with it relaxes the density pass's register
// budget alone (4 resident blocks of 256 threads); bit 6 pairs the density pass's
// candidate loads; bit 7 with bit 3 packs each particle's force-pass inputs
// into one 32-byte record.
template <int MINB, bool DYN, bool FM>
static void launch_density_nl_d(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    const bool x2 = (s.variant & 64) != 0, pack = (s.variant & 128) != 0;
    const int grid = DYN ? s.grid_dyn : s.grid_p;
    if (x2 && pack)
        k_density<false, false, MINB, true, true, true, DYN, FM><<<grid, s.tile, 0, st>>>(a);
    else if (x2)
        k_density<false, false, MINB, true, true, false, DYN, FM><<<grid, s.tile, 0, st>>>(a);
    else if (pack)
        k_density<false, false, MINB, true, false, true, DYN, FM><<<grid, s.tile, 0, st>>>(a);
    else
        k_density<false, false, MINB, true, false, false, DYN, FM><<<grid, s.tile, 0, st>>>(a);
}

// Bit 16 (65536): the list-writing density pass takes its work in warp
// slices from a counter (dynamic scheduling; same bits).  Bit 17 (131072):
// fast arithmetic (density_term_fast; not the same bits).
template <int MINB>
static void launch_density_nl(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    const bool fm = (s.variant & 131072) != 0;
    if (s.variant & 65536) {
        if (fm)
            launch_density_nl_d<MINB, true, true>(a, s, st);
        else
            launch_density_nl_d<MINB, true, false>(a, s, st);
    } else if (fm)
        launch_density_nl_d<MINB, false, true>(a, s, st);
    else
        launch_density_nl_d<MINB, false, false>(a, s, st);
}

// Variant bit 8 (with bit 3): the cooperative passes, G lanes per particle.
// Density: 32 lanes (bit 11: 16).  Force: 8 lanes (bit 9: 4, bit 10: 16).
// Bit 7 packs the force-pass inputs as in the per-lane passes; bit 2
// relaxes the force pass's register budget.
static void launch_density_coop(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    const bool pack = (s.variant & 128) != 0;
    if (s.variant & 2048) {
        if (pack)
            k_density_coop<16, true><<<s.grid_p, s.tile, 0, st>>>(a);
        else
            k_density_coop<16, false><<<s.grid_p, s.tile, 0, st>>>(a);
    } else {
        if (pack)
            k_density_coop<32, true><<<s.grid_p, s.tile, 0, st>>>(a);
        else
            k_density_coop<32, false><<<s.grid_p, s.tile, 0, st>>>(a);
    }
}

template <int MINB>
static void launch_force_coop_b(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    const bool pack = (s.variant & 128) != 0;
    const int gsel = (s.variant >> 9) & 3;
    if (gsel == 1) {
        if (pack)
            k_force_coop<4, true, MINB><<<s.grid_p, s.tile, 0, st>>>(a);
        else
            k_force_coop<4, false, MINB><<<s.grid_p, s.tile, 0, st>>>(a);
    } else if (gsel == 2) {
        if (pack)
            k_force_coop<16, true, MINB><<<s.grid_p, s.tile, 0, st>>>(a);
        else
            k_force_coop<16, false, MINB><<<s.grid_p, s.tile, 0, st>>>(a);
    } else {
        if (pack)
            k_force_coop<8, true, MINB><<<s.grid_p, s.tile, 0, st>>>(a);
        else
            k_force_coop<8, false, MINB><<<s.grid_p, s.tile, 0, st>>>(a);
    }
}

// Bit 2 relaxes the cooperative force pass's register budget (3 resident
// blocks of 256 threads instead of 4).
static void launch_force_coop(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    if (s.variant & 4)
        launch_force_coop_b<3>(a, s, st);
    else
        launch_force_coop_b<4>(a, s, st);
}

static bool coop(const LaunchShape& s) { return (s.variant & (256 | 8)) == (256 | 8); }

void launch_density(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    if (coop(s)) {
        launch_density_coop(a, s, st);
        return;
    }
    const bool relaxed = (s.variant & 4) != 0;
    if (s.variant & 8) {
        if (relaxed)
            launch_density_nl<4>(a, s, st);
        else if (s.variant & 32)
            launch_density_nl<4>(a, s, st);
        else
            launch_density_nl<8>(a, s, st);
    } else if (s.variant & 1) {
        if (relaxed)
            k_density<false, true, 4><<<s.grid_p, s.tile, list_bytes(s), st>>>(a);
        else
            k_density<false, true, 8><<<s.grid_p, s.tile, list_bytes(s), st>>>(a);
    } else {
        if (relaxed)
            k_density<false, false, 4><<<s.grid_p, s.tile, 0, st>>>(a);
        else
            k_density<false, false, 8><<<s.grid_p, s.tile, 0, st>>>(a);
    }
}
void launch_density_ordered(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    k_density<true, false, 1><<<s.grid_p, s.tile, 0, st>>>(a);
}
void launch_force(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    if (coop(s)) {
        launch_force_coop(a, s, st);
        return;
    }
    // the list variants walk their lists (or, on overflow, the cells) per
    // lane and need no shared memory; bit 15 (32768) has the pipelined list
    // walks take their work in warp slices from a counter (same bits)
    const bool dyn = (s.variant & 32768) != 0;
    if ((s.variant & 262144) && (s.variant & (131072 | 128 | 24)) == (131072 | 128 | 24) && s.fmap) {
        // bit 18: the TMA gather pipeline (fast arithmetic, packed records)
        k_force_tma<3><<<s.grid_p, s.tile + 32, force_tma_smem(s.tile), st>>>(a, *static_cast<const CUtensorMap*>(s.fmap));
        return;
    }
    if ((s.variant & 131072) && (s.variant & 24) == 24) {
        // bit 17: fast arithmetic (force_pair_fast), pipelined list walk
        const bool pack = (s.variant & 128) != 0;
        if (pack) {
            if (dyn)
                k_force<false, 4, 3, true, true><<<s.grid_dyn, s.tile, 0, st>>>(a);
            else
                k_force<false, 4, 3, false, true><<<s.grid_p, s.tile, 0, st>>>(a);
        } else if (dyn)
            k_force<false, 4, 2, true, true><<<s.grid_dyn, s.tile, 0, st>>>(a);
        else
            k_force<false, 4, 2, false, true><<<s.grid_p, s.tile, 0, st>>>(a);
        return;
    }
    if ((s.variant & 136) == 136) {
        if (dyn) {
            if (s.variant & 4)
                k_force<false, 3, 3, true><<<s.grid_dyn, s.tile, 0, st>>>(a);
            else
                k_force<false, 4, 3, true><<<s.grid_dyn, s.tile, 0, st>>>(a);
        } else if (s.variant & 4)
            k_force<false, 3, 3><<<s.grid_p, s.tile, 0, st>>>(a);
        else
            k_force<false, 4, 3><<<s.grid_p, s.tile, 0, st>>>(a);
    } else if ((s.variant & 24) == 24) {
        if (dyn) {
            if (s.variant & 4)
                k_force<false, 3, 2, true><<<s.grid_dyn, s.tile, 0, st>>>(a);
            else
                k_force<false, 4, 2, true><<<s.grid_dyn, s.tile, 0, st>>>(a);
        } else if (s.variant & 4)
            k_force<false, 3, 2><<<s.grid_p, s.tile, 0, st>>>(a);
        else
            k_force<false, 4, 2><<<s.grid_p, s.tile, 0, st>>>(a);
    } else if (s.variant & 8) {
        if (s.variant & 4)
            k_force<false, 3, 1><<<s.grid_p, s.tile, 0, st>>>(a);
        else
            k_force<false, 4, 1><<<s.grid_p, s.tile, 0, st>>>(a);
    } else if (s.variant & 4)
        k_force<false, 3><<<s.grid_p, s.tile, list_bytes(s), st>>>(a);
    else
        k_force<false, 4><<<s.grid_p, s.tile, list_bytes(s), st>>>(a);
}
void launch_force_ordered(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    k_force<true, 1><<<s.grid_p, s.tile, 0, st>>>(a);
}
void launch_terrain(const DevArrays& a, const LaunchShape& s, cudaStream_t st) {
    k_terrain<<<s.grid_t, s.tile / 4, 0, st>>>(a);
}
void launch_tick(const DevArrays& a, int nscenes, cudaStream_t st) {
    k_tick<<<(nscenes + 127) / 128, 128, 0, st>>>(a.steps_left, nscenes);
}
void launch_neighbour_counts(const DevArrays& a, const LaunchShape& s, int32_t* out_by_id, cudaStream_t st) {
    k_neighbour_counts<<<s.grid_p, s.tile, 0, st>>>(a, out_by_id);
}
void launch_diag(const DevArrays& a, int nlist, double* partial, long long* isums, int* nan_count,
                 cudaStream_t st) {
    if (nlist > 0) k_diag<<<nlist * kDiagBlocks, 256, 0, st>>>(a, partial, isums, nan_count);
}

}  // namespace sph
