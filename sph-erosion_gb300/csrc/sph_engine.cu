// Host engine: arenas, scenes, work lists, step orchestration, CUDA graphs.
#include "sph_engine.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace sph {

void check_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return;
    const int code = (e == cudaErrorMemoryAllocation) ? SPH_ERR_NOMEM : SPH_ERR_CUDA;
    throw Error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

constexpr int kPAlign = kRangeAlign;  // particle ranges start on a tile boundary for every tile size
constexpr int64_t kTAlign = kRangeAlign;
// Largest arena size in entries: offsets and in-scene indices stay inside the
// kernels' 32-bit index arithmetic with room for a tile of overrun.
constexpr int64_t kMaxArenaIndex = ((int64_t)1 << 31) - ((int64_t)1 << 20);

int64_t round_up(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

inline float bits_to_float(int v) {
    float f;
    std::memcpy(&f, &v, sizeof f);
    return f;
}
inline int float_to_bits(float f) {
    int v;
    std::memcpy(&v, &f, sizeof v);
    return v;
}

}  // namespace

namespace {
int bits_for(int n) {
    int b = 0;
    while ((1 << b) < n) ++b;
    return b;
}

// (y, z) Morton code: bit b of y, then bit b of z, while each still has bits.
uint32_t yz_morton(int cy, int cz, int by, int bz) {
    uint32_t m = 0;
    int o = 0;
    for (int b = 0; b < std::max(by, bz); ++b) {
        if (b < by) m |= (uint32_t)((cy >> b) & 1) << o++;
        if (b < bz) m |= (uint32_t)((cz >> b) & 1) << o++;
    }
    return m;
}
}  // namespace

// Row numbers of a grid's cell rows: the ny * nz rows (y, z) ordered along
// the (y, z) Morton curve and numbered densely in that order, so that
// neighbouring rows stay close in the sorted particle order while the key
// space holds no codes outside the grid; tab[z * ny + y] = the row's number.
void row_table(int ny, int nz, uint32_t* tab) {
    const int by = bits_for(ny), bz = bits_for(nz);
    std::vector<std::pair<uint32_t, uint32_t>> rows((size_t)ny * nz);
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            rows[(size_t)z * ny + y] = {yz_morton(y, z, by, bz), (uint32_t)((size_t)z * ny + y)};
    std::sort(rows.begin(), rows.end());
    for (size_t r = 0; r < rows.size(); ++r) tab[rows[r].second] = (uint32_t)r;
}

// Largest float s with sqrtf(s) <= h.  sqrtf is correctly rounded and
// monotonic, so for every float s >= 0: sqrtf(s) <= h  <=>  s <= smax.  The
// kernels test the squared distance against it, which selects exactly the
// reference's neighbours (glm::length(r) <= h, fluid_system.h:119) without a
// square root per candidate.
float smax_for(float h) {
    float s = h * h;
    while (std::sqrt(s) > h) s = std::nextafter(s, 0.0f);
    for (;;) {
        float nx = std::nextafter(s, INFINITY);
        if (std::sqrt(nx) <= h)
            s = nx;
        else
            break;
    }
    return s;
}

// Smallest float f whose double value is >= 1e-4: for any float d,
// (double)d < 10e-5 (fluid_system.h:438)  <=>  d < threshold.
float coincidence_threshold() {
    float f = (float)1e-4;
    while ((double)f < 1e-4) f = std::nextafter(f, INFINITY);
    for (;;) {
        float pv = std::nextafter(f, 0.0f);
        if ((double)pv >= 1e-4)
            f = pv;
        else
            break;
    }
    return f;
}

// ---- RangeAlloc -------------------------------------------------------------
void RangeAlloc::reset(int64_t cap) {
    free_.clear();
    cap_ = cap;
    used_ = 0;
    if (cap > 0) free_[0] = cap;
}

bool RangeAlloc::alloc(int64_t len, int64_t* off) {
    if (len <= 0) {
        *off = 0;
        return true;
    }
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second >= len) {
            *off = it->first;
            const int64_t rest = it->second - len, roff = it->first + len;
            free_.erase(it);
            if (rest > 0) free_[roff] = rest;
            used_ += len;
            return true;
        }
    }
    return false;
}

void RangeAlloc::release(int64_t off, int64_t len) {
    if (len <= 0) return;
    used_ -= len;
    auto it = free_.emplace(off, len).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        free_.erase(nx);
    }
    if (it != free_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            free_.erase(it);
        }
    }
}

void RangeAlloc::grow(int64_t cap) {
    if (cap <= cap_) return;
    const int64_t old = cap_;
    cap_ = cap;
    used_ += cap - old;  // release() below subtracts the new space again
    release(old, cap - old);
}

// ---- DevBuf -------------------------------------------------------------------
template <class T>
void DevBuf<T>::resize(int64_t cnt, bool keep, cudaStream_t st) {
    if (cnt == n) return;
    T* np = nullptr;
    if (cnt > 0) {
        SPH_CK(cudaMalloc(&np, (size_t)cnt * sizeof(T)));
        SPH_CK(cudaMemsetAsync(np, 0, (size_t)cnt * sizeof(T), st));
        if (keep && p && n > 0)
            SPH_CK(cudaMemcpyAsync(np, p, (size_t)std::min(n, cnt) * sizeof(T), cudaMemcpyDeviceToDevice, st));
        SPH_CK(cudaStreamSynchronize(st));
    }
    if (p) cudaFree(p);
    p = np;
    n = cnt;
}

template <class T>
void DevBuf<T>::release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
}

// ---- System -----------------------------------------------------------------
System::System(const sph_system_config& cfg) : cfg_(cfg) {
    if (cfg_.tile == 0) cfg_.tile = 256;
    if (cfg_.tile != 128 && cfg_.tile != 256) throw Error(SPH_ERR_INVALID, "tile must be 128 or 256");
    if (cfg_.max_scenes <= 0) cfg_.max_scenes = 1024;
    if (cfg_.particle_capacity > kMaxArenaIndex || cfg_.key_capacity > kMaxArenaIndex ||
        cfg_.terrain_capacity > kMaxArenaIndex)
        throw Error(SPH_ERR_INVALID, "capacities are limited to 2^31 - 2^20 entries");
    dev_ = cfg_.device;
    SPH_CK(cudaSetDevice(dev_));
    SPH_CK(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, dev_));
    SPH_CK(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    SPH_CK(cudaStreamCreateWithFlags(&cst_, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
        SPH_CK(cudaEventCreateWithFlags(&gathered_[k], cudaEventDisableTiming));
        SPH_CK(cudaEventCreateWithFlags(&copied_[k], cudaEventDisableTiming));
    }
    SPH_CK(cudaMallocHost(&up_dev_, sizeof(SceneDev) * kUploadRing));
    SPH_CK(cudaMallocHost(&up_steps_, sizeof(int) * kUploadRing));
    for (auto& e : up_ev_) SPH_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    configure_kernels();
    SPH_CK(cudaGetLastError());
    pa_.reset(0);
    ka_.reset(0);
    ca_.reset(0);
    ta_.reset(0);
    tba_.reset(0);
    dscenes_.resize(cfg_.max_scenes, false, st_);
    steps_.resize(cfg_.max_scenes, false, st_);
    nwork_.resize(4, false, st_);
    slist_.resize(cfg_.max_scenes, false, st_);
    status_.resize(3, false, st_);  // status word + the two work counters
    SPH_CK(cudaMemsetAsync(status_.p, 0, 3 * sizeof(unsigned), st_));
    diag_part_.resize((int64_t)kDiagBlocks * kDiagDoubles, false, st_);
    diag_i_.resize(3, false, st_);
    diag_nan_.resize(1, false, st_);
    initial_arenas();
}

// Arena sizes of a fresh system (config capacities).
void System::initial_arenas() {
    grow_particles(std::max<int64_t>(round_up(std::max<int64_t>(cfg_.particle_capacity, 1), kPAlign), kPAlign));
    grow_keys(std::max<int64_t>(round_up(std::max<int64_t>(cfg_.key_capacity, 1), kChunk), kChunk));
    grow_chunks(1024);
    grow_tables(4096);
    grow_terrain(std::max<int64_t>(round_up(std::max<int64_t>(cfg_.terrain_capacity, 1), kTAlign), kTAlign));
}

// With no live scene, return all arena memory and start again from the
// initial sizes: arenas only grow, so after a peak of resident scenes their
// free space would otherwise stay charged to the budget.
bool System::trim() {
    for (const Scene& sc : scenes_)
        if (sc.live) return false;
    SPH_CK(cudaStreamSynchronize(st_));
    SPH_CK(cudaStreamSynchronize(cst_));
    drop_graph();
    DevBuf<float4>* f4[] = {&pos_, &vel_, &spos_, &svel_, &dyn_, &fdat_};
    for (auto* b : f4) b->release();
    DevBuf<uint32_t>* u4[] = {&key_, &slot_, &perm_, &nlist_, &counts_, &offsets_, &chunk_, &tab_};
    for (auto* b : u4) b->release();
    nbid_.release();
    snbid_.release();
    ncnt_.release();
    rec_.release();
    tbase_.release();
    theight_.release();
    tdelta_.release();
    stage_.release();
    scratch_i_.release();
    for (auto& b : astage_) b.release();
    pa_.reset(0);
    ka_.reset(0);
    ca_.reset(0);
    ta_.reset(0);
    tba_.reset(0);
    initial_arenas();
    work_dirty_ = true;
    return true;
}

System::~System() {
    drop_graph();
    if (st_) cudaStreamSynchronize(st_);
    if (cst_) cudaStreamSynchronize(cst_);
    for (int k = 0; k < 2; ++k) {
        astage_[k].release();
        if (gathered_[k]) cudaEventDestroy(gathered_[k]);
        if (copied_[k]) cudaEventDestroy(copied_[k]);
    }
    if (cst_) cudaStreamDestroy(cst_);
    for (auto& e : up_ev_)
        if (e) cudaEventDestroy(e);
    if (up_dev_) cudaFreeHost(up_dev_);
    if (up_steps_) cudaFreeHost(up_steps_);
    DevBuf<float4>* f4[] = {&pos_, &vel_, &spos_, &svel_, &dyn_};
    for (auto* b : f4) b->release();
    key_.release(); slot_.release(); perm_.release();
    nbid_.release(); snbid_.release(); rec_.release();
    nlist_.release(); ncnt_.release(); fdat_.release();
    counts_.release(); offsets_.release(); chunk_.release(); tab_.release();
    tbase_.release(); theight_.release(); tdelta_.release();
    dscenes_.release(); steps_.release(); ptiles_.release(); ctiles_.release(); ttiles_.release();
    nwork_.release(); slist_.release(); status_.release(); scratch_i_.release(); stage_.release();
    diag_part_.release(); diag_i_.release(); diag_nan_.release();
    if (st_) cudaStreamDestroy(st_);
}

Scene& System::scene(int id) {
    if (id < 0 || id >= (int)scenes_.size() || !scenes_[id].live) throw Error(SPH_ERR_INVALID, "no such scene");
    return scenes_[id];
}
const Scene& System::scene(int id) const {
    if (id < 0 || id >= (int)scenes_.size() || !scenes_[id].live) throw Error(SPH_ERR_INVALID, "no such scene");
    return scenes_[id];
}

int64_t System::memory_bytes() const {
    int64_t b = 0;
    b += pos_.bytes() + vel_.bytes() + spos_.bytes() + svel_.bytes() + dyn_.bytes();
    b += key_.bytes() + slot_.bytes() + perm_.bytes() + nbid_.bytes() + snbid_.bytes() + rec_.bytes();
    b += nlist_.bytes() + ncnt_.bytes() + fdat_.bytes();
    b += counts_.bytes() + offsets_.bytes() + chunk_.bytes() + tab_.bytes();
    b += tbase_.bytes() + theight_.bytes() + tdelta_.bytes();
    b += dscenes_.bytes() + steps_.bytes() + ptiles_.bytes() + ctiles_.bytes() + ttiles_.bytes();
    b += scratch_i_.bytes();
    return b;
}

// Bytes one scene of n particles and a tw x td terrain needs in the arenas.
int64_t System::scene_bytes(int n, int tw, int td, const sph_params& p, bool lists) const {
    Scene tmp;
    tmp.prm = p;
    const_cast<System*>(this)->geometry(tmp);
    const int64_t pcap = round_up(std::max(n, 1), kPAlign);
    int64_t per_p = 5 * 16 + 3 * 4 + 2 * 4 + ((p.flags & SPH_FLAG_RECORD) ? kRecFloats * 4 : 0);
    if (lists && (cfg_.variant & 8))  // neighbour lists: optional, dropped when the budget has no room
        per_p += (int64_t)kNbCap * 4 + 4 + ((cfg_.variant & 128) ? 32 : 0);
    return pcap * per_p + (int64_t)tmp.k_cap * 8 + (int64_t)tmp.nchunks * 4 + tmp.tab_len * 4 +
           round_up((int64_t)tw * td, kTAlign) * 16 + (int64_t)(pcap / cfg_.tile + tmp.nchunks) * 8;
}

void System::check_budget(int64_t extra) const {
    if (cfg_.hbm_budget > 0 && memory_bytes() + extra > cfg_.hbm_budget)
        throw Error(SPH_ERR_CAPACITY, "HBM budget exceeded");
}

void System::drop_graph() {
    if (gexec_) cudaGraphExecDestroy(gexec_);
    if (graph_) cudaGraphDestroy(graph_);
    gexec_ = nullptr;
    graph_ = nullptr;
    graph_dirty_ = true;
}

void System::grow_particles(int64_t cap) {
    const int64_t need = cap - pos_.n;
    if (need <= 0) return;
    check_budget(need * (5 * 16 + 3 * 4 + 2 * 4 + (rec_.n ? kRecFloats * 4 : 0)));
    DevBuf<float4>* f4[] = {&pos_, &vel_, &spos_, &svel_, &dyn_};
    for (auto* b : f4) b->resize(cap, true, st_);
    key_.resize(cap, true, st_);
    slot_.resize(cap, true, st_);
    perm_.resize(cap, true, st_);
    nbid_.resize(cap, true, st_);
    snbid_.resize(cap, true, st_);
    if (rec_.n) rec_.resize(cap * kRecFloats, true, st_);
    pa_.grow(cap);
    work_dirty_ = true;  // the neighbour lists follow the arena's size
    drop_graph();
}
void System::grow_keys(int64_t cap) {
    if (cap <= counts_.n) return;
    check_budget((cap - counts_.n) * 8);
    counts_.resize(cap, true, st_);
    offsets_.resize(cap, true, st_);
    ka_.grow(cap);
    drop_graph();
}
void System::grow_chunks(int64_t cap) {
    if (cap <= chunk_.n) return;
    chunk_.resize(cap, true, st_);
    ca_.grow(cap);
    drop_graph();
}
void System::grow_tables(int64_t cap) {
    if (cap <= tab_.n) return;
    tab_.resize(cap, true, st_);
    tba_.grow(cap);
    drop_graph();
}
void System::grow_terrain(int64_t cap) {
    if (cap <= tbase_.n) return;
    check_budget((cap - tbase_.n) * 16);
    tbase_.resize(cap, true, st_);
    theight_.resize(cap, true, st_);
    tdelta_.resize(cap, true, st_);
    ta_.grow(cap);
    drop_graph();
}

// which: 0 particles, 1 keys, 2 chunks, 3 tables, 4 terrain.  Every arena
// stays below kMaxArenaIndex entries: the kernels index them with 32-bit
// offsets (a particle, key or vertex offset plus an index within the scene).
// A scene that would need more gets SPH_ERR_CAPACITY (a server waits for
// retirements).
void System::ensure_arena(RangeAlloc& ra, int64_t need, int which) {
    int64_t off;
    if (ra.alloc(need, &off)) {
        ra.release(off, need);
        return;
    }
    const int64_t align = which == 0 ? kPAlign : which == 1 ? kChunk : which == 4 ? kTAlign : 1;
    const int64_t limit = kMaxArenaIndex / align * align;
    if (ra.cap() + need > limit) throw Error(SPH_ERR_CAPACITY, "arena index range exhausted (2^31 entries)");
    // Double the arena; under an HBM budget fall back to growing by exactly
    // what is missing when doubling would not fit.
    auto grow = [&](int64_t cap) {
        cap = std::min(round_up(cap, align), limit);
        switch (which) {
            case 0: grow_particles(cap); break;
            case 1: grow_keys(cap); break;
            case 2: grow_chunks(cap); break;
            case 3: grow_tables(cap); break;
            default: grow_terrain(cap); break;
        }
    };
    const int64_t doubled = std::max(ra.cap() * 2, ra.cap() + need);
    if (cfg_.hbm_budget > 0) {
        try {
            grow(doubled);
        } catch (const Error& e) {
            if (e.code != SPH_ERR_CAPACITY) throw;
            grow(ra.cap() + need);
        }
    } else {
        grow(doubled);
    }
}

// Uniform grid of a scene.  Cell edge along y and z = h * cell_mult *
// (1 + 2^-12); along x the same over xsub, 2 when one cell is h or more
// (reach 1: rows are then trimmed to the sphere in half cells), else 1
// (exact either way: a power of two).  The slack keeps any two particles
// within h at most `reach` cells apart along y and z, and reach * xsub along
// x, after the FP32 rounding of the key arithmetic, so the traversal never
// misses a neighbour.
void System::geometry(Scene& sc) {
    const sph_params& p = sc.prm;
    sc.cell = (p.smoothing_radius * p.cell_mult) * 1.000244140625f;
    sc.inv_cell = 1.0f / sc.cell;
    sc.reach = (int)std::ceil(1.0 / (double)p.cell_mult - 1e-9);
    sc.xsub = sc.reach == 1 ? 2 : 1;
    int d[3];
    for (int a = 0; a < 3; ++a) {
        const float ext = p.box_half[a] + p.box_half[a];
        const float edge = a == 0 ? sc.cell / (float)sc.xsub : sc.cell;
        int nd = (int)std::ceil((double)ext / (double)edge);
        d[a] = std::max(nd, 1);
        sc.lo[a] = p.box_center[a] - p.box_half[a];
    }
    sc.nx = d[0];
    sc.ny = d[1];
    sc.nz = d[2];
    const int64_t nk = (int64_t)sc.nx * sc.ny * sc.nz + 1;
    if (nk > (int64_t)1 << 30) throw Error(SPH_ERR_CAPACITY, "uniform grid too large (raise cell_mult or shrink the box)");
    sc.nkeys = (int)nk;
    sc.k_cap = (int)round_up(nk, kChunk);
    sc.nchunks = sc.k_cap / kChunk;
    sc.tab_len = sc.ny * sc.nz;
}

void System::fill_dev(Scene& sc) {
    const sph_params& p = sc.prm;
    SceneDev& d = sc.dev;
    std::memset(&d, 0, sizeof d);
    d.p_off = (int)sc.p_off;
    d.n = sc.n;
    d.p_cap = sc.p_cap;
    d.k_off = (int)sc.k_off;
    d.nkeys = sc.nkeys;
    d.k_cap = sc.k_cap;
    d.c_off = (int)sc.c_off;
    d.nchunks = sc.nchunks;
    d.t_off = (int)sc.t_off;
    d.tw = sc.tw;
    d.td = sc.td;
    d.tab_off = (int)sc.tab_off;
    d.nx = sc.nx;
    d.ny = sc.ny;
    d.nz = sc.nz;
    d.reach = sc.reach;
    d.flags = 0;
    if (sc.tw > 0) d.flags |= kFlagTerrain;
    if (sc.tw > 0 && p.erosion) d.flags |= kFlagErosion;
    if (p.flags & SPH_FLAG_RECORD) d.flags |= kFlagRecord;
    if (p.flags & SPH_FLAG_ORDERED) d.flags |= kFlagOrdered;
    for (int a = 0; a < 3; ++a) d.lo[a] = sc.lo[a];
    d.inv_cell = sc.inv_cell;
    d.inv_cell_x = sc.inv_cell * (float)sc.xsub;  // exact: 1 / (cell / xsub)
    d.xsub = sc.xsub;
    // h in cell units for the row trimming, enlarged by 1e-5 relative plus four
    // ulps of the largest in-grid cell coordinate, so that the FP32 rounding of
    // the two particles' cell coordinates can never drop a neighbour
    {
        const float tmax = (float)std::max(sc.nx, std::max(sc.ny, sc.nz));
        const double ulp = (double)std::nextafter(tmax, INFINITY) - (double)tmax;
        d.hcell = (float)((double)p.smoothing_radius * (double)sc.inv_cell * (1.0 + 1e-5) + 4.0 * ulp + 1e-4);
    }
    // kernel constants, same FP32 expressions as fluid_system.h:415-452
    // with PI = 3.141592f (Erosion/sphere.h:8)
    const float h = p.smoothing_radius;
    const float PI = 3.141592f;
    d.h = h;
    d.hh = h * h;
    d.smax = smax_for(h);
    d.cthr = coincidence_threshold();
    d.mass = p.mass;
    d.p0 = p.rest_density;
    d.k = p.gas_stiffness;
    d.visc = p.viscosity;
    d.sigma = p.surface_tension;
    d.dt = p.dt;
    d.cr = p.restitution;
    for (int a = 0; a < 3; ++a) d.g[a] = p.gravity[a];
    d.c_poly6 = 315.0f / (64.0f * PI * powf(h, 9.0f));
    d.c_grad = 945.0f / (32.0f * PI * powf(h, 9.0f));
    d.c_spiky = 45.0f / (PI * powf(h, 6.0f));
    {
        const float three = (1.0f * 1.0f + 1.0f * 1.0f) + 1.0f * 1.0f;
        d.inv_sqrt3 = 1.0f / sqrtf(three);
    }
    const bool iso = p.box_half[0] == p.box_half[1] && p.box_half[1] == p.box_half[2];
    for (int a = 0; a < 3; ++a) {
        d.box_c[a] = p.box_center[a];
        d.box_l[a] = p.box_half[a];
        d.box_w[a] = iso ? 1.0f : 1.0f / p.box_half[a];
    }
    if (sc.tw > 0) {
        const float sx = (p.box_half[0] + p.box_half[0]) / (float)(sc.tw - 1);
        const float sz = (p.box_half[2] + p.box_half[2]) / (float)(sc.td - 1);
        d.t_xlo = p.box_center[0] - p.box_half[0];
        d.t_ylo = p.box_center[1] - p.box_half[1];
        d.t_zlo = p.box_center[2] - p.box_half[2];
        d.t_isx = 1.0f / sx;
        d.t_isz = 1.0f / sz;
        d.t_wmax = (float)(sc.tw - 1);
        d.t_dmax = (float)(sc.td - 1);
        // one sediment unit = 2^-30 of a particle's rest volume, spread over
        // the area of one vertex cell
        d.height_unit = (float)(((double)p.mass / (double)p.rest_density) * std::ldexp(1.0, -30) /
                                ((double)sx * (double)sz));
    }
    d.k_capacity = p.k_capacity;
    d.k_pick = p.k_pickup;
    d.k_dep = p.k_deposit;
    d.layer = p.erosion_layer;
}

// Stream-ordered: kernels enqueued before see the old descriptor, later ones
// the new.  The copy reads a pinned ring slot, so it does not make the host
// wait for the stream (a copy from pageable memory may); a slot is rewritten
// only after the copy that read it has run.
void System::upload_scene(int id) {
    Scene& sc = scenes_[id];
    fill_dev(sc);
    const int k = up_next_;
    up_next_ = (up_next_ + 1) % kUploadRing;
    SPH_CK(cudaEventSynchronize(up_ev_[k]));
    up_dev_[k] = sc.dev;
    up_steps_[k] = sc.steps;
    SPH_CK(cudaMemcpyAsync(dscenes_.p + id, up_dev_ + k, sizeof(SceneDev), cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaMemcpyAsync(steps_.p + id, up_steps_ + k, sizeof(int), cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaEventRecord(up_ev_[k], st_));
}

void validate_params(const sph_params& p) {
    if (!(p.smoothing_radius > 0.0f) || !std::isfinite(p.smoothing_radius))
        throw Error(SPH_ERR_INVALID, "smoothing_radius must be positive");
    for (int a = 0; a < 3; ++a)
        if (!(p.box_half[a] > 0.0f) || !std::isfinite(p.box_half[a]))
            throw Error(SPH_ERR_INVALID, "box_half must be positive");
    if (!(p.cell_mult >= 0.25f) || !(p.cell_mult <= 8.0f)) throw Error(SPH_ERR_INVALID, "cell_mult must be in [0.25, 8]");
}

int System::create_scene(const sph_params& p, int capacity, int tw, int td) {
    validate_params(p);
    if (capacity < 0 || tw < 0 || td < 0) throw Error(SPH_ERR_INVALID, "negative size");
    if ((tw > 0) != (td > 0) || (tw > 0 && (tw < 2 || td < 2)))
        throw Error(SPH_ERR_INVALID, "terrain needs at least 2 x 2 vertices");
    int id = -1;
    for (int i = 0; i < (int)scenes_.size(); ++i)
        if (!scenes_[i].live) {
            id = i;
            break;
        }
    if (id < 0) {
        if ((int)scenes_.size() >= cfg_.max_scenes) throw Error(SPH_ERR_CAPACITY, "max_scenes reached");
        scenes_.emplace_back();
        id = (int)scenes_.size() - 1;
    }
    Scene sc;
    sc.prm = p;
    geometry(sc);
    sc.p_cap = (int)round_up(std::max(capacity, 1), kPAlign);
    sc.tw = tw;
    sc.td = td;
    // Arena growth is charged against the budget where it happens
    // (ensure_arena); here only a scene that could never fit is refused.
    if (cfg_.hbm_budget > 0 && scene_bytes(sc.p_cap, tw, td, p, false) > cfg_.hbm_budget)
        throw Error(SPH_ERR_CAPACITY, "scene larger than the HBM budget");
    ensure_arena(pa_, sc.p_cap, 0);
    ensure_arena(ka_, sc.k_cap, 1);
    ensure_arena(ca_, sc.nchunks, 2);
    ensure_arena(tba_, sc.tab_len, 3);
    const int64_t tlen = tw > 0 ? round_up((int64_t)tw * td, kTAlign) : 0;
    if (tlen) ensure_arena(ta_, tlen, 4);
    {
        // all ranges or none
        bool okp = pa_.alloc(sc.p_cap, &sc.p_off), okk = okp && ka_.alloc(sc.k_cap, &sc.k_off);
        bool okc = okk && ca_.alloc(sc.nchunks, &sc.c_off), okt = okc && tba_.alloc(sc.tab_len, &sc.tab_off);
        bool oka = okt && (!tlen || ta_.alloc(tlen, &sc.t_off));
        if (!oka) {
            if (okt) tba_.release(sc.tab_off, sc.tab_len);
            if (okc) ca_.release(sc.c_off, sc.nchunks);
            if (okk) ka_.release(sc.k_off, sc.k_cap);
            if (okp) pa_.release(sc.p_off, sc.p_cap);
            throw Error(SPH_ERR_NOMEM, "arena allocation failed");
        }
    }
    if (p.flags & SPH_FLAG_RECORD && rec_.n == 0) {
        rec_.resize(pos_.n * kRecFloats, false, st_);
        drop_graph();
    }
    // row tables and clean key ranges
    std::vector<uint32_t> tab(sc.tab_len);
    row_table(sc.ny, sc.nz, tab.data());
    SPH_CK(cudaMemcpyAsync(tab_.p + sc.tab_off, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaMemsetAsync(counts_.p + sc.k_off, 0, (size_t)sc.k_cap * 4, st_));
    SPH_CK(cudaMemsetAsync(chunk_.p + sc.c_off, 0, (size_t)sc.nchunks * 4, st_));
    if (tlen) {
        SPH_CK(cudaMemsetAsync(tbase_.p + sc.t_off, 0, (size_t)tlen * 4, st_));
        SPH_CK(cudaMemsetAsync(theight_.p + sc.t_off, 0, (size_t)tlen * 4, st_));
        SPH_CK(cudaMemsetAsync(tdelta_.p + sc.t_off, 0, (size_t)tlen * 8, st_));
    }
    sc.live = true;
    scenes_[id] = sc;
    upload_scene(id);
    work_dirty_ = true;
    return id;
}

void System::destroy_scene(int id) {
    Scene& sc = scene(id);
    SPH_CK(cudaStreamSynchronize(st_));
    pa_.release(sc.p_off, sc.p_cap);
    ka_.release(sc.k_off, sc.k_cap);
    ca_.release(sc.c_off, sc.nchunks);
    tba_.release(sc.tab_off, sc.tab_len);
    if (sc.tw > 0) ta_.release(sc.t_off, round_up((int64_t)sc.tw * sc.td, kTAlign));
    sc.live = false;
    sc.n = 0;
    sc.steps = 0;
    int zero = 0;
    SPH_CK(cudaMemcpyAsync(steps_.p + id, &zero, sizeof(int), cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaStreamSynchronize(st_));
    work_dirty_ = true;
}

void System::set_params(int id, const sph_params& p) {
    validate_params(p);
    Scene& sc = scene(id);
    Scene ng = sc;
    ng.prm = p;
    geometry(ng);
    if (ng.k_cap != sc.k_cap || ng.nchunks != sc.nchunks || ng.tab_len != sc.tab_len) {
        SPH_CK(cudaStreamSynchronize(st_));
        ka_.release(sc.k_off, sc.k_cap);
        ca_.release(sc.c_off, sc.nchunks);
        tba_.release(sc.tab_off, sc.tab_len);
        // key ranges hold no state between steps (counts start from zero), so
        // a refused resize re-acquires ranges for the old grid, wherever
        // they land, and the scene keeps its old parameters
        auto place = [&](Scene& g) {
            ensure_arena(ka_, g.k_cap, 1);
            ensure_arena(ca_, g.nchunks, 2);
            ensure_arena(tba_, g.tab_len, 3);
            int64_t ko, co, to;
            if (!ka_.alloc(g.k_cap, &ko)) throw Error(SPH_ERR_NOMEM, "arena allocation failed");
            if (!ca_.alloc(g.nchunks, &co)) {
                ka_.release(ko, g.k_cap);
                throw Error(SPH_ERR_NOMEM, "arena allocation failed");
            }
            if (!tba_.alloc(g.tab_len, &to)) {
                ka_.release(ko, g.k_cap);
                ca_.release(co, g.nchunks);
                throw Error(SPH_ERR_NOMEM, "arena allocation failed");
            }
            g.k_off = ko;
            g.c_off = co;
            g.tab_off = to;
            std::vector<uint32_t> tab(g.tab_len);
            row_table(g.ny, g.nz, tab.data());
            SPH_CK(cudaMemcpyAsync(tab_.p + g.tab_off, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, st_));
            SPH_CK(cudaMemsetAsync(counts_.p + g.k_off, 0, (size_t)g.k_cap * 4, st_));
            SPH_CK(cudaMemsetAsync(chunk_.p + g.c_off, 0, (size_t)g.nchunks * 4, st_));
        };
        work_dirty_ = true;
        try {
            place(ng);
        } catch (...) {
            place(sc);  // the space just released fits the old grid
            upload_scene(id);
            SPH_CK(cudaStreamSynchronize(st_));
            throw;
        }
    } else if (ng.nx != sc.nx || ng.ny != sc.ny || ng.nz != sc.nz) {
        std::vector<uint32_t> tab(ng.tab_len);
        row_table(ng.ny, ng.nz, tab.data());
        SPH_CK(cudaMemcpyAsync(tab_.p + ng.tab_off, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, st_));
    }
    if ((p.flags & SPH_FLAG_RECORD) && rec_.n == 0) {
        SPH_CK(cudaStreamSynchronize(st_));
        rec_.resize(pos_.n * kRecFloats, false, st_);
        drop_graph();
    }
    if ((p.flags ^ sc.prm.flags) & (SPH_FLAG_ORDERED | SPH_FLAG_RECORD)) work_dirty_ = true;
    sc = ng;
    upload_scene(id);
}

void System::set_steps(int id, int steps) {
    Scene& sc = scene(id);
    sc.steps = steps < 0 ? -1 : steps;
    SPH_CK(cudaMemcpyAsync(steps_.p + id, &sc.steps, sizeof(int), cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaStreamSynchronize(st_));
    work_dirty_ = true;
}

void System::ensure_particle_cap(Scene& sc, int need) {
    if (need <= sc.p_cap) return;
    const int ncap = (int)round_up(std::max<int64_t>(need, (int64_t)sc.p_cap * 2), kPAlign);
    SPH_CK(cudaStreamSynchronize(st_));
    ensure_arena(pa_, ncap, 0);
    int64_t noff;
    if (!pa_.alloc(ncap, &noff)) throw Error(SPH_ERR_NOMEM, "arena allocation failed");
    if (sc.n > 0) {
        SPH_CK(cudaMemcpyAsync(pos_.p + noff, pos_.p + sc.p_off, (size_t)sc.n * 16, cudaMemcpyDeviceToDevice, st_));
        SPH_CK(cudaMemcpyAsync(vel_.p + noff, vel_.p + sc.p_off, (size_t)sc.n * 16, cudaMemcpyDeviceToDevice, st_));
        SPH_CK(cudaMemcpyAsync(nbid_.p + noff, nbid_.p + sc.p_off, (size_t)sc.n * 4, cudaMemcpyDeviceToDevice, st_));
        SPH_CK(cudaMemcpyAsync(dyn_.p + noff, dyn_.p + sc.p_off, (size_t)sc.n * 16, cudaMemcpyDeviceToDevice, st_));
        SPH_CK(cudaStreamSynchronize(st_));
    }
    pa_.release(sc.p_off, sc.p_cap);
    sc.p_off = noff;
    sc.p_cap = ncap;
    work_dirty_ = true;
}

void System::set_particles(int id, int n, const float* pos3, const float* vel3) {
    if (n < 0 || (n > 0 && !pos3)) throw Error(SPH_ERR_INVALID, "bad particle arrays");
    Scene& sc = scene(id);
    SPH_CK(cudaStreamSynchronize(st_));
    ensure_particle_cap(sc, n);
    std::vector<float4> hp(n), hv(n);
    std::vector<int32_t> nb(n, -1);
    for (int i = 0; i < n; ++i) {
        hp[i] = make_float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], bits_to_float(i));
        hv[i] = vel3 ? make_float4(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2], bits_to_float(0))
                     : make_float4(0.f, 0.f, 0.f, bits_to_float(0));
    }
    if (n > 0) {
        SPH_CK(cudaMemcpyAsync(pos_.p + sc.p_off, hp.data(), (size_t)n * 16, cudaMemcpyHostToDevice, st_));
        SPH_CK(cudaMemcpyAsync(vel_.p + sc.p_off, hv.data(), (size_t)n * 16, cudaMemcpyHostToDevice, st_));
        SPH_CK(cudaMemcpyAsync(nbid_.p + sc.p_off, nb.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st_));
        SPH_CK(cudaMemsetAsync(dyn_.p + sc.p_off, 0, (size_t)n * 16, st_));
    }
    SPH_CK(cudaStreamSynchronize(st_));
    if (sc.n != n) work_dirty_ = true;
    sc.n = n;
    upload_scene(id);
}

// Initialize(n) / AddParticles(n) (fluid_system.h:74-102, :232-251): a lattice
// of ceil(cbrt(n))^3 particles at spacing 0.025 from (-0.2,-0.05,-0.15) plus
// the origin, appended after the existing particles with the next ids.
int System::add_lattice(int id, int n, const float origin[3]) {
    if (n < 0) throw Error(SPH_ERR_INVALID, "negative count");
    Scene& sc = scene(id);
    std::vector<float4> hp, hv;
    const double cn = std::cbrt((double)n);
    int next = sc.n;
    for (int i = 0; i < cn; i++)
        for (int j = 0; j < cn; j++)
            for (int k = 0; k < cn; k++) {
                const float x = -0.2 + i * 0.025;
                const float y = -0.05 + j * 0.025;
                const float z = -0.15 + k * 0.025;
                hp.push_back(make_float4(x + origin[0], y + origin[1], z + origin[2], bits_to_float(next++)));
                hv.push_back(make_float4(0.f, 0.f, 0.f, bits_to_float(0)));
            }
    const int add = (int)hp.size();
    if (add == 0) return 0;
    SPH_CK(cudaStreamSynchronize(st_));
    ensure_particle_cap(sc, sc.n + add);
    std::vector<int32_t> nb(add, -1);
    SPH_CK(cudaMemcpyAsync(pos_.p + sc.p_off + sc.n, hp.data(), (size_t)add * 16, cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaMemcpyAsync(vel_.p + sc.p_off + sc.n, hv.data(), (size_t)add * 16, cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaMemcpyAsync(nbid_.p + sc.p_off + sc.n, nb.data(), (size_t)add * 4, cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaMemsetAsync(dyn_.p + sc.p_off + sc.n, 0, (size_t)add * 16, st_));
    SPH_CK(cudaStreamSynchronize(st_));
    sc.n += add;
    work_dirty_ = true;
    upload_scene(id);
    return add;
}

void System::get_particles(int id, float* pos3, float* vel3, float* density, int32_t* sed) {
    Range r("sph/readback");
    Scene& sc = scene(id);
    SPH_CK(cudaStreamSynchronize(st_));
    check_status();
    const int n = sc.n;
    if (n == 0) return;
    // gather into id order on the device, then copy only what was asked for
    if (stage_.n < (int64_t)8 * n) stage_.resize((int64_t)8 * n, false, st_);
    float* d_pos = stage_.p;
    float* d_vel = stage_.p + (size_t)3 * n;
    float* d_den = stage_.p + (size_t)6 * n;
    int32_t* d_sed = reinterpret_cast<int32_t*>(stage_.p + (size_t)7 * n);
    launch_gather_by_id(pos_.p, vel_.p, dyn_.p, (int)sc.p_off, n, pos3 ? d_pos : nullptr, vel3 ? d_vel : nullptr,
                        density ? d_den : nullptr, sed ? d_sed : nullptr, st_);
    SPH_CK(cudaGetLastError());
    if (pos3) SPH_CK(cudaMemcpyAsync(pos3, d_pos, (size_t)n * 12, cudaMemcpyDeviceToHost, st_));
    if (vel3) SPH_CK(cudaMemcpyAsync(vel3, d_vel, (size_t)n * 12, cudaMemcpyDeviceToHost, st_));
    if (density) SPH_CK(cudaMemcpyAsync(density, d_den, (size_t)n * 4, cudaMemcpyDeviceToHost, st_));
    if (sed) SPH_CK(cudaMemcpyAsync(sed, d_sed, (size_t)n * 4, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaStreamSynchronize(st_));
}

// The same readback without waiting: the gather into id order runs on the
// library stream after the work already enqueued (so it sees the state of the
// last step), the copies into the caller's buffers on a second stream, so
// that they overlap the steps enqueued next.  Two staging buffers alternate;
// a gather waits for the copies that last used its buffer.  The caller's
// buffers are complete after sph_system_sync; with pageable buffers the
// copies cannot overlap anything (the driver completes them before
// returning), so the caller should pass pinned memory.
void System::get_particles_async(int id, float* pos3, float* vel3, float* density, int32_t* sed) {
    Range r("sph/readback_async");
    Scene& sc = scene(id);
    const int n = sc.n;
    if (n == 0) return;
    const int k = aslot_;
    aslot_ ^= 1;
    if (astage_[k].n < (int64_t)8 * n) {
        SPH_CK(cudaStreamSynchronize(cst_));
        astage_[k].resize((int64_t)8 * n, false, st_);
    }
    SPH_CK(cudaStreamWaitEvent(st_, copied_[k], 0));
    float* d_pos = astage_[k].p;
    float* d_vel = astage_[k].p + (size_t)3 * n;
    float* d_den = astage_[k].p + (size_t)6 * n;
    int32_t* d_sed = reinterpret_cast<int32_t*>(astage_[k].p + (size_t)7 * n);
    launch_gather_by_id(pos_.p, vel_.p, dyn_.p, (int)sc.p_off, n, pos3 ? d_pos : nullptr, vel3 ? d_vel : nullptr,
                        density ? d_den : nullptr, sed ? d_sed : nullptr, st_);
    SPH_CK(cudaGetLastError());
    SPH_CK(cudaEventRecord(gathered_[k], st_));
    SPH_CK(cudaStreamWaitEvent(cst_, gathered_[k], 0));
    if (pos3) SPH_CK(cudaMemcpyAsync(pos3, d_pos, (size_t)n * 12, cudaMemcpyDeviceToHost, cst_));
    if (vel3) SPH_CK(cudaMemcpyAsync(vel3, d_vel, (size_t)n * 12, cudaMemcpyDeviceToHost, cst_));
    if (density) SPH_CK(cudaMemcpyAsync(density, d_den, (size_t)n * 4, cudaMemcpyDeviceToHost, cst_));
    if (sed) SPH_CK(cudaMemcpyAsync(sed, d_sed, (size_t)n * 4, cudaMemcpyDeviceToHost, cst_));
    SPH_CK(cudaEventRecord(copied_[k], cst_));
}

void System::get_records(int id, float* rec27, int* nbid, int32_t* sed) {
    Scene& sc = scene(id);
    SPH_CK(cudaStreamSynchronize(st_));
    check_status();
    const int n = sc.n;
    if (n == 0) return;
    std::vector<float4> hp(n), hv(n), hd(n);
    std::vector<float> hr;
    std::vector<int32_t> hn(n);
    SPH_CK(cudaMemcpyAsync(hp.data(), pos_.p + sc.p_off, (size_t)n * 16, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaMemcpyAsync(hv.data(), vel_.p + sc.p_off, (size_t)n * 16, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaMemcpyAsync(hd.data(), dyn_.p + sc.p_off, (size_t)n * 16, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaMemcpyAsync(hn.data(), nbid_.p + sc.p_off, (size_t)n * 4, cudaMemcpyDeviceToHost, st_));
    const bool have_rec = (sc.prm.flags & SPH_FLAG_RECORD) && rec_.n > 0;
    if (have_rec) {
        hr.resize((size_t)n * kRecFloats);
        SPH_CK(cudaMemcpyAsync(hr.data(), rec_.p + (size_t)sc.p_off * kRecFloats, hr.size() * 4,
                               cudaMemcpyDeviceToHost, st_));
    }
    SPH_CK(cudaStreamSynchronize(st_));
    for (int p = 0; p < n; ++p) {
        const int i = float_to_bits(hp[p].w);
        if (i < 0 || i >= n) throw Error(SPH_ERR_DEVICE, "corrupt particle id");
        if (rec27) {
            float* r = rec27 + (size_t)27 * i;
            r[0] = hp[p].x; r[1] = hp[p].y; r[2] = hp[p].z;
            r[3] = hv[p].x; r[4] = hv[p].y; r[5] = hv[p].z;
            r[9] = hd[p].x;
            r[10] = hd[p].w;
            for (int q = 0; q < kRecFloats; ++q) {
                const int dst = q < 3 ? 6 + q : 8 + q;  // acc -> 6..8, forces/normal -> 11..25
                r[dst] = have_rec ? hr[(size_t)p * kRecFloats + q] : 0.0f;
            }
            r[26] = 0.0f;
        }
        if (nbid) nbid[i] = hn[p];
        if (sed) sed[i] = float_to_bits(hv[p].w);
    }
}

void System::diag(int id, sph_diag* out) { diag_many(&id, 1, out); }

// FP64 diagnostics, mass units and state fingerprints of k scenes: one
// launch, one set of copies, one wait.
void System::diag_many(const int* ids, int k, sph_diag* out) {
    if (k > cfg_.max_scenes) throw Error(SPH_ERR_INVALID, "more scenes than the system holds");
    for (int q = 0; q < k; ++q) scene(ids[q]);
    if (work_dirty_) rebuild_work();
    if (diag_part_.n < (int64_t)k * kDiagBlocks * kDiagDoubles)
        diag_part_.resize((int64_t)k * kDiagBlocks * kDiagDoubles, false, st_);
    if (diag_i_.n < (int64_t)3 * k) diag_i_.resize((int64_t)3 * k, false, st_);
    if (diag_nan_.n < k) diag_nan_.resize(k, false, st_);
    SPH_CK(cudaMemcpyAsync(slist_.p, ids, (size_t)k * sizeof(int), cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaMemsetAsync(diag_i_.p, 0, (size_t)3 * k * sizeof(long long), st_));
    SPH_CK(cudaMemsetAsync(diag_nan_.p, 0, (size_t)k * sizeof(int), st_));
    launch_diag(arrays(), k, diag_part_.p, diag_i_.p, diag_nan_.p, st_);
    SPH_CK(cudaGetLastError());
    std::vector<double> part((size_t)k * kDiagBlocks * kDiagDoubles);
    std::vector<long long> is((size_t)3 * k);
    std::vector<int> nan(k);
    SPH_CK(cudaMemcpyAsync(part.data(), diag_part_.p, part.size() * 8, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaMemcpyAsync(is.data(), diag_i_.p, is.size() * 8, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaMemcpyAsync(nan.data(), diag_nan_.p, nan.size() * 4, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaStreamSynchronize(st_));
    for (int q = 0; q < k; ++q) {
        const Scene& sc = scene(ids[q]);
        double acc[kDiagDoubles] = {0};
        for (int b = 0; b < kDiagBlocks; ++b)
            for (int c = 0; c < kDiagDoubles; ++c)
                acc[c] += part[((size_t)q * kDiagBlocks + b) * kDiagDoubles + c];
        sph_diag* o = out + q;
        std::memset(o, 0, sizeof *o);
        o->fluid_mass = (double)sc.n * (double)sc.prm.mass;
        o->momentum[0] = acc[0];
        o->momentum[1] = acc[1];
        o->momentum[2] = acc[2];
        o->kinetic = acc[3];
        o->potential = acc[4];
        o->sediment_units = is[3 * q];
        o->terrain_units = is[3 * q + 1];
        o->total_units = is[3 * q] + is[3 * q + 1];
        o->unit_volume = ((double)sc.prm.mass / (double)sc.prm.rest_density) * std::ldexp(1.0, -30);
        o->n = sc.n;
        o->nan_particles = nan[q];
        o->state_hash = (uint64_t)is[3 * q + 2];
    }
}

void System::upload_terrain_height(Scene& sc) {
    // snapshot = base + delta * unit with delta = 0
    SPH_CK(cudaMemcpyAsync(theight_.p + sc.t_off, tbase_.p + sc.t_off, (size_t)sc.tw * sc.td * 4,
                           cudaMemcpyDeviceToDevice, st_));
}

void System::set_terrain(int id, int w, int d, const float* heights) {
    Scene& sc = scene(id);
    if (w == 0 && d == 0) {
        // no terrain: the step's contact and erosion are off for this scene
        SPH_CK(cudaStreamSynchronize(st_));
        if (sc.tw > 0) ta_.release(sc.t_off, round_up((int64_t)sc.tw * sc.td, kTAlign));
        sc.tw = sc.td = 0;
        sc.t_off = 0;
        upload_scene(id);
        work_dirty_ = true;
        return;
    }
    if (w < 2 || d < 2 || !heights) throw Error(SPH_ERR_INVALID, "terrain needs at least 2 x 2 heights");
    SPH_CK(cudaStreamSynchronize(st_));
    if (w != sc.tw || d != sc.td) {
        if (sc.tw > 0) ta_.release(sc.t_off, round_up((int64_t)sc.tw * sc.td, kTAlign));
        const int64_t tlen = round_up((int64_t)w * d, kTAlign);
        ensure_arena(ta_, tlen, 4);
        if (!ta_.alloc(tlen, &sc.t_off)) throw Error(SPH_ERR_NOMEM, "arena allocation failed");
        sc.tw = w;
        sc.td = d;
        work_dirty_ = true;
    }
    SPH_CK(cudaMemcpyAsync(tbase_.p + sc.t_off, heights, (size_t)w * d * 4, cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaMemsetAsync(tdelta_.p + sc.t_off, 0, (size_t)w * d * 8, st_));
    upload_terrain_height(sc);
    SPH_CK(cudaStreamSynchronize(st_));
    upload_scene(id);
    work_dirty_ = true;
}

void System::gen_terrain(int id, uint64_t seed, int octaves, float amp, float lac, float gain, int kind) {
    Scene& sc = scene(id);
    if (sc.tw < 2) throw Error(SPH_ERR_STATE, "scene has no terrain grid");
    std::vector<float> h((size_t)sc.tw * sc.td);
    fbm_heights(seed, sc.tw, sc.td, octaves, amp, lac, gain, kind, h.data());
    set_terrain(id, sc.tw, sc.td, h.data());
}

void System::get_terrain(int id, float* heights, int64_t* delta) {
    Scene& sc = scene(id);
    if (sc.tw < 2) throw Error(SPH_ERR_STATE, "scene has no terrain");
    SPH_CK(cudaStreamSynchronize(st_));
    const size_t nt = (size_t)sc.tw * sc.td;
    if (heights) SPH_CK(cudaMemcpyAsync(heights, theight_.p + sc.t_off, nt * 4, cudaMemcpyDeviceToHost, st_));
    if (delta) SPH_CK(cudaMemcpyAsync(delta, tdelta_.p + sc.t_off, nt * 8, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaStreamSynchronize(st_));
}

void System::terrain_dims(int id, int* w, int* d) const {
    const Scene& sc = scene(id);
    *w = sc.tw;
    *d = sc.td;
}

void System::grid_dims(int id, int* dims4) const {
    const Scene& sc = scene(id);
    dims4[0] = sc.nx;
    dims4[1] = sc.ny;
    dims4[2] = sc.nz;
    dims4[3] = sc.nkeys;
}

// ---- work lists and launches -------------------------------------------------
void System::rebuild_work() {
    std::vector<Work> pt, ct, tt;
    any_fast_ = any_ordered_ = any_terrain_ = any_limited_ = any_record_ = false;
    const int tile = cfg_.tile;
    for (int id = 0; id < (int)scenes_.size(); ++id) {
        const Scene& sc = scenes_[id];
        if (!sc.live || sc.n == 0) continue;
        for (int t = 0; t * tile < sc.n; ++t) pt.push_back({id, (int)sc.p_off + t * tile});
        for (int c = 0; c < sc.nchunks; ++c) ct.push_back({id, c});
        if (sc.tw > 0)
            for (int64_t t = 0; t * tile < (int64_t)sc.tw * sc.td; ++t) tt.push_back({id, (int)(sc.t_off + t * tile)});
        if (sc.prm.flags & SPH_FLAG_ORDERED)
            any_ordered_ = true;
        else
            any_fast_ = true;
        if (sc.tw > 0) any_terrain_ = true;
        if (sc.prm.flags & SPH_FLAG_RECORD) any_record_ = true;
    }
    for (const Scene& sc : scenes_)
        if (sc.live && sc.steps >= 0) any_limited_ = true;
    auto up = [&](DevBuf<Work>& b, const std::vector<Work>& v) {
        if ((int64_t)v.size() > b.n) {
            b.resize(std::max<int64_t>((int64_t)v.size(), b.n * 2), false, st_);
            drop_graph();
        }
        if (!v.empty())
            SPH_CK(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(Work), cudaMemcpyHostToDevice, st_));
    };
    up(ptiles_, pt);
    up(ctiles_, ct);
    up(ttiles_, tt);
    int counts[4] = {(int)pt.size(), (int)ct.size(), (int)tt.size(), 0};
    SPH_CK(cudaMemcpyAsync(nwork_.p, counts, sizeof counts, cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaStreamSynchronize(st_));
    if (n_ptiles_ != counts[0] || n_ctiles_ != counts[1] || n_ttiles_ != counts[2]) drop_graph();
    n_ptiles_ = counts[0];
    n_ctiles_ = counts[1];
    n_ttiles_ = counts[2];
    work_dirty_ = false;
    ensure_nlist();
    drop_graph();
}

// Neighbour lists for variant bit 3, sized to the particle arena.  Without
// room in the HBM budget the variant runs without them (bit 3 ignored).
void System::ensure_nlist() {
    nl_ready_ = false;
    if (!(cfg_.variant & 8) || !any_fast_) {
        if (nlist_.n || fdat_.n) {
            nlist_.release();
            ncnt_.release();
            fdat_.release();
            drop_graph();
        }
        return;
    }
    const int64_t slots = (int64_t)kNbCap * pos_.n;
    const int64_t recs = (cfg_.variant & 128) ? 2 * pos_.n : 0;
    if (nlist_.n != slots || ncnt_.n != pos_.n || fdat_.n != recs) {
        const int64_t extra = (slots - nlist_.n) * 4 + (pos_.n - ncnt_.n) * 4 + (recs - fdat_.n) * 16;
        if (cfg_.hbm_budget > 0 && memory_bytes() + extra > cfg_.hbm_budget) return;
        nlist_.resize(slots, false, st_);
        ncnt_.resize(pos_.n, false, st_);
        if (recs)
            fdat_.resize(recs, false, st_);
        else
            fdat_.release();
        drop_graph();
    }
    nl_ready_ = true;
    ensure_fmap();
}

// The tensor map of the packed records: fdat_ seen as a 2-D tensor of
// float32, 8 wide (one particle's two float4), one row per arena particle,
// copied one row per box (the shape tile::gather4 takes).  Built through the
// driver's cuTensorMapEncodeTiled, reached via the runtime's entry-point
// query; without it (or without packed records) the force pass keeps its
// other forms.
void System::ensure_fmap() {
    if (!(cfg_.variant & 262144) || fdat_.n == 0) {
        fmap_ok_ = false;
        return;
    }
    const int64_t rows = fdat_.n / 2;
    if (fmap_ok_ && fmap_base_ == fdat_.p && fmap_rows_ == rows) return;
    fmap_ok_ = false;
    using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static Encode encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn) {
            cudaGetLastError();
            return;
        }
        encode = reinterpret_cast<Encode>(fn);
    }
    if (rows >= ((int64_t)1 << 31)) return;
    const cuuint64_t dims[2] = {8, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {32};
    const cuuint32_t box[2] = {8, 1};
    const cuuint32_t elem[2] = {1, 1};
    if (encode(&fmap_, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, fdat_.p, dims, strides, box, elem,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return;
    fmap_base_ = fdat_.p;
    fmap_rows_ = rows;
    fmap_ok_ = true;
    drop_graph();
}

DevArrays System::arrays() const {
    DevArrays a;
    a.scenes = dscenes_.p;
    a.steps_left = steps_.p;
    a.ptiles = ptiles_.p;
    a.n_ptiles = nwork_.p;
    a.ctiles = ctiles_.p;
    a.n_ctiles = nwork_.p + 1;
    a.ttiles = ttiles_.p;
    a.n_ttiles = nwork_.p + 2;
    a.scene_list = slist_.p;
    a.pos = pos_.p;
    a.vel = vel_.p;
    a.spos = spos_.p;
    a.svel = svel_.p;
    a.dyn = dyn_.p;
    a.key = key_.p;
    a.slot = slot_.p;
    a.perm = perm_.p;
    a.nbid = nbid_.p;
    a.snbid = snbid_.p;
    a.rec = rec_.p;
    a.nlist = nlist_.p;
    a.ncnt = ncnt_.p;
    a.fdat = fdat_.p;
    a.counts = counts_.p;
    a.offsets = offsets_.p;
    a.chunk_sum = chunk_.p;
    a.tab = tab_.p;
    a.tbase = tbase_.p;
    a.tdelta = tdelta_.p;
    a.theight = theight_.p;
    a.status = status_.p;
    a.ctr = status_.p + 1;
    a.tile = cfg_.tile;
    return a;
}

LaunchShape System::shape() const {
    LaunchShape s;
    s.tile = cfg_.tile;
    s.grid_p = n_ptiles_;
    s.grid_c = n_ctiles_;
    s.grid_t = n_ttiles_;
    s.variant = nl_ready_ ? cfg_.variant : (cfg_.variant & ~504);
    // enough blocks to fill every SM (2048 threads each); blocks that start
    // after the counter ran out exit at once
    const int64_t slices = (int64_t)n_ptiles_ * (cfg_.tile / 32);
    s.grid_dyn = (int)std::min<int64_t>((slices * 32 + cfg_.tile - 1) / cfg_.tile, (int64_t)nsm_ * (2048 / cfg_.tile));
    s.fmap = (nl_ready_ && fmap_ok_) ? &fmap_ : nullptr;
    return s;
}

void System::enqueue_sort(const DevArrays& a, const LaunchShape& s) {
    launch_keys(a, s, st_);
    launch_scan(a, s, st_);
    launch_scatter(a, s, st_);
    launch_reorder(a, s, st_);
}

void System::enqueue_step(const DevArrays& a, const LaunchShape& s, cudaEvent_t* ev) {
    auto mark = [&](int i) {
        if (ev) SPH_CK(cudaEventRecord(ev[i], st_));
    };
    mark(0);
    {
        Range r("sph/sort");
        launch_keys(a, s, st_);
        mark(1);
        launch_scan(a, s, st_);
        mark(2);
        launch_scatter(a, s, st_);
        mark(3);
        launch_reorder(a, s, st_);
        mark(4);
    }
    {
        Range r("sph/density");
        if (any_fast_) launch_density(a, s, st_);
        if (any_ordered_) launch_density_ordered(a, s, st_);
        mark(5);
    }
    {
        Range r("sph/force");
        if (any_fast_) launch_force(a, s, st_);
        if (any_ordered_) launch_force_ordered(a, s, st_);
        mark(6);
    }
    {
        Range r("sph/terrain");
        if (any_terrain_ && s.grid_t > 0) launch_terrain(a, s, st_);
        mark(7);
        if (any_limited_) launch_tick(a, (int)scenes_.size(), st_);
        mark(8);
    }
}

void System::capture_graph() {
    Range r("sph/capture_graph");
    drop_graph();
    const DevArrays a = arrays();
    const LaunchShape s = shape();
    SPH_CK(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < cfg_.graph_steps; ++i) enqueue_step(a, s, nullptr);
    cudaGraph_t g = nullptr;
    SPH_CK(cudaStreamEndCapture(st_, &g));
    graph_ = g;
    SPH_CK(cudaGraphInstantiate(&gexec_, graph_, 0));
    graph_dirty_ = false;
}

void System::step(int nsteps) {
    Range r("sph/step");
    if (nsteps < 0) throw Error(SPH_ERR_INVALID, "negative step count");
    if (work_dirty_) rebuild_work();
    if (n_ptiles_ > 0 && nsteps > 0) {
        const DevArrays a = arrays();
        const LaunchShape s = shape();
        int done = 0;
        const int g = cfg_.graph_steps;
        if (g > 0 && nsteps >= g) {
            if (graph_dirty_ || !gexec_) capture_graph();
            while (nsteps - done >= g) {
                SPH_CK(cudaGraphLaunch(gexec_, st_));
                done += g;
            }
        }
        for (; done < nsteps; ++done) enqueue_step(a, s, nullptr);
        SPH_CK(cudaGetLastError());
        advance_step_mirror(nsteps);
    }
}

// Host copy of the per-scene step budgets, decremented like k_tick does.
void System::advance_step_mirror(int nsteps) {
    if (!any_limited_) return;
    for (Scene& sc : scenes_)
        if (sc.live && sc.steps > 0) sc.steps = std::max(0, sc.steps - nsteps);
}

void System::sync() {
    SPH_CK(cudaStreamSynchronize(st_));
    SPH_CK(cudaStreamSynchronize(cst_));
    check_status();
}

// Kernel-reported conditions (ordered-mode neighbour overflow) become an
// error of the next host call that reads results.
void System::check_status() {
    const unsigned v = read_status();
    if (v == 0) return;
    const unsigned zero = 0;
    SPH_CK(cudaMemcpyAsync(status_.p, &zero, sizeof zero, cudaMemcpyHostToDevice, st_));
    SPH_CK(cudaStreamSynchronize(st_));
    if (v & 1u)
        throw Error(SPH_ERR_DEVICE, "ordered mode: a particle had more in-range neighbours than the list holds");
    if (v & 2u) throw Error(SPH_ERR_DEVICE, "counting sort found inconsistent cell counts");
    if (v & 4u) throw Error(SPH_ERR_DEVICE, "the force pass's TMA pipeline timed out waiting for a stage");
    throw Error(SPH_ERR_DEVICE, "kernel status " + std::to_string(v));
}

float System::time_steps(int nsteps) {
    if (work_dirty_) rebuild_work();
    if (cfg_.graph_steps > 0 && nsteps >= cfg_.graph_steps && (graph_dirty_ || !gexec_) && n_ptiles_ > 0)
        capture_graph();
    cudaEvent_t e0, e1;
    SPH_CK(cudaEventCreate(&e0));
    SPH_CK(cudaEventCreate(&e1));
    SPH_CK(cudaEventRecord(e0, st_));
    step(nsteps);
    SPH_CK(cudaEventRecord(e1, st_));
    SPH_CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    SPH_CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

void System::profile_stages(int nsteps, float* ms) {
    if (work_dirty_) rebuild_work();
    for (int i = 0; i < 8; ++i) ms[i] = 0.f;
    if (n_ptiles_ == 0 || nsteps <= 0) return;
    cudaEvent_t ev[9];
    for (auto& e : ev) SPH_CK(cudaEventCreate(&e));
    const DevArrays a = arrays();
    const LaunchShape s = shape();
    for (int k = 0; k < nsteps; ++k) {
        enqueue_step(a, s, ev);
        SPH_CK(cudaEventSynchronize(ev[8]));
        for (int i = 0; i < 8; ++i) {
            float t = 0.f;
            SPH_CK(cudaEventElapsedTime(&t, ev[i], ev[i + 1]));
            ms[i] += t;
        }
    }
    for (int i = 0; i < 8; ++i) ms[i] /= (float)nsteps;
    for (auto& e : ev) cudaEventDestroy(e);
    advance_step_mirror(nsteps);
}

unsigned System::read_status() {
    unsigned v = 0;
    SPH_CK(cudaMemcpyAsync(&v, status_.p, sizeof v, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaStreamSynchronize(st_));
    return v;
}

void System::debug_sort(int id, uint32_t* keys_by_id, int32_t* sorted_ids) {
    Scene& sc = scene(id);
    if (work_dirty_) rebuild_work();
    if (sc.n == 0) return;
    enqueue_sort(arrays(), shape());
    SPH_CK(cudaGetLastError());
    const int n = sc.n;
    std::vector<float4> hp(n), hs(n);
    std::vector<uint32_t> hk(n);
    SPH_CK(cudaMemcpyAsync(hp.data(), pos_.p + sc.p_off, (size_t)n * 16, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaMemcpyAsync(hs.data(), spos_.p + sc.p_off, (size_t)n * 16, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaMemcpyAsync(hk.data(), key_.p + sc.p_off, (size_t)n * 4, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaStreamSynchronize(st_));
    for (int i = 0; i < n; ++i) {
        const int pid = float_to_bits(hp[i].w);
        if (keys_by_id) keys_by_id[pid] = hk[i];
        if (sorted_ids) sorted_ids[i] = float_to_bits(hs[i].w);
    }
}

void System::traversal_stats(int id, int64_t* out4) {
    Scene& sc = scene(id);
    if (work_dirty_) rebuild_work();
    out4[0] = sc.n;
    out4[1] = out4[2] = out4[3] = 0;
    if (sc.n == 0) return;
    const DevArrays a = arrays();
    enqueue_sort(a, shape());
    if (diag_i_.n < 4) diag_i_.resize(4, false, st_);
    SPH_CK(cudaMemsetAsync(diag_i_.p, 0, 4 * sizeof(long long), st_));
    launch_traversal_stats(a, id, reinterpret_cast<unsigned long long*>(diag_i_.p), st_);
    SPH_CK(cudaGetLastError());
    long long h[3];
    SPH_CK(cudaMemcpyAsync(h, diag_i_.p, sizeof h, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaStreamSynchronize(st_));
    out4[1] = h[0];
    out4[2] = h[1];
    out4[3] = h[2];
}

void System::neighbour_counts(int id, int32_t* out) {
    Scene& sc = scene(id);
    if (work_dirty_) rebuild_work();
    if (sc.n == 0) return;
    if (scratch_i_.n < pos_.n) scratch_i_.resize(pos_.n, false, st_);
    const DevArrays a = arrays();
    enqueue_sort(a, shape());
    launch_neighbour_counts(a, shape(), scratch_i_.p, st_);
    SPH_CK(cudaGetLastError());
    SPH_CK(cudaMemcpyAsync(out, scratch_i_.p + sc.p_off, (size_t)sc.n * 4, cudaMemcpyDeviceToHost, st_));
    SPH_CK(cudaStreamSynchronize(st_));
}

// ---- autotuner ------------------------------------------------------------------
void System::autotune(int steps, sph_tune_result* out) {
    Range r("sph/autotune");
    if (steps <= 0) throw Error(SPH_ERR_INVALID, "autotune needs steps > 0");
    std::memset(out, 0, sizeof *out);
    if (work_dirty_) rebuild_work();
    SPH_CK(cudaStreamSynchronize(st_));
    // snapshot of every scene's evolving state: particles (whole arena, so
    // ranges stay valid), terrain deltas and heights, step budgets
    const int64_t np = pos_.n, nt = tbase_.n;
    DevBuf<float4> spos, svel;
    DevBuf<int32_t> snb;
    DevBuf<long long> sdel;
    DevBuf<float> shgt;
    spos.resize(np, false, st_);
    svel.resize(np, false, st_);
    snb.resize(np, false, st_);
    sdel.resize(nt, false, st_);
    shgt.resize(nt, false, st_);
    auto copy = [&](void* dst, const void* src, size_t bytes) {
        if (bytes) SPH_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st_));
    };
    copy(spos.p, pos_.p, np * 16);
    copy(svel.p, vel_.p, np * 16);
    copy(snb.p, nbid_.p, np * 4);
    copy(sdel.p, tdelta_.p, nt * 8);
    copy(shgt.p, theight_.p, nt * 4);
    std::vector<int> steps0;
    for (const Scene& sc : scenes_) steps0.push_back(sc.steps);
    SPH_CK(cudaStreamSynchronize(st_));
    auto restore = [&]() {
        copy(pos_.p, spos.p, np * 16);
        copy(vel_.p, svel.p, np * 16);
        copy(nbid_.p, snb.p, np * 4);
        copy(tdelta_.p, sdel.p, nt * 8);
        copy(theight_.p, shgt.p, nt * 4);
        for (size_t i = 0; i < scenes_.size(); ++i)
            if (scenes_[i].live) set_steps((int)i, steps0[i]);
        SPH_CK(cudaStreamSynchronize(st_));
    };
    auto apply = [&](int tile, float cm, int variant) {
        if (cfg_.tile != tile || cfg_.variant != variant) {
            cfg_.tile = tile;
            cfg_.variant = variant;
            work_dirty_ = true;
            drop_graph();
        }
        for (size_t i = 0; i < scenes_.size(); ++i) {
            if (!scenes_[i].live || scenes_[i].prm.cell_mult == cm) continue;
            sph_params p = scenes_[i].prm;
            p.cell_mult = cm;
            set_params((int)i, p);
        }
        if (pos_.n != np || tbase_.n != nt) throw Error(SPH_ERR_STATE, "arena changed while tuning");
    };
    auto free_snapshot = [&]() {
        spos.release();
        svel.release();
        snb.release();
        sdel.release();
        shgt.release();
    };
    const int tiles[2] = {128, 256};
    const float cms[2] = {1.0f, 0.5f};
    // per-lane passes (0, 4: cells; 28, 88, 120, 216: lists; 32856, 32888:
    // the force pass in dynamically scheduled warp slices; 163928, 163960,
    // 164088: the same in fast arithmetic, 164088 with packed records) and
    // cooperative passes (264: 32 + 8 lanes per particle, 776: 4 force
    // lanes, 2312: 16 density lanes).  The TMA gather pipeline (bit 18) is
    // left out: 3-4x slower than 164088 on every state measured.
    const int variants[] = {0,      4,      28,     88,  120, 216, 32856, 32888,
                            163928, 163960, 164088, 264, 776, 2312};
    static_assert(2 * 2 * (sizeof variants / sizeof variants[0]) <= 64, "sph_tune_result holds 64 trials");
    float best = 1e30f;
    int bt = cfg_.tile, bv = cfg_.variant;
    float bc = scenes_.empty() ? 1.0f : scenes_[0].prm.cell_mult;
    try {
        for (float cm : cms)
            for (int variant : variants)
                for (int tile : tiles) {
                    apply(tile, cm, variant);
                    step(2);  // warm-up: graphs captured, caches primed
                    SPH_CK(cudaStreamSynchronize(st_));
                    const float ms = time_steps(steps) / (float)steps;
                    restore();
                    const int k = out->n_tried++;
                    out->tiles[k] = tile;
                    out->cell_mults[k] = cm;
                    out->variants[k] = variant;
                    out->ms[k] = ms;
                    if (ms < best) {
                        best = ms;
                        bt = tile;
                        bc = cm;
                        bv = variant;
                    }
                }
        apply(bt, bc, bv);
        restore();
    } catch (...) {
        free_snapshot();
        throw;
    }
    free_snapshot();
    out->tile = bt;
    out->cell_mult = bc;
    out->variant = bv;
    out->ms_per_step = best;
}

template struct DevBuf<float4>;
template struct DevBuf<float>;
template struct DevBuf<uint32_t>;
template struct DevBuf<int32_t>;
template struct DevBuf<long long>;
template struct DevBuf<double>;
template struct DevBuf<SceneDev>;
template struct DevBuf<Work>;

}  // namespace sph
