// Scene checkpoint / restore and 8-bit heightfield ingest.
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "sph_engine.h"

namespace sph {

namespace {

constexpr char kMagic[4] = {'S', 'P', 'H', 'E'};
constexpr uint32_t kVersion = 1;

struct File {
    FILE* f = nullptr;
    std::string path;
    File(const char* p, const char* mode) : path(p ? p : "") {
        if (!p) throw Error(SPH_ERR_INVALID, "null path");
        f = std::fopen(p, mode);
        if (!f) throw Error(SPH_ERR_INVALID, "cannot open " + path);
    }
    ~File() {
        if (f) std::fclose(f);
    }
    void put(const void* d, size_t n) {
        if (n && std::fwrite(d, 1, n, f) != n) throw Error(SPH_ERR_INVALID, "write failed: " + path);
    }
    void get(void* d, size_t n) {
        if (n && std::fread(d, 1, n, f) != n) throw Error(SPH_ERR_INVALID, "truncated checkpoint: " + path);
    }
    void close() {
        if (f && std::fclose(f) != 0) {
            f = nullptr;
            throw Error(SPH_ERR_INVALID, "close failed: " + path);
        }
        f = nullptr;
    }
};

}  // namespace

void System::save(int id, const char* path) {
    Scene& sc = scene(id);
    SPH_CK(cudaStreamSynchronize(st_));
    check_status();
    const int n = sc.n;
    const size_t nt = (size_t)sc.tw * sc.td;
    std::vector<float4> hp(n), hv(n);
    std::vector<int32_t> hn(n);
    std::vector<float> base(nt);
    std::vector<long long> delta(nt);
    if (n) {
        SPH_CK(cudaMemcpyAsync(hp.data(), pos_.p + sc.p_off, (size_t)n * 16, cudaMemcpyDeviceToHost, st_));
        SPH_CK(cudaMemcpyAsync(hv.data(), vel_.p + sc.p_off, (size_t)n * 16, cudaMemcpyDeviceToHost, st_));
        SPH_CK(cudaMemcpyAsync(hn.data(), nbid_.p + sc.p_off, (size_t)n * 4, cudaMemcpyDeviceToHost, st_));
    }
    if (nt) {
        SPH_CK(cudaMemcpyAsync(base.data(), tbase_.p + sc.t_off, nt * 4, cudaMemcpyDeviceToHost, st_));
        SPH_CK(cudaMemcpyAsync(delta.data(), tdelta_.p + sc.t_off, nt * 8, cudaMemcpyDeviceToHost, st_));
    }
    SPH_CK(cudaStreamSynchronize(st_));
    File f(path, "wb");
    const uint32_t psize = sizeof(sph_params);
    const int32_t hdr[4] = {n, sc.tw, sc.td, sc.steps};
    f.put(kMagic, 4);
    f.put(&kVersion, 4);
    f.put(&psize, 4);
    f.put(&sc.prm, psize);
    f.put(hdr, sizeof hdr);
    f.put(hp.data(), (size_t)n * 16);
    f.put(hv.data(), (size_t)n * 16);
    f.put(hn.data(), (size_t)n * 4);
    f.put(base.data(), nt * 4);
    f.put(delta.data(), nt * 8);
    f.close();
}

void System::load(int id, const char* path) {
    scene(id);
    File f(path, "rb");
    char magic[4];
    uint32_t version = 0, psize = 0;
    f.get(magic, 4);
    f.get(&version, 4);
    f.get(&psize, 4);
    if (std::memcmp(magic, kMagic, 4) != 0 || version != kVersion || psize != sizeof(sph_params))
        throw Error(SPH_ERR_INVALID, "not a version-1 scene checkpoint: " + f.path);
    sph_params prm;
    f.get(&prm, psize);
    int32_t hdr[4];
    f.get(hdr, sizeof hdr);
    const int n = hdr[0], tw = hdr[1], td = hdr[2], steps = hdr[3];
    if (n < 0 || tw < 0 || td < 0 || (tw > 0) != (td > 0)) throw Error(SPH_ERR_INVALID, "corrupt checkpoint header");
    const size_t nt = (size_t)tw * td;
    std::vector<float4> hp(n), hv(n);
    std::vector<int32_t> hn(n);
    std::vector<float> base(nt);
    std::vector<long long> delta(nt);
    f.get(hp.data(), (size_t)n * 16);
    f.get(hv.data(), (size_t)n * 16);
    f.get(hn.data(), (size_t)n * 4);
    f.get(base.data(), nt * 4);
    f.get(delta.data(), nt * 8);
    for (int i = 0; i < n; ++i) {
        int pid;
        std::memcpy(&pid, &hp[i].w, 4);
        if (pid < 0 || pid >= n) throw Error(SPH_ERR_INVALID, "corrupt particle id in checkpoint");
    }
    if (nt == 0 && scene(id).tw > 0) throw Error(SPH_ERR_STATE, "checkpoint has no terrain but the scene has one");
    set_params(id, prm);
    if (nt) {
        set_terrain(id, tw, td, base.data());  // base heights, deltas cleared
        Scene& sc = scene(id);
        // snapshot heights = base + delta * unit, rounded as the terrain kernel does
        std::vector<float> h(nt);
        const float hu = sc.dev.height_unit;
        for (size_t t = 0; t < nt; ++t) h[t] = base[t] + (float)delta[t] * hu;
        SPH_CK(cudaMemcpyAsync(tdelta_.p + sc.t_off, delta.data(), nt * 8, cudaMemcpyHostToDevice, st_));
        SPH_CK(cudaMemcpyAsync(theight_.p + sc.t_off, h.data(), nt * 4, cudaMemcpyHostToDevice, st_));
    }
    Scene& sc = scene(id);
    SPH_CK(cudaStreamSynchronize(st_));
    ensure_particle_cap(sc, n);
    if (n) {
        SPH_CK(cudaMemcpyAsync(pos_.p + sc.p_off, hp.data(), (size_t)n * 16, cudaMemcpyHostToDevice, st_));
        SPH_CK(cudaMemcpyAsync(vel_.p + sc.p_off, hv.data(), (size_t)n * 16, cudaMemcpyHostToDevice, st_));
        SPH_CK(cudaMemcpyAsync(nbid_.p + sc.p_off, hn.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st_));
        SPH_CK(cudaMemsetAsync(dyn_.p + sc.p_off, 0, (size_t)n * 16, st_));
    }
    SPH_CK(cudaStreamSynchronize(st_));
    if (sc.n != n) work_dirty_ = true;
    sc.n = n;
    upload_scene(id);
    set_steps(id, steps);
}

void System::load_heightfield_u8(int id, const unsigned char* map512, float metres_per_level) {
    if (!map512) throw Error(SPH_ERR_INVALID, "null heightfield");
    constexpr int kSide = 512;
    std::vector<float> h((size_t)kSide * kSide);
    for (int x = 0; x < kSide; ++x)
        for (int z = 0; z < kSide; ++z) h[(size_t)z * kSide + x] = (float)map512[(size_t)kSide * x + z] * metres_per_level;
    set_terrain(id, kSide, kSide, h.data());
}

}  // namespace sph
