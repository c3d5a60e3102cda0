// Allocation-free density pass: sph_density_static (include/sph_erosion.h).
//
// Some callers of this library cannot allocate device memory: a host
// application that owns every byte of the GPU through its own pool, a
// real-time loop that must not take cudaMalloc's implicit synchronisation, or
// a plugin running where allocation is forbidden.  This entry point computes
// the reference's pass 1 (density and pressure, Erosion/fluid_system.h:107-124)
// for a caller's particle buffer with the same sort and density kernels as a
// scene step, but all of its scratch lives in one file-scope device array of
// fixed size, so it calls no cudaMalloc, cudaFree or allocating library
// routine.
//
// The array is held by every GPU that loads the library, until the process
// exits.  All calls share it and it keeps the last call's contents; what must
// start at zero is cleared by each call.  Calls whose work overlaps on the GPU
// (different streams, or different host threads) race on the array and must
// be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sph_erosion.h"
#include "sph_engine.h"
#include "sph_kernels.h"

namespace sph {
namespace {

constexpr int kStaticTile = 256;
constexpr int kMaxTiles = SPH_STATIC_MAX_PARTICLES / kStaticTile;
constexpr int kMaxChunks = SPH_STATIC_MAX_KEYS / kChunk;

constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }

// Byte layout of the scratch array.
constexpr size_t kOffScene = 0;
constexpr size_t kOffSteps = align256(kOffScene + sizeof(SceneDev));
constexpr size_t kOffNwork = align256(kOffSteps + sizeof(int));
constexpr size_t kOffStatus = align256(kOffNwork + 4 * sizeof(int));
constexpr size_t kOffPtiles = align256(kOffStatus + sizeof(unsigned));
constexpr size_t kOffCtiles = align256(kOffPtiles + kMaxTiles * sizeof(Work));
constexpr size_t kOffTab = align256(kOffCtiles + kMaxChunks * sizeof(Work));
constexpr size_t kOffChunk = align256(kOffTab + SPH_STATIC_MAX_TABLE * sizeof(uint32_t));
constexpr size_t kN = SPH_STATIC_MAX_PARTICLES;
constexpr size_t kOffPos = align256(kOffChunk + kMaxChunks * sizeof(uint32_t));
constexpr size_t kOffVel = kOffPos + kN * 16;
constexpr size_t kOffSpos = kOffVel + kN * 16;
constexpr size_t kOffSvel = kOffSpos + kN * 16;
constexpr size_t kOffDyn = kOffSvel + kN * 16;
constexpr size_t kOffKey = kOffDyn + kN * 16;
constexpr size_t kOffSlot = kOffKey + kN * 4;
constexpr size_t kOffPerm = kOffSlot + kN * 4;
constexpr size_t kOffCounts = align256(kOffPerm + kN * 4);
constexpr size_t kOffOffsets = kOffCounts + (size_t)SPH_STATIC_MAX_KEYS * 4;
constexpr size_t kScratchBytes = align256(kOffOffsets + (size_t)SPH_STATIC_MAX_KEYS * 4);
static_assert(kScratchBytes == SPH_STATIC_SCRATCH_BYTES, "public scratch size out of date");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Device address of g_scratch per device, resolved once with that device
// current.  Host code must not use the symbol itself as an address.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {nullptr};

unsigned char* scratch_for_current_device() {
    int dev = -1;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) throw Error(SPH_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        check_cuda(cudaGetSymbolAddress(&p, g_scratch), "cudaGetSymbolAddress(g_scratch)");
        g_addr[dev] = static_cast<unsigned char*>(p);
    }
    return g_addr[dev];
}

__global__ void k_pack(const float* __restrict__ pos3, int n, float4* __restrict__ pos, float4* __restrict__ vel) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos[i] = make_float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], __int_as_float(i));
    vel[i] = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
}

__global__ void k_unpack(const float4* __restrict__ spos, const float4* __restrict__ dyn, int n,
                         float* __restrict__ density, float* __restrict__ pressure) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int id = __float_as_int(spos[p].w);
    if (id < 0 || id >= n) return;
    const float4 d = dyn[p];
    density[id] = d.x;
    if (pressure) pressure[id] = d.w;
}

}  // namespace
}  // namespace sph

extern "C" SPH_API int sph_density_static(const sph_params* p, int n, const float* pos3_dev, float* density_dev,
                                          float* pressure_dev, void* stream) {
    using namespace sph;
    try {
        if (!p || n < 0 || (n > 0 && (!pos3_dev || !density_dev)))
            throw Error(SPH_ERR_INVALID, "sph_density_static: null argument or negative count");
        if (n > SPH_STATIC_MAX_PARTICLES)
            throw Error(SPH_ERR_CAPACITY, "sph_density_static: " + std::to_string(n) + " particles exceed the fixed " +
                                              std::to_string(SPH_STATIC_MAX_PARTICLES) + "-particle scratch");
        validate_params(*p);  // the same checks as sph_scene_create
        Scene sc;
        sc.prm = *p;
        System::geometry(sc);
        if (sc.k_cap > SPH_STATIC_MAX_KEYS || sc.tab_len > SPH_STATIC_MAX_TABLE)
            throw Error(SPH_ERR_CAPACITY, "sph_density_static: the uniform grid has " + std::to_string(sc.k_cap) +
                                              " keys, more than the fixed " + std::to_string(SPH_STATIC_MAX_KEYS) +
                                              "-key scratch (shrink the box or raise cell_mult)");
        if (n == 0) return SPH_OK;
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        // the call ends by synchronising its stream, which a stream being
        // captured cannot do: refuse before touching it
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
            cudaGetLastError();
            throw Error(SPH_ERR_INVALID, "sph_density_static: the stream is being captured (the call synchronises it)");
        }
        unsigned char* base = scratch_for_current_device();

        sc.n = n;
        sc.p_cap = n;
        sc.p_off = 0;
        sc.k_off = 0;
        sc.c_off = 0;
        sc.tab_off = 0;
        sc.tw = sc.td = 0;
        sc.t_off = 0;
        sc.prm.flags &= ~(SPH_FLAG_ORDERED | SPH_FLAG_RECORD);
        System::fill_dev(sc);
        // host images of the small tables
        std::vector<Work> pt, ct;
        for (int t = 0; t * kStaticTile < n; ++t) pt.push_back({0, t * kStaticTile});
        for (int c = 0; c < sc.nchunks; ++c) ct.push_back({0, c});
        std::vector<uint32_t> tab(sc.tab_len);
        row_table(sc.ny, sc.nz, tab.data());
        const int steps = -1;
        const int nwork[4] = {(int)pt.size(), (int)ct.size(), 0, 0};
        check_cuda(cudaMemcpyAsync(base + kOffScene, &sc.dev, sizeof(SceneDev), cudaMemcpyHostToDevice, st), "copy");
        check_cuda(cudaMemcpyAsync(base + kOffSteps, &steps, sizeof steps, cudaMemcpyHostToDevice, st), "copy");
        check_cuda(cudaMemcpyAsync(base + kOffNwork, nwork, sizeof nwork, cudaMemcpyHostToDevice, st), "copy");
        check_cuda(cudaMemcpyAsync(base + kOffPtiles, pt.data(), pt.size() * sizeof(Work), cudaMemcpyHostToDevice, st),
                   "copy");
        check_cuda(cudaMemcpyAsync(base + kOffCtiles, ct.data(), ct.size() * sizeof(Work), cudaMemcpyHostToDevice, st),
                   "copy");
        check_cuda(cudaMemcpyAsync(base + kOffTab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, st), "copy");
        // what the sort expects to start at zero
        check_cuda(cudaMemsetAsync(base + kOffCounts, 0, (size_t)sc.k_cap * 4, st), "memset");
        check_cuda(cudaMemsetAsync(base + kOffChunk, 0, (size_t)sc.nchunks * 4, st), "memset");
        check_cuda(cudaMemsetAsync(base + kOffStatus, 0, sizeof(unsigned), st), "memset");

        DevArrays a;
        std::memset(&a, 0, sizeof a);
        a.scenes = reinterpret_cast<const SceneDev*>(base + kOffScene);
        a.steps_left = reinterpret_cast<int*>(base + kOffSteps);
        a.ptiles = reinterpret_cast<const Work*>(base + kOffPtiles);
        a.n_ptiles = reinterpret_cast<const int*>(base + kOffNwork);
        a.ctiles = reinterpret_cast<const Work*>(base + kOffCtiles);
        a.n_ctiles = reinterpret_cast<const int*>(base + kOffNwork) + 1;
        a.ttiles = nullptr;
        a.n_ttiles = reinterpret_cast<const int*>(base + kOffNwork) + 2;
        a.pos = reinterpret_cast<float4*>(base + kOffPos);
        a.vel = reinterpret_cast<float4*>(base + kOffVel);
        a.spos = reinterpret_cast<float4*>(base + kOffSpos);
        a.svel = reinterpret_cast<float4*>(base + kOffSvel);
        a.dyn = reinterpret_cast<float4*>(base + kOffDyn);
        a.key = reinterpret_cast<uint32_t*>(base + kOffKey);
        a.slot = reinterpret_cast<uint32_t*>(base + kOffSlot);
        a.perm = reinterpret_cast<uint32_t*>(base + kOffPerm);
        a.counts = reinterpret_cast<uint32_t*>(base + kOffCounts);
        a.offsets = reinterpret_cast<uint32_t*>(base + kOffOffsets);
        a.chunk_sum = reinterpret_cast<uint32_t*>(base + kOffChunk);
        a.tab = reinterpret_cast<const uint32_t*>(base + kOffTab);
        a.status = reinterpret_cast<unsigned*>(base + kOffStatus);
        LaunchShape s;
        s.tile = kStaticTile;
        s.grid_p = (int)pt.size();
        s.grid_c = (int)ct.size();
        s.grid_t = 0;
        s.variant = 0;
        s.grid_dyn = 0;
        s.fmap = nullptr;

        const int nb = (n + 255) / 256;
        k_pack<<<nb, 256, 0, st>>>(pos3_dev, n, a.pos, a.vel);
        launch_keys(a, s, st);
        launch_scan(a, s, st);
        launch_scatter(a, s, st);
        launch_reorder(a, s, st);
        launch_density(a, s, st);
        k_unpack<<<nb, 256, 0, st>>>(a.spos, a.dyn, n, density_dev, pressure_dev);
        check_cuda(cudaGetLastError(), "launch");
        unsigned status = 0;
        check_cuda(cudaMemcpyAsync(&status, base + kOffStatus, sizeof status, cudaMemcpyDeviceToHost, st), "copy");
        check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        if (status) throw Error(SPH_ERR_DEVICE, "sph_density_static: counting sort reported inconsistent counts");
        return SPH_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return SPH_ERR_INVALID;
    }
}
