// Seeded fBm value-noise heightmaps (the repository's own generator; the
// reference loads an 8-bit PNG instead, Erosion/main.cpp:88-103).
//
// Specification:
//   lattice value v(o, i, j) = (SplitMix64(s_o ^ i*A ^ j*B) >> 40) / 2^24,
//     s_o = SplitMix64(seed + o), A = 0x632BE59BD9B4E019, B = 0x8CB92BA72F3D8DD7;
//   noise(x, z): smoothstep-weighted bilinear blend of the four lattice values;
//   vertex (ix, iz) samples u = ix/(w-1), v = iz/(d-1) at frequency 4 * lac^o;
//   ridged variant per octave: (1 - |2n - 1|)^2;
//   height = amplitude * sum_o gain^o n_o / sum_o gain^o, in double, rounded once
//   to float; the carved variant (kind 2) is amplitude * (1 - ridged sum /
//   norm): the ridges become sharp valleys cut into a plateau.
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace sph {

namespace {

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

double lattice_value(uint64_t oseed, long long i, long long j) {
    const uint64_t h =
        splitmix64(oseed ^ ((uint64_t)i * 0x632BE59BD9B4E019ULL) ^ ((uint64_t)j * 0x8CB92BA72F3D8DD7ULL));
    return (double)(h >> 40) * (1.0 / 16777216.0);
}

double noise2(uint64_t oseed, double x, double z) {
    const double fx = std::floor(x), fz = std::floor(z);
    const long long i = (long long)fx, j = (long long)fz;
    const double tx = x - fx, tz = z - fz;
    const double sx = tx * tx * (3.0 - 2.0 * tx);
    const double sz = tz * tz * (3.0 - 2.0 * tz);
    const double v00 = lattice_value(oseed, i, j), v10 = lattice_value(oseed, i + 1, j);
    const double v01 = lattice_value(oseed, i, j + 1), v11 = lattice_value(oseed, i + 1, j + 1);
    const double a = v00 + sx * (v10 - v00);
    const double b = v01 + sx * (v11 - v01);
    return a + sz * (b - a);
}

}  // namespace

void fbm_heights(uint64_t seed, int w, int d, int octaves, float amplitude, float lacunarity, float gain, int kind,
                 float* out, int max_threads) {
    std::vector<uint64_t> oseed(octaves > 0 ? octaves : 1);
    double norm = 0.0, amp = 1.0;
    for (int o = 0; o < octaves; ++o) {
        oseed[o] = splitmix64(seed + (uint64_t)o);
        norm += amp;
        amp *= (double)gain;
    }
    auto rows = [&](int z0, int z1) {
        for (int iz = z0; iz < z1; ++iz)
            for (int ix = 0; ix < w; ++ix) {
                const double u = (w > 1) ? (double)ix / (double)(w - 1) : 0.0;
                const double v = (d > 1) ? (double)iz / (double)(d - 1) : 0.0;
                double freq = 4.0, a = 1.0, sum = 0.0;
                for (int o = 0; o < octaves; ++o) {
                    double n = noise2(oseed[o], u * freq, v * freq);
                    if (kind != 0) {
                        const double r = 1.0 - std::fabs(2.0 * n - 1.0);
                        n = r * r;
                    }
                    sum += a * n;
                    a *= (double)gain;
                    freq *= (double)lacunarity;
                }
                const double f = kind == 2 ? 1.0 - sum / norm : sum / norm;
                out[(size_t)iz * (size_t)w + (size_t)ix] = (float)((double)amplitude * f);
            }
    };
    const int64_t work = (int64_t)w * d * (octaves > 0 ? octaves : 1);
    unsigned nt = std::thread::hardware_concurrency();
    if (nt == 0) nt = 1;
    if (max_threads > 0 && nt > (unsigned)max_threads) nt = (unsigned)max_threads;
    if (work < (1 << 20) || nt == 1) {
        rows(0, d);
        return;
    }
    if (nt > 32) nt = 32;
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t) {
        const int z0 = (int)((int64_t)d * t / nt), z1 = (int)((int64_t)d * (t + 1) / nt);
        th.emplace_back(rows, z0, z1);
    }
    for (auto& x : th) x.join();
}

}  // namespace sph
