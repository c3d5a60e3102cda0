/* Test infrastructure only: the oracle.  See sph_oracle.h for what it covers
 * and who may load it.  Compile with -ffp-contract=off. */
#include "sph_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- the step, in FP32 (reference order) and FP64 ------------------------ */
#define REAL float
#define SQRT sqrtf
#define POW powf
#define POW2(x) powf((x), 2.0f)
#define POW3(x) powf((x), 3.0f)
#define RINT rintf
#define FN(x) f32_##x
#include "sph_oracle_step.inc"
#undef POW2
#undef POW3
#undef FN

/* FP32 with correctly rounded small powers instead of libm powf: x^2 = x*x
 * (one rounding) and x^3 from exact TwoProduct terms (x*x = p + e and
 * p*x = c + f exactly via fmaf; Ogita, Rump and Oishi 2005), c + (f + e*x).
 * glibc's powf is within 0.82 ulp but not always correctly rounded, so this
 * variant isolates the reference's arithmetic from its libm. */
static inline float cube_cr(float x) {
    float p = x * x;
    float e = fmaf(x, x, -p);
    float c = p * x;
    float f = fmaf(p, x, -c);
    float t = fmaf(e, x, f);
    return c + t;
}
#define POW2(x) ((x) * (x))
#define POW3(x) cube_cr(x)
#define FN(x) f32x_##x
#include "sph_oracle_step.inc"
#undef REAL
#undef SQRT
#undef POW
#undef POW2
#undef POW3
#undef RINT
#undef FN

#define REAL double
#define SQRT sqrt
#define POW pow
#define POW2(x) ((x) * (x))
#define POW3(x) ((x) * (x) * (x))
#define RINT rint
#define FN(x) f64_##x
#include "sph_oracle_step.inc"
#undef REAL
#undef SQRT
#undef POW
#undef POW2
#undef POW3
#undef RINT
#undef FN

static void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

void oracle_run_f32(const oracle_params* p, int n, float* pos, float* vel, int* nbid, int32_t* sed,
                    const float* base, int64_t* delta, float* rec, int nsteps, int nthreads) {
    set_threads(nthreads);
    f32_run(p, n, pos, vel, nbid, sed, base, delta, rec, nsteps);
}

void oracle_run_f32x(const oracle_params* p, int n, float* pos, float* vel, int* nbid, int32_t* sed,
                     const float* base, int64_t* delta, float* rec, int nsteps, int nthreads) {
    set_threads(nthreads);
    f32x_run(p, n, pos, vel, nbid, sed, base, delta, rec, nsteps);
}

void oracle_run_f64(const oracle_params* p, int n, double* pos, double* vel, int* nbid, int32_t* sed,
                    const float* base, int64_t* delta, double* rec, int nsteps, int nthreads) {
    set_threads(nthreads);
    f64_run(p, n, pos, vel, nbid, sed, base, delta, rec, nsteps);
}

int oracle_sample_f32(const oracle_params* p, int n, const float* pos, const float* vel, const int32_t* sed,
                      const float* base, const int64_t* delta, int m, const int* ids, float* rec, float* pos_out,
                      float* vel_out, int* nbid_inout, int32_t* sed_out, int32_t* q_out, int* qv_out,
                      int nthreads) {
    set_threads(nthreads);
    return f32_sample(p, n, pos, vel, sed, base, delta, m, ids, rec, pos_out, vel_out, nbid_inout, sed_out, q_out,
                      qv_out);
}

int oracle_sample_f32x(const oracle_params* p, int n, const float* pos, const float* vel, const int32_t* sed,
                       const float* base, const int64_t* delta, int m, const int* ids, float* rec, float* pos_out,
                       float* vel_out, int* nbid_inout, int32_t* sed_out, int32_t* q_out, int* qv_out,
                       int nthreads) {
    set_threads(nthreads);
    return f32x_sample(p, n, pos, vel, sed, base, delta, m, ids, rec, pos_out, vel_out, nbid_inout, sed_out, q_out,
                       qv_out);
}

int oracle_sample_f64(const oracle_params* p, int n, const double* pos, const double* vel, const int32_t* sed,
                      const float* base, const int64_t* delta, int m, const int* ids, double* rec, double* pos_out,
                      double* vel_out, int* nbid_inout, int32_t* sed_out, int32_t* q_out, int* qv_out,
                      int nthreads) {
    set_threads(nthreads);
    return f64_sample(p, n, pos, vel, sed, base, delta, m, ids, rec, pos_out, vel_out, nbid_inout, sed_out, q_out,
                      qv_out);
}

/* ---- CPU-baseline timing sample ------------------------------------------ */
double oracle_time_sample(const oracle_params* p, int n, const float* pos, const float* vel, int i0, int m,
                          int nthreads) {
    f32_kconst kc = f32_make_kconst(p->h);
    float h = kc.h, mass = p->mass, p0 = p->p0, k = p->k;
    float* dens = (float*)malloc(sizeof(float) * (size_t)n);
    float* pres = (float*)malloc(sizeof(float) * (size_t)n);
    double acc_sum = 0.0;
    int i;
    set_threads(nthreads);
    for (i = 0; i < n; i++) {
        dens[i] = p0;
        pres[i] = 0.0f;
    }
#pragma omp parallel for schedule(static)
    for (i = i0; i < i0 + m; i++) {
        f32_v3 xi = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        float density = 0;
        int j;
        for (j = 0; j < n; j++) {
            f32_v3 xj = {pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]};
            f32_v3 r = f32_sub(xi, xj);
            float distance = f32_length(r);
            if (distance <= h) density += mass * f32_kern(&kc, f32_length(r));
        }
        dens[i] = density;
        pres[i] = k * (density - p0);
    }
#pragma omp parallel for schedule(static) reduction(+ : acc_sum)
    for (i = i0; i < i0 + m; i++) {
        f32_v3 xi = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        f32_v3 vi = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
        f32_v3 fp = {0, 0, 0}, fv = {0, 0, 0}, nn = {0, 0, 0};
        float ai = pres[i] / (dens[i] * dens[i]);
        float cfl = 0;
        int j;
        for (j = 0; j < n; j++) {
            f32_v3 xj = {pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]};
            f32_v3 r = f32_sub(xi, xj);
            float distance = f32_length(r);
            if (distance <= h && i != j) {
                float inv = 1.0f / sqrtf(f32_dot(r, r));
                float pw2 = powf(h - distance, 2.0f);
                float coef = (ai + pres[j] / (dens[j] * dens[j])) * mass;
                float b = mass / dens[j];
                float lv = kc.c_spiky * (h - distance);
                float pw = powf(kc.hh - distance * distance, 2.0f);
                fp.x += coef * (-(((r.x * inv) * kc.c_spiky) * pw2));
                fp.y += coef * (-(((r.y * inv) * kc.c_spiky) * pw2));
                fp.z += coef * (-(((r.z * inv) * kc.c_spiky) * pw2));
                fv.x += ((vel[3 * j] - vi.x) * b) * lv;
                fv.y += ((vel[3 * j + 1] - vi.y) * b) * lv;
                fv.z += ((vel[3 * j + 2] - vi.z) * b) * lv;
                nn.x += b * (-((r.x * kc.c_grad) * pw));
                nn.y += b * (-((r.y * kc.c_grad) * pw));
                nn.z += b * (-((r.z * kc.c_grad) * pw));
            }
        }
        for (j = 0; j < n; j++) {
            f32_v3 xj = {pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]};
            f32_v3 r = f32_sub(xi, xj);
            float distance = f32_length(r);
            if (distance <= h) {
                float len = f32_length(r);
                float ld = ((-kc.c_grad) * (kc.hh - len * len)) * (((3.0f * h) * h) - ((7.0f * len) * len));
                cfl += (mass / dens[j]) * ld;
            }
        }
        acc_sum += (double)(fp.x + fp.y + fp.z + fv.x + fv.y + fv.z + cfl * (nn.x + nn.y + nn.z));
    }
    free(dens);
    free(pres);
    return acc_sum;
}

void oracle_neighbour_counts(int n, const float* pos, float h, int* counts, int nthreads) {
    int i;
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (i = 0; i < n; i++) {
        f32_v3 xi = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        int c = 0, j;
        for (j = 0; j < n; j++) {
            f32_v3 xj = {pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]};
            if (f32_length(f32_sub(xi, xj)) <= h && i != j) c++;
        }
        counts[i] = c;
    }
}

/* ---- uniform grid: Morton-row keys and stable counting sort --------------- */

/* Cell edge along y and z = h * cell_mult * (1 + 2^-12); along x the same
 * over xsub = 2 when the reach ceil(1/cell_mult) is 1, else over 1.  The
 * small slack guarantees that two particles within h never land more than
 * the reach apart along y and z (reach * xsub along x) after FP32 rounding
 * of the key arithmetic. */
void oracle_grid_make(const oracle_params* p, float cell_mult, oracle_grid* g) {
    int a;
    int dims[3];
    int reach = (int)ceil(1.0 / (double)cell_mult - 1e-9);
    int xsub = reach == 1 ? 2 : 1;
    g->cell = (p->h * cell_mult) * 1.000244140625f;
    g->inv_cell = 1.0f / g->cell;
    g->inv_cell_x = g->inv_cell * (float)xsub;
    for (a = 0; a < 3; a++) {
        float ext = p->box_l[a] + p->box_l[a];
        float edge = a == 0 ? g->cell / (float)xsub : g->cell;
        int nd = (int)ceil((double)ext / (double)edge);
        if (nd < 1) nd = 1;
        dims[a] = nd;
        g->lo[a] = p->box_c[a] - p->box_l[a];
    }
    g->nx = dims[0];
    g->ny = dims[1];
    g->nz = dims[2];
    g->nkeys = g->nx * g->ny * g->nz + 1;
}

static int cell_coord(float x, float lo, float inv, int n) {
    float t = (x - lo) * inv;
    if (!(t > 0.0f)) t = 0.0f; /* also maps NaN to 0 */
    if (t > (float)(n - 1)) t = (float)(n - 1);
    return (int)t;
}

static int bits_for(int n) {
    int b = 0;
    while ((1 << b) < n) b++;
    return b;
}

/* (y, z) Morton code: bit b of y, then bit b of z, while each still has bits */
static uint32_t yz_morton(int cy, int cz, int by, int bz) {
    uint32_t m = 0;
    int b, o = 0;
    int top = by > bz ? by : bz;
    for (b = 0; b < top; b++) {
        if (b < by) m |= (uint32_t)((cy >> b) & 1) << o++;
        if (b < bz) m |= (uint32_t)((cz >> b) & 1) << o++;
    }
    return m;
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}

/* Row numbers: the ny * nz cell rows in (y, z) Morton order, numbered
 * densely; rank[z * ny + y] = the number of row (y, z).  The key of a cell is
 * rank * nx + x. */
static uint32_t* row_ranks(const oracle_grid* g) {
    size_t nr = (size_t)g->ny * g->nz, r;
    int y, z, by = bits_for(g->ny), bz = bits_for(g->nz);
    uint64_t* rows = (uint64_t*)malloc(nr * sizeof(uint64_t));
    uint32_t* rank = (uint32_t*)malloc(nr * sizeof(uint32_t));
    for (z = 0; z < g->nz; z++)
        for (y = 0; y < g->ny; y++)
            rows[(size_t)z * g->ny + y] = ((uint64_t)yz_morton(y, z, by, bz) << 32) | (uint64_t)((size_t)z * g->ny + y);
    qsort(rows, nr, sizeof(uint64_t), cmp_u64);
    for (r = 0; r < nr; r++) rank[rows[r] & 0xffffffffu] = (uint32_t)r;
    free(rows);
    return rank;
}

void oracle_cell_keys(const oracle_grid* g, int n, const float* pos, uint32_t* keys) {
    uint32_t* rank = row_ranks(g);
    int i;
    for (i = 0; i < n; i++) {
        int cx = cell_coord(pos[3 * i], g->lo[0], g->inv_cell_x, g->nx);
        int cy = cell_coord(pos[3 * i + 1], g->lo[1], g->inv_cell, g->ny);
        int cz = cell_coord(pos[3 * i + 2], g->lo[2], g->inv_cell, g->nz);
        keys[i] = rank[(size_t)cz * g->ny + cy] * (uint32_t)g->nx + (uint32_t)cx;
    }
    free(rank);
}

void oracle_stable_sort(int n, const uint32_t* keys, int nkeys, int* perm) {
    int* off = (int*)calloc((size_t)nkeys + 1, sizeof(int));
    int i, k;
    for (i = 0; i < n; i++) off[keys[i] + 1]++;
    for (k = 0; k < nkeys; k++) off[k + 1] += off[k];
    for (i = 0; i < n; i++) perm[off[keys[i]]++] = i;
    free(off);
}

/* ---- seeded fBm value noise ------------------------------------------------ */
static uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

/* lattice value in [0, 1): 24 high bits of a SplitMix64 hash of the octave
 * seed and the two lattice coordinates */
static double lattice(uint64_t oseed, long long i, long long j) {
    uint64_t hsh = splitmix64(oseed ^ ((uint64_t)i * 0x632BE59BD9B4E019ULL) ^ ((uint64_t)j * 0x8CB92BA72F3D8DD7ULL));
    return (double)(hsh >> 40) * (1.0 / 16777216.0);
}

static double value_noise(uint64_t oseed, double x, double z) {
    double fx = floor(x), fz = floor(z);
    long long i = (long long)fx, j = (long long)fz;
    double tx = x - fx, tz = z - fz;
    double sx = tx * tx * (3.0 - 2.0 * tx);
    double sz = tz * tz * (3.0 - 2.0 * tz);
    double v00 = lattice(oseed, i, j), v10 = lattice(oseed, i + 1, j);
    double v01 = lattice(oseed, i, j + 1), v11 = lattice(oseed, i + 1, j + 1);
    double a = v00 + sx * (v10 - v00);
    double b = v01 + sx * (v11 - v01);
    return a + sz * (b - a);
}

void oracle_fbm(uint64_t seed, int w, int d, int octaves, float amplitude, float lacunarity, float gain,
                int kind, float* out) {
    int ix, iz, o;
    double norm = 0.0, amp = 1.0;
    for (o = 0; o < octaves; o++) {
        norm += amp;
        amp *= (double)gain;
    }
    for (iz = 0; iz < d; iz++) {
        for (ix = 0; ix < w; ix++) {
            double u = (w > 1) ? (double)ix / (double)(w - 1) : 0.0;
            double v = (d > 1) ? (double)iz / (double)(d - 1) : 0.0;
            double freq = 4.0, a = 1.0, sum = 0.0;
            for (o = 0; o < octaves; o++) {
                uint64_t oseed = splitmix64(seed + (uint64_t)o);
                double nv = value_noise(oseed, u * freq, v * freq);
                if (kind != 0) {
                    double r = 1.0 - fabs(2.0 * nv - 1.0);
                    nv = r * r;
                }
                sum += a * nv;
                a *= (double)gain;
                freq *= (double)lacunarity;
            }
            out[(size_t)iz * (size_t)w + (size_t)ix] =
                (float)((double)amplitude * (kind == 2 ? 1.0 - sum / norm : sum / norm));
        }
    }
}

/* ---- reference lattice (Initialize / AddParticles) ------------------------ */
int oracle_lattice(int n, const float* origin, float* pos_out, int cap) {
    int i, j, k, c = 0;
    double cn = cbrt((double)n);
    for (i = 0; i < cn; i++)
        for (j = 0; j < cn; j++)
            for (k = 0; k < cn; k++) {
                float x = (float)(-0.2 + i * 0.025);
                float y = (float)(-0.05 + j * 0.025);
                float z = (float)(-0.15 + k * 0.025);
                if (c < cap) {
                    pos_out[3 * c] = x + origin[0];
                    pos_out[3 * c + 1] = y + origin[1];
                    pos_out[3 * c + 2] = z + origin[2];
                }
                c++;
            }
    return c;
}

/* ---- Grid::UpdateGrid surface mesh (grid.h:118-176) ------------------------ */
static int hmap(const unsigned char* map, int x, int y) { return map[512 * x + y]; }

int oracle_mesh(const unsigned char* map, int dimx, int dimy, int dimz, float* verts, unsigned* idx,
                int idx_cap) {
    int x, z, c = 0, ni = 0;
    for (z = 0; z < dimz; z++)
        for (x = 0; x < dimx; x++) {
            int y = hmap(map, x, z);
            float u[3] = {0, 0, 0}, dn[3] = {0, 0, 0}, r[3] = {0, 0, 0}, l[3] = {0, 0, 0};
            float nrm[3], cr[3], len2, inv;
            int a;
            if (dimy <= y) y = dimy - 1;
            verts[c++] = (float)x;
            verts[c++] = (float)y;
            verts[c++] = (float)z;
            if (x - 1 >= 0) {
                l[0] = (float)(x - (x - 1));
                l[1] = (float)(y - hmap(map, x - 1, z));
                l[2] = 0.0f;
            }
            if (x + 1 < dimx) {
                r[0] = (float)((x + 1) - x);
                r[1] = (float)(hmap(map, x + 1, z) - y);
                r[2] = 0.0f;
            }
            if (z - 1 >= 0) {
                u[0] = 0.0f;
                u[1] = (float)(y - hmap(map, x, z - 1));
                u[2] = (float)(z - (z - 1));
            }
            /* the reference compares z + 1 against m_Dim.y here (grid.h:167) */
            if (z + 1 < dimy) {
                dn[0] = 0.0f;
                dn[1] = (float)(hmap(map, x, z + 1) - y);
                dn[2] = (float)((z + 1) - z);
            }
            /* cross(u,l) + cross(u,r) + cross(d,l) + cross(d,r), then normalize */
            {
                const float* A[4] = {u, u, dn, dn};
                const float* B[4] = {l, r, l, r};
                int t;
                float s[3] = {0, 0, 0};
                for (t = 0; t < 4; t++) {
                    const float* p = A[t];
                    const float* q = B[t];
                    cr[0] = p[1] * q[2] - q[1] * p[2];
                    cr[1] = p[2] * q[0] - q[2] * p[0];
                    cr[2] = p[0] * q[1] - q[0] * p[1];
                    if (t == 0) {
                        s[0] = cr[0];
                        s[1] = cr[1];
                        s[2] = cr[2];
                    } else {
                        s[0] = s[0] + cr[0];
                        s[1] = s[1] + cr[1];
                        s[2] = s[2] + cr[2];
                    }
                }
                len2 = (s[0] * s[0] + s[1] * s[1]) + s[2] * s[2];
                inv = 1.0f / sqrtf(len2);
                for (a = 0; a < 3; a++) nrm[a] = s[a] * inv;
            }
            verts[c++] = nrm[0];
            verts[c++] = nrm[1];
            verts[c++] = nrm[2];
        }
    /* genIndices (grid.h:118-136) */
    {
        int i, j;
        for (z = 0, j = dimz - 1; z < dimz && j >= 0; z++, j--)
            for (x = 0, i = dimx - 1; x < dimx && i >= 0; x++, i--) {
                if (x + 1 < dimx && z + 1 < dimz) {
                    if (ni + 3 <= idx_cap) {
                        idx[ni] = (unsigned)(z * dimx + x);
                        idx[ni + 1] = (unsigned)(z * dimx + (x + 1));
                        idx[ni + 2] = (unsigned)((z + 1) * dimx + x);
                    }
                    ni += 3;
                }
                if (j - 1 >= 0 && i - 1 >= 0) {
                    if (ni + 3 <= idx_cap) {
                        idx[ni] = (unsigned)(j * dimx + i);
                        idx[ni + 1] = (unsigned)(j * dimx + (i - 1));
                        idx[ni + 2] = (unsigned)((j - 1) * dimx + i);
                    }
                    ni += 3;
                }
            }
    }
    return ni;
}
