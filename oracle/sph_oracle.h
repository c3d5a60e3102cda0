/* Test infrastructure only: the oracle for the SPH-erosion simulation step.
 *
 * A CPU restatement, in plain C, of the reference's FluidSystemSPH::Run
 * (Erosion/fluid_system.h:104-183) with its kernels (:410-453), integration
 * and box collision (:306-407), in two precisions:
 *   - FP32 in the reference's exact operation order (all-pairs, ascending j),
 *     which must agree bit for bit with the reference built headless;
 *   - FP64 with the same constants, used to state each field's rounding error.
 * It also restates the repository's own extensions, which have no reference
 * code: the heightfield terrain contact, the erosion exchange in int64 fixed
 * point, the cell keys and stable counting sort, and the seeded fBm terrain.
 *
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark load
 * this library, always as the checker; the product never does.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Scene parameters.  The reference case is box_c = 0, box_l = (len,len,len),
 * terrain and erosion off. */
typedef struct oracle_params {
    float g[3];
    float dt;
    float p0;          /* rest density */
    float mass;
    float visc;
    float surf_tens;
    float k;           /* gas stiffness */
    float cr;          /* restitution used by the terrain contact */
    float h;           /* smoothing radius */
    float box_c[3];    /* box centre */
    float box_l[3];    /* box half extents */
    /* terrain: vertex grid tw (along x) by td (along z) over the box floor */
    int terrain;       /* 0 = off */
    int tw, td;
    float height_unit; /* metres of height per sediment unit on one vertex */
    /* erosion */
    int erosion;       /* 0 = off */
    float k_capacity;  /* carried-volume fraction per (m/s) of speed */
    float k_pickup;    /* 1/s */
    float k_deposit;   /* 1/s */
    float layer;       /* contact layer thickness above the surface (m) */
} oracle_params;

/* One per-particle record, the fields of FluidParticle (fluid_system.h:49-64):
 * pos[3] vel[3] acc[3] density pressure fpress[3] fvisc[3] fgrav[3] fsurf[3]
 * normal[3] pad  -> 27 floats. */
#define ORACLE_REC 27

/* Advance nsteps.  pos/vel: 3n floats (in/out).  nbid: n ints (in/out,
 * NeighbId semantics).  sed: n int32 sediment units (in/out, may be null when
 * erosion is off).  base: tw*td float heights above the box floor; delta:
 * tw*td int64 units (in/out).  rec: n*ORACLE_REC floats of the last step
 * (may be null).  nthreads <= 0 means all. */
void oracle_run_f32(const oracle_params* p, int n, float* pos, float* vel, int* nbid, int32_t* sed,
                    const float* base, int64_t* delta, float* rec, int nsteps, int nthreads);
/* As oracle_run_f32 with correctly rounded x^2 and x^3 in place of powf. */
void oracle_run_f32x(const oracle_params* p, int n, float* pos, float* vel, int* nbid, int32_t* sed,
                     const float* base, int64_t* delta, float* rec, int nsteps, int nthreads);
void oracle_run_f64(const oracle_params* p, int n, double* pos, double* vel, int* nbid, int32_t* sed,
                    const float* base, int64_t* delta, double* rec, int nsteps, int nthreads);

/* One step of the particles ids[0..m) only, from the state of all n (pos,
 * vel: 3n; sed: n units, may be null; base/delta: the terrain).  Each
 * neighbour sum runs over the particle's in-range set in ascending index,
 * found through a uniform grid, which is term for term the all-pairs sum of
 * oracle_run_*: the results equal what oracle_run_* computes for those
 * particles.  Per sample: rec (ORACLE_REC floats), next pos and vel (3
 * each), NeighbId (nbid_inout: in = the state's, out = the step's), sediment,
 * units moved from the terrain (q) and their vertex (qv, -1 when none).  Any
 * output may be null.  Returns 0, or -1 if an in-range set exceeds 4096. */
int oracle_sample_f32(const oracle_params* p, int n, const float* pos, const float* vel, const int32_t* sed,
                      const float* base, const int64_t* delta, int m, const int* ids, float* rec, float* pos_out,
                      float* vel_out, int* nbid_inout, int32_t* sed_out, int32_t* q_out, int* qv_out,
                      int nthreads);
int oracle_sample_f32x(const oracle_params* p, int n, const float* pos, const float* vel, const int32_t* sed,
                       const float* base, const int64_t* delta, int m, const int* ids, float* rec, float* pos_out,
                       float* vel_out, int* nbid_inout, int32_t* sed_out, int32_t* q_out, int* qv_out,
                       int nthreads);
int oracle_sample_f64(const oracle_params* p, int n, const double* pos, const double* vel, const int32_t* sed,
                      const float* base, const int64_t* delta, int m, const int* ids, double* rec, double* pos_out,
                      double* vel_out, int* nbid_inout, int32_t* sed_out, int32_t* q_out, int* qv_out,
                      int nthreads);

/* Timing sample for the CPU baseline: the reference's three all-pairs passes
 * and the integration for particles [i0, i0+m) against all n particles
 * (densities of the other particles are taken as p0).  Writes nothing back. */
double oracle_time_sample(const oracle_params* p, int n, const float* pos, const float* vel, int i0, int m,
                          int nthreads);

/* Neighbour counts with the reference's test |x_i - x_j| <= h, j != i. */
void oracle_neighbour_counts(int n, const float* pos, float h, int* counts, int nthreads);

/* Uniform-grid restatement: cell dims, Morton-row keys and stable order. */
typedef struct oracle_grid {
    int nx, ny, nz;
    int nkeys;         /* nx * ny * nz, plus one sentinel key */
    float cell;        /* cell edge along y and z; along x cell / xsub (2 at reach 1, else 1) */
    float inv_cell;
    float lo[3];       /* grid origin (box minimum) */
    float inv_cell_x;  /* xsub * inv_cell */
} oracle_grid;
void oracle_grid_make(const oracle_params* p, float cell_mult, oracle_grid* g);
void oracle_cell_keys(const oracle_grid* g, int n, const float* pos, uint32_t* keys);
/* perm[r] = index of the r-th particle in (key, index) order. */
void oracle_stable_sort(int n, const uint32_t* keys, int nkeys, int* perm);

/* Seeded fBm value-noise heightmap (the repository's own generator):
 * kind 0 = value fBm, 1 = ridged fBm.  out: w*d floats, metres. */
void oracle_fbm(uint64_t seed, int w, int d, int octaves, float amplitude, float lacunarity, float gain,
                int kind, float* out);

/* Reference lattice: Initialize(n) / AddParticles(n) positions
 * (fluid_system.h:74-102, :232-251).  Returns the count written. */
int oracle_lattice(int n, const float* origin, float* pos_out, int cap);

/* Surface mesh of Grid::UpdateGrid (grid.h:138-176) for an 8-bit map of
 * side 512 (x-major): verts 6 floats per (x,z), indices per genIndices. */
int oracle_mesh(const unsigned char* map, int dimx, int dimy, int dimz, float* verts, unsigned* idx,
                int idx_cap);

#ifdef __cplusplus
}
#endif
#endif
