"""Seeded synthetic scenes of the benchmark configurations.

No public dataset exists for this path; every scene is generated from a
stated seed.  Sizes, layouts and constants:

* plain_small (16,384 particles): 32 x 16 x 32 dam-break block at spacing
  h/2 = 0.02 in a unit box (half extent 0.5) over a 128 x 128 value-noise
  fBm heightmap (4 octaves, amplitude 0.2, lacunarity 2, gain 0.5, seed 0).
* plain_1m (1,048,576 particles): a 170 x 31 x 200 block at spacing 0.02,
  truncated to the first 2^20 particles in y-slowest order, in a 4 x 1 x 4
  box over a 1024 x 1024 fBm heightmap (6 octaves, amplitude 0.3, seed 0).

Both blocks start one spacing above the highest possible terrain point, at
rest, with zero sediment.  Physical constants: h = 0.04, rest density 1000,
mass = 1000 * 0.02^3, gas stiffness 3, viscosity 0.1, surface tension 0.0728
(the reference's default), dt = 1e-3, g = (0, -9.81, 0); erosion capacity
0.01 per m/s, pickup 5/s, deposition 2/s, contact layer h.
"""
from __future__ import annotations

import numpy as np

H = 0.04
SPACING = H / 2
PHYS = dict(smoothing_radius=H, rest_density=1000.0, mass=1000.0 * SPACING ** 3, gas_stiffness=3.0,
            viscosity=0.1, surface_tension=0.0728, dt=1e-3, gravity=(0.0, -9.81, 0.0), restitution=0.5,
            erosion=1, k_capacity=0.01, k_pickup=5.0, k_deposit=2.0, erosion_layer=H)


def lattice_block(nx, ny, nz, spacing, origin, limit=None) -> np.ndarray:
    """Cubic lattice, x fastest, then z, then y (y-slowest), optionally
    truncated to the first `limit` points."""
    y, z, x = np.meshgrid(np.arange(ny), np.arange(nz), np.arange(nx), indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.float64) * spacing
    pts += np.asarray(origin, np.float64)
    if limit is not None:
        pts = pts[:limit]
    return pts.astype(np.float32)


def plain_small(erosion=True, terrain=True):
    box_half = (0.5, 0.5, 0.5)
    amp = 0.2
    lo = -0.5 + SPACING / 2
    origin = (lo, -0.5 + amp + SPACING, lo)
    pos = lattice_block(32, 16, 32, SPACING, origin)
    prm = dict(PHYS, box_half=box_half, erosion=1 if erosion else 0)
    spec = dict(name="plain_small", params=prm, pos=pos, n=len(pos))
    if terrain:
        spec["terrain"] = dict(w=128, d=128, seed=0, octaves=4, amplitude=amp, lacunarity=2.0, gain=0.5, kind=0)
    return spec


def plain_1m(erosion=True):
    box_half = (2.0, 0.5, 2.0)
    amp = 0.3
    lo = -2.0 + SPACING / 2
    origin = (lo, -0.5 + amp + SPACING, lo)
    pos = lattice_block(170, 31, 200, SPACING, origin, limit=1 << 20)
    prm = dict(PHYS, box_half=box_half, erosion=1 if erosion else 0)
    return dict(name="plain_1m", params=prm, pos=pos, n=len(pos),
                terrain=dict(w=1024, d=1024, seed=0, octaves=6, amplitude=amp, lacunarity=2.0, gain=0.5, kind=0))


def scaled_block(n, box_half=(0.5, 0.5, 0.5), amp=0.2):
    """A dam-break block of about n particles in the corner of the box:
    footprint up to 70% of x and all of z, as many layers as needed."""
    nz = max(1, min(int(2 * box_half[2] / SPACING) - 1, int(round(np.sqrt(n)))))
    nx = max(1, min(int(0.7 * 2 * box_half[0] / SPACING), int(np.ceil(n / nz))))
    ny = int(np.ceil(n / (nx * nz)))
    lo = (-box_half[0] + SPACING / 2, -box_half[1] + amp + SPACING, -box_half[2] + SPACING / 2)
    return lattice_block(nx, ny, nz, SPACING, lo, limit=n)


def skew_rain(n=8388608, seed=5, terrain_side=None):
    """Skewed-occupancy stress: n particles released as rainfall (x, z uniform
    over the box floor, y uniform in the top 10% of the box height) over a
    terrain_side^2 carved-valley terrain (inverted ridged fBm, 6 octaves,
    amplitude 0.5), at rest.  The box (16 x 2 x 16 m at n = 8,388,608, its
    floor scaled with n otherwise) makes the rain layer's mean density about
    1.3x the rest density; the rain then pools in the valleys into very
    uneven cell occupancy.  The terrain keeps 4096 vertices per 16 m."""
    f = float(np.sqrt(n / 8388608.0))
    box_half = (8.0 * f, 1.0, 8.0 * f)
    if terrain_side is None:
        terrain_side = max(64, int(round(4096 * f)))
    rng = np.random.default_rng(seed)
    pos = np.empty((n, 3), np.float32)
    pos[:, 0] = rng.uniform(-box_half[0] + SPACING / 2, box_half[0] - SPACING / 2, n)
    pos[:, 2] = rng.uniform(-box_half[2] + SPACING / 2, box_half[2] - SPACING / 2, n)
    top = box_half[1]
    pos[:, 1] = rng.uniform(top - 0.1 * 2 * box_half[1], top - SPACING / 2, n)
    prm = dict(PHYS, box_half=box_half)
    return dict(name="skew_rain", params=prm, pos=pos, n=n,
                terrain=dict(w=terrain_side, d=terrain_side, seed=seed, octaves=6, amplitude=0.5, lacunarity=2.0,
                             gain=0.5, kind=2))


def batched_requests(n_scenes=256, seed=1000, steps=0):
    """The batched form: n_scenes independent scenes, scene i seeded with
    seed + i; particle counts log-uniform in [2048, 131072]; heightmap side
    uniform in {64, 128, 256, 512}; block coverage and terrain amplitude are
    drawn by the library's recipe from each scene's seed."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(2048), np.log(131072), n_scenes)).astype(np.int64)
    side = rng.choice([64, 128, 256, 512], n_scenes)
    return [dict(seed=seed + i, particles=int(n[i]), terrain_side=int(side[i]), steps=steps)
            for i in range(n_scenes)]


def serving_trace(n_requests=10000, rate=200.0, seed=2000):
    """The request stream: Poisson arrivals at `rate` per second (exponential
    gaps), particle counts log-uniform in [4096, 262144], heightmap side
    uniform in {128, 256, 512}, step counts uniform in [100, 2000]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    n = np.exp(rng.uniform(np.log(4096), np.log(262144), n_requests)).astype(np.int64)
    side = rng.choice([128, 256, 512], n_requests)
    steps = rng.integers(100, 2001, n_requests)
    return [dict(seed=seed + i, particles=int(n[i]), terrain_side=int(side[i]), steps=int(steps[i]),
                 arrival_s=float(t[i])) for i in range(n_requests)]


def base_params(cell_mult=0.5, flags=0):
    """Physical constants shared by every seeded scene."""
    import sph_gb300 as S

    return S.default_params(**dict(PHYS, cell_mult=cell_mult, flags=flags))


def build_scene(system, spec, flags=0, capacity=0):
    """Create a scene of `spec` in a sph_gb300.System."""
    import sph_gb300 as S

    prm = S.default_params(**spec["params"], flags=flags)
    t = spec.get("terrain")
    sc = system.scene(prm, capacity=max(capacity, spec["n"]), terrain=(t["w"], t["d"]) if t else (0, 0))
    if t:
        sc.gen_terrain(t["seed"], t["octaves"], t["amplitude"], t["lacunarity"], t["gain"], t["kind"])
    sc.set_particles(spec["pos"])
    return sc
