"""Shared helpers of the GPU parity tests: run a scene through the C ABI and
compare fields with a stated tolerance."""
import numpy as np

import sph_gb300 as S

# Reference defaults (Erosion/fluid_system.h:460-479) with the F-key dt.
REF = dict(gravity=(0.0, -9.82, 0.0), dt=0.01, rest_density=998.29, mass=0.02, viscosity=3.5,
           surface_tension=0.0728, gas_stiffness=3.0, restitution=0.5, smoothing_radius=0.0457,
           box_half=(0.2, 0.2, 0.2))
# The plain-small scene's constants (no terrain: the reference has none).
C1 = dict(gravity=(0.0, -9.81, 0.0), dt=1e-3, rest_density=1000.0, mass=float(np.float32(0.008)), viscosity=0.1,
          surface_tension=0.0728, gas_stiffness=3.0, restitution=0.5, smoothing_radius=0.04,
          box_half=(0.5, 0.5, 0.5))

FIELDS = {"pos": slice(0, 3), "vel": slice(3, 6), "acc": slice(6, 9), "density": slice(9, 10),
          "pressure": slice(10, 11), "fpress": slice(11, 14), "fvisc": slice(14, 17), "fgrav": slice(17, 20),
          "fsurf": slice(20, 23), "normal": slice(23, 26)}

# Parity tolerance of the FP32 fields against the reference (and the oracle):
# max |a - b| over a field <= RTOL * max |b| of that field.
RTOL = 1e-4


def run(params: dict, pos, steps, vel=None, flags=S.SPH_FLAG_RECORD, graph_steps=16, tile=256, cell_mult=1.0,
        variant=None):
    """Run `steps` (int or list of step counts) and return {steps: (rec, nbid)}."""
    with S.System(particle_capacity=max(len(pos), 1), graph_steps=graph_steps, tile=tile, variant=variant) as sysm:
        sc = sysm.scene(S.default_params(**params, flags=flags, cell_mult=cell_mult), capacity=len(pos))
        sc.set_particles(pos, vel)
        out = {}
        done = 0
        for s in ([steps] if isinstance(steps, int) else steps):
            sysm.step(s - done)
            done = s
            out[s] = sc.get_records()
        return out


def field_errors(a, b):
    """Normwise relative error of each record field."""
    res = {}
    for name, sl in FIELDS.items():
        x, y = a[:, sl].astype(np.float64), b[:, sl].astype(np.float64)
        scale = np.abs(y).max()
        res[name] = float(np.abs(x - y).max() / scale) if scale > 0 else float(np.abs(x - y).max())
    return res


def ulp_diff(a, b):
    a = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


def height_unit(prm: dict, terrain):
    """The product's terrain height per delta unit, FP32: (mass / rest_density)
    * 2^-30 over the area of one vertex cell of a (w, d) terrain."""
    tw, td = terrain
    bh = prm.get("box_half", (0.2, 0.2, 0.2))
    f32 = np.float32
    sx = f32(f32(f32(bh[0]) + f32(bh[0])) / f32(tw - 1))
    sz = f32(f32(f32(bh[2]) + f32(bh[2])) / f32(td - 1))
    return f32((float(f32(prm.get("mass", 0.02))) / float(f32(prm.get("rest_density", 998.29)))) * 2.0 ** -30
               / (float(sx) * float(sz)))


def oracle_params(O, prm: dict, terrain=None):
    """The oracle's parameter block for a product parameter dict (same FP32
    values); with terrain=(w, d) the height unit follows the product's rule:
    (mass / rest_density) * 2^-30 over the area of one vertex cell."""
    bh = prm.get("box_half", (0.2, 0.2, 0.2))
    kw = dict(g=prm.get("gravity", (0.0, -9.82, 0.0)), dt=prm.get("dt", 0.0), p0=prm.get("rest_density", 998.29),
              mass=prm.get("mass", 0.02), visc=prm.get("viscosity", 3.5), surf_tens=prm.get("surface_tension", 0.0728),
              k=prm.get("gas_stiffness", 3.0), cr=prm.get("restitution", 0.5), h=prm.get("smoothing_radius", 0.0457),
              box_c=prm.get("box_center", (0.0, 0.0, 0.0)), box_l=bh)
    if terrain is not None:
        tw, td = terrain
        hu = height_unit(prm, terrain)
        kw.update(terrain=(tw, td), height_unit=float(hu), erosion=bool(prm.get("erosion", 0)),
                  k_capacity=prm.get("k_capacity", 0.01), k_pickup=prm.get("k_pickup", 5.0),
                  k_deposit=prm.get("k_deposit", 2.0), layer=prm.get("erosion_layer", 0.0457))
    return O.make_params(**kw)


def run_terrain(params: dict, pos, heights, steps, vel=None, flags=S.SPH_FLAG_RECORD):
    """Run with a terrain; returns {steps: (rec, nbid, sed, heights, delta, diag)}."""
    d, w = heights.shape
    with S.System(particle_capacity=max(len(pos), 1)) as sysm:
        sc = sysm.scene(S.default_params(**params, flags=flags), capacity=len(pos), terrain=(w, d))
        sc.set_terrain(heights)
        sc.set_particles(pos, vel)
        out = {}
        done = 0
        for s in ([steps] if isinstance(steps, int) else steps):
            sysm.step(s - done)
            done = s
            rec, nb = sc.get_records()
            st = sc.get_particles()
            hg, dl = sc.get_terrain()
            out[s] = (rec, nb, st["sed"], hg, dl, sc.diag())
        return out
