"""Test infrastructure only: ctypes bindings for the oracle (liboracle.so) and,
where it was built, the reference harness (_ref/libsphref.so).

Only tests, the smoke check and the benchmark's CPU-baseline leg import this
module, and only as the checker.  The product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libsphref.so")
REC = 27  # floats per particle record (FluidParticle fields)

# record field slices (Erosion/fluid_system.h:49-64)
FIELDS = {
    "pos": slice(0, 3), "vel": slice(3, 6), "acc": slice(6, 9), "density": slice(9, 10),
    "pressure": slice(10, 11), "fpress": slice(11, 14), "fvisc": slice(14, 17),
    "fgrav": slice(17, 20), "fsurf": slice(20, 23), "normal": slice(23, 26),
}


class OracleParams(C.Structure):
    _fields_ = [
        ("g", C.c_float * 3), ("dt", C.c_float), ("p0", C.c_float), ("mass", C.c_float),
        ("visc", C.c_float), ("surf_tens", C.c_float), ("k", C.c_float), ("cr", C.c_float),
        ("h", C.c_float), ("box_c", C.c_float * 3), ("box_l", C.c_float * 3),
        ("terrain", C.c_int), ("tw", C.c_int), ("td", C.c_int), ("height_unit", C.c_float),
        ("erosion", C.c_int), ("k_capacity", C.c_float), ("k_pickup", C.c_float),
        ("k_deposit", C.c_float), ("layer", C.c_float),
    ]


class OracleGrid(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("nkeys", C.c_int), ("cell", C.c_float), ("inv_cell", C.c_float), ("lo", C.c_float * 3),
        ("inv_cell_x", C.c_float),
    ]


# Parameter defaults of the reference (Erosion/fluid_system.h:460-479).
REFERENCE_DEFAULTS = dict(g=(0.0, -9.82, 0.0), dt=0.0, p0=998.29, mass=0.02, visc=3.5, surf_tens=0.0728,
                          k=3.0, cr=0.5, h=0.0457, len=0.2)


def make_params(g=(0.0, -9.82, 0.0), dt=0.0, p0=998.29, mass=0.02, visc=3.5, surf_tens=0.0728, k=3.0,
                cr=0.5, h=0.0457, box_c=(0.0, 0.0, 0.0), box_l=(0.2, 0.2, 0.2), terrain=None,
                height_unit=0.0, erosion=False, k_capacity=0.0, k_pickup=0.0, k_deposit=0.0, layer=0.0,
                **_ignored) -> OracleParams:
    p = OracleParams()
    p.g[:] = [float(x) for x in g]
    p.dt, p.p0, p.mass, p.visc = dt, p0, mass, visc
    p.surf_tens, p.k, p.cr, p.h = surf_tens, k, cr, h
    p.box_c[:] = [float(x) for x in box_c]
    p.box_l[:] = [float(x) for x in box_l]
    if terrain is not None:
        p.terrain, p.tw, p.td = 1, int(terrain[0]), int(terrain[1])
    p.height_unit = height_unit
    p.erosion = 1 if erosion else 0
    p.k_capacity, p.k_pickup, p.k_deposit, p.layer = k_capacity, k_pickup, k_deposit, layer
    return p


def build(force: bool = False) -> None:
    """Compile liboracle.so (and the reference harness where its sources exist)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def build_ref(ref_root: str = "/root/reference") -> bool:
    if not os.path.isdir(ref_root):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={ref_root}"], check=True)
    return os.path.exists(REF_PATH)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        f32p, f64p, i32p, i64p = (np.ctypeslib.ndpointer(np.float32, flags="C"),
                                  np.ctypeslib.ndpointer(np.float64, flags="C"),
                                  np.ctypeslib.ndpointer(np.int32, flags="C"),
                                  np.ctypeslib.ndpointer(np.int64, flags="C"))
        L.oracle_run_f32.argtypes = [C.POINTER(OracleParams), C.c_int, f32p, f32p, i32p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.oracle_run_f32x.argtypes = L.oracle_run_f32.argtypes
        L.oracle_run_f64.argtypes = [C.POINTER(OracleParams), C.c_int, f64p, f64p, i32p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        for nm, fp in (("oracle_sample_f32", f32p), ("oracle_sample_f32x", f32p), ("oracle_sample_f64", f64p)):
            fn = getattr(L, nm)
            fn.argtypes = [C.POINTER(OracleParams), C.c_int, fp, fp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                           i32p, fp, fp, fp, i32p, i32p, i32p, i32p, C.c_int]
            fn.restype = C.c_int
        L.oracle_time_sample.argtypes = [C.POINTER(OracleParams), C.c_int, f32p, f32p, C.c_int, C.c_int,
                                         C.c_int]
        L.oracle_time_sample.restype = C.c_double
        L.oracle_neighbour_counts.argtypes = [C.c_int, f32p, C.c_float, i32p, C.c_int]
        L.oracle_grid_make.argtypes = [C.POINTER(OracleParams), C.c_float, C.POINTER(OracleGrid)]
        L.oracle_cell_keys.argtypes = [C.POINTER(OracleGrid), C.c_int, f32p,
                                       np.ctypeslib.ndpointer(np.uint32, flags="C")]
        L.oracle_stable_sort.argtypes = [C.c_int, np.ctypeslib.ndpointer(np.uint32, flags="C"), C.c_int, i32p]
        L.oracle_fbm.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                 C.c_int, f32p]
        L.oracle_lattice.argtypes = [C.c_int, f32p, f32p, C.c_int]
        L.oracle_lattice.restype = C.c_int
        L.oracle_mesh.argtypes = [np.ctypeslib.ndpointer(np.uint8, flags="C"), C.c_int, C.c_int, C.c_int,
                                  f32p, np.ctypeslib.ndpointer(np.uint32, flags="C"), C.c_int]
        L.oracle_mesh.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def run(params: OracleParams, pos, vel=None, nsteps=1, nbid=None, sed=None, base=None, delta=None,
        precision="f32", record=True, nthreads=0):
    """Advance a particle set nsteps with the oracle.  precision: "f32" (the
    reference's arithmetic, libm powf), "f32x" (FP32 with correctly rounded
    powers, the arithmetic of the kernels) or "f64".  Returns a dict with the
    new state, the last step's per-particle record and the terrain delta."""
    dt = np.float64 if precision == "f64" else np.float32
    n = len(pos)
    pos = np.ascontiguousarray(np.asarray(pos, dt).reshape(n, 3)).copy()
    vel = np.zeros((n, 3), dt) if vel is None else np.ascontiguousarray(np.asarray(vel, dt).reshape(n, 3)).copy()
    nbid = np.full(n, -1, np.int32) if nbid is None else np.ascontiguousarray(nbid, np.int32).copy()
    sed = np.zeros(n, np.int32) if sed is None else np.ascontiguousarray(sed, np.int32).copy()
    ntex = params.tw * params.td if params.terrain else 0
    base = np.zeros(max(ntex, 1), np.float32) if base is None else np.ascontiguousarray(base, np.float32).ravel()
    delta = (np.zeros(max(ntex, 1), np.int64) if delta is None
             else np.ascontiguousarray(delta, np.int64).ravel().copy())
    rec = np.zeros((n, REC), dt) if record else None
    fn = {"f32": lib().oracle_run_f32, "f32x": lib().oracle_run_f32x, "f64": lib().oracle_run_f64}[precision]
    fn(C.byref(params), n, pos, vel, nbid, _ptr(sed), _ptr(base), _ptr(delta), _ptr(rec), int(nsteps),
       int(nthreads))
    return dict(pos=pos, vel=vel, nbid=nbid, sed=sed, delta=delta, rec=rec)


def sample(params: OracleParams, pos, vel, ids, sed=None, base=None, delta=None, nbid=None, precision="f32",
           nthreads=0):
    """One step of the particles `ids` from the state of all of them: the
    values oracle_run computes for those particles, with each neighbour sum
    over the in-range set in ascending index (found through a grid, so large
    scenes are cheap).  Returns a dict with rec, pos, vel, nbid, sed, q and
    qv of the sample, in the order of `ids`."""
    dt = np.float64 if precision == "f64" else np.float32
    n = len(pos)
    pos = np.ascontiguousarray(np.asarray(pos, dt).reshape(n, 3))
    vel = np.ascontiguousarray(np.asarray(vel, dt).reshape(n, 3))
    ids = np.ascontiguousarray(ids, np.int32)
    m = len(ids)
    if m and (ids.min() < 0 or ids.max() >= n):
        raise ValueError("sample ids out of range")
    sed = None if sed is None else np.ascontiguousarray(sed, np.int32)
    ntex = params.tw * params.td if params.terrain else 0
    base = np.zeros(max(ntex, 1), np.float32) if base is None else np.ascontiguousarray(base, np.float32).ravel()
    delta = np.zeros(max(ntex, 1), np.int64) if delta is None else np.ascontiguousarray(delta, np.int64).ravel()
    if ntex and (base.size < ntex or delta.size < ntex):
        raise ValueError("terrain arrays smaller than tw * td")
    out = dict(rec=np.zeros((m, REC), dt), pos=np.zeros((m, 3), dt), vel=np.zeros((m, 3), dt),
               nbid=(np.full(m, -1, np.int32) if nbid is None else np.ascontiguousarray(nbid, np.int32)[ids].copy()),
               sed=np.zeros(m, np.int32), q=np.zeros(m, np.int32), qv=np.zeros(m, np.int32))
    fn = {"f32": lib().oracle_sample_f32, "f32x": lib().oracle_sample_f32x, "f64": lib().oracle_sample_f64}[precision]
    rc = fn(C.byref(params), n, pos, vel, _ptr(sed), _ptr(base), _ptr(delta), m, ids, out["rec"], out["pos"],
            out["vel"], out["nbid"], out["sed"], out["q"], out["qv"], int(nthreads))
    if rc != 0:
        raise RuntimeError("oracle sample: an in-range set exceeds 4096 particles")
    return out


def run_grid(params: OracleParams, pos, vel=None, nsteps=1, nbid=None, sed=None, base=None, delta=None,
             precision="f32", nthreads=0):
    """oracle.run's result (same arithmetic, same sums, bit for bit) for
    larger scenes: each step is oracle.sample over every particle, whose
    neighbour sums run over the in-range sets found through a grid instead
    of all pairs.  Returns the same dict as run (rec of the last step)."""
    dt = np.float64 if precision == "f64" else np.float32
    n = len(pos)
    pos = np.ascontiguousarray(np.asarray(pos, dt).reshape(n, 3)).copy()
    vel = np.zeros((n, 3), dt) if vel is None else np.ascontiguousarray(np.asarray(vel, dt).reshape(n, 3)).copy()
    nbid = np.full(n, -1, np.int32) if nbid is None else np.ascontiguousarray(nbid, np.int32).copy()
    sed = np.zeros(n, np.int32) if sed is None else np.ascontiguousarray(sed, np.int32).copy()
    ntex = params.tw * params.td if params.terrain else 0
    base = np.zeros(max(ntex, 1), np.float32) if base is None else np.ascontiguousarray(base, np.float32).ravel()
    delta = (np.zeros(max(ntex, 1), np.int64) if delta is None
             else np.ascontiguousarray(delta, np.int64).ravel().copy())
    ids = np.arange(n, dtype=np.int32)
    rec = None
    for _ in range(int(nsteps)):
        s = sample(params, pos, vel, ids, sed=sed, base=base, delta=delta, nbid=nbid, precision=precision,
                   nthreads=nthreads)
        pos, vel, nbid, rec = s["pos"], s["vel"], s["nbid"], s["rec"]
        if params.terrain and params.erosion:
            sed = s["sed"]
            m = s["qv"] >= 0
            np.subtract.at(delta, s["qv"][m], s["q"][m].astype(np.int64))
    return dict(pos=pos, vel=vel, nbid=nbid, sed=sed, delta=delta, rec=rec)


def neighbour_counts(pos, h, nthreads=0):
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    out = np.zeros(len(pos), np.int32)
    lib().oracle_neighbour_counts(len(pos), pos, float(h), out, int(nthreads))
    return out


def grid(params: OracleParams, cell_mult=1.0) -> OracleGrid:
    g = OracleGrid()
    lib().oracle_grid_make(C.byref(params), float(cell_mult), C.byref(g))
    return g


def cell_keys(g: OracleGrid, pos):
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    out = np.zeros(len(pos), np.uint32)
    lib().oracle_cell_keys(C.byref(g), len(pos), pos, out)
    return out


def stable_sort(keys, nkeys):
    keys = np.ascontiguousarray(keys, np.uint32)
    perm = np.zeros(len(keys), np.int32)
    lib().oracle_stable_sort(len(keys), keys, int(nkeys), perm)
    return perm


def fbm(seed, w, d, octaves, amplitude, lacunarity=2.0, gain=0.5, kind=0):
    out = np.zeros(w * d, np.float32)
    lib().oracle_fbm(int(seed), int(w), int(d), int(octaves), float(amplitude), float(lacunarity), float(gain),
                     int(kind), out)
    return out.reshape(d, w)


def lattice(n, origin=(0.0, 0.0, 0.0)):
    o = np.asarray(origin, np.float32)
    cap = int(np.ceil(np.cbrt(max(n, 1))) + 1) ** 3
    out = np.zeros((cap, 3), np.float32)
    c = lib().oracle_lattice(int(n), o, out, cap)
    return out[:c].copy()


def mesh(hmap512, dimx, dimy, dimz):
    m = np.ascontiguousarray(hmap512, np.uint8).ravel()
    verts = np.zeros(dimx * dimz * 6, np.float32)
    cap = 6 * dimx * dimz + 6
    idx = np.zeros(cap, np.uint32)
    ni = lib().oracle_mesh(m, dimx, dimy, dimz, verts, idx, cap)
    return verts, idx[:ni].copy()


def time_sample(params, pos, vel, i0, m, nthreads=0):
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    vel = np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
    return lib().oracle_time_sample(C.byref(params), len(pos), pos, vel, int(i0), int(m), int(nthreads))


# ---------------------------------------------------------------------------
class Reference:
    """The reference's own FluidSystemSPH, built headless (only where the
    reference sources are present)."""

    def __init__(self):
        if not os.path.exists(REF_PATH):
            raise FileNotFoundError(REF_PATH)
        L = C.CDLL(REF_PATH)
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C")
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
        L.ref_new.restype = C.c_void_p
        L.ref_free.argtypes = [C.c_void_p]
        L.ref_initialize.argtypes = [C.c_void_p, C.c_int]
        L.ref_add_particles.argtypes = [C.c_void_p, C.c_int]
        L.ref_reset.argtypes = [C.c_void_p]
        L.ref_set_origin.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float]
        L.ref_set_params.argtypes = [C.c_void_p, f32p]
        L.ref_get_params.argtypes = [C.c_void_p, f32p]
        L.ref_set_particles.argtypes = [C.c_void_p, C.c_int, f32p, C.c_void_p]
        L.ref_count.argtypes = [C.c_void_p]
        L.ref_count.restype = C.c_int
        L.ref_run.argtypes = [C.c_void_p, C.c_int]
        L.ref_get.argtypes = [C.c_void_p, f32p, i32p, i32p]
        L.ref_neighbour_counts.argtypes = [C.c_void_p, i32p]
        L.ref_grid_new.restype = C.c_void_p
        L.ref_grid_new.argtypes = [C.c_int, C.c_int, C.c_int]
        L.ref_grid_free.argtypes = [C.c_void_p]
        L.ref_grid_load.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(np.uint8, flags="C")]
        L.ref_grid_update.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.ref_grid_surface_size.argtypes = [C.c_void_p]
        L.ref_grid_indices_size.argtypes = [C.c_void_p]
        L.ref_grid_surface.argtypes = [C.c_void_p, f32p]
        L.ref_grid_indices.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(np.uint32, flags="C")]
        L.ref_grid_height_at.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.ref_grid_collision.argtypes = [C.c_void_p, f32p, f32p, f32p, f32p, f32p]
        L.ref_grid_collision.restype = C.c_int
        self.L = L
        self.h = L.ref_new()

    def close(self):
        if self.h:
            self.L.ref_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, g=(0.0, -9.82, 0.0), dt=0.0, p0=998.29, mass=0.02, visc=3.5, surf_tens=0.0728,
                   k=3.0, cr=0.5, h=0.0457, len=0.2, **_ignored):
        v = np.array([g[0], g[1], g[2], dt, p0, mass, visc, surf_tens, k, cr, h, len], np.float32)
        self.L.ref_set_params(self.h, v)

    def initialize(self, n):
        self.L.ref_initialize(self.h, int(n))

    def add_particles(self, n):
        self.L.ref_add_particles(self.h, int(n))

    def reset(self):
        self.L.ref_reset(self.h)

    def set_origin(self, o):
        self.L.ref_set_origin(self.h, float(o[0]), float(o[1]), float(o[2]))

    def set_particles(self, pos, vel=None):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        self.L.ref_set_particles(self.h, len(pos), pos, None if v is None else v.ctypes.data_as(C.c_void_p))

    def count(self):
        return self.L.ref_count(self.h)

    def run(self, nsteps=1):
        self.L.ref_run(self.h, int(nsteps))

    def get(self):
        n = self.count()
        rec = np.zeros((n, REC), np.float32)
        ids = np.zeros(n, np.int32)
        nb = np.zeros(n, np.int32)
        self.L.ref_get(self.h, rec, ids, nb)
        return rec, ids, nb

    def neighbour_counts(self):
        out = np.zeros(self.count(), np.int32)
        self.L.ref_neighbour_counts(self.h, out)
        return out
