"""ctypes binding of libsph_gb300.so (include/sph_erosion.h).

The product path is the CUDA library; this module only marshals arguments.
Loading fails loudly when the library has not been built: there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsph_gb300.so")

SPH_FLAG_RECORD = 1
SPH_FLAG_ORDERED = 2
ERRORS = {-1: "invalid", -2: "cuda", -3: "nomem", -4: "capacity", -5: "state", -6: "device"}


class SphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sph error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("gravity", C.c_float * 3), ("dt", C.c_float), ("rest_density", C.c_float), ("mass", C.c_float),
        ("viscosity", C.c_float), ("surface_tension", C.c_float), ("gas_stiffness", C.c_float),
        ("restitution", C.c_float), ("smoothing_radius", C.c_float), ("box_center", C.c_float * 3),
        ("box_half", C.c_float * 3), ("cell_mult", C.c_float), ("erosion", C.c_int), ("k_capacity", C.c_float),
        ("k_pickup", C.c_float), ("k_deposit", C.c_float), ("erosion_layer", C.c_float), ("flags", C.c_int),
    ]


class Particle(C.Structure):
    _fields_ = [
        ("id", C.c_int), ("position", C.c_float * 3), ("velocity", C.c_float * 3),
        ("acceleration", C.c_float * 3), ("density", C.c_float), ("pressure", C.c_float),
        ("pressure_force", C.c_float * 3), ("viscosity_force", C.c_float * 3), ("gravity_force", C.c_float * 3),
        ("surface_force", C.c_float * 3), ("surface_normal", C.c_float * 3), ("neighb_id", C.c_int),
        ("sediment", C.c_int32),
    ]


class Diag(C.Structure):
    _fields_ = [
        ("fluid_mass", C.c_double), ("momentum", C.c_double * 3), ("kinetic", C.c_double),
        ("potential", C.c_double), ("sediment_units", C.c_int64), ("terrain_units", C.c_int64),
        ("total_units", C.c_int64), ("unit_volume", C.c_double), ("n", C.c_int32), ("nan_particles", C.c_int32),
        ("state_hash", C.c_uint64),
    ]

    def as_dict(self):
        return {"fluid_mass": self.fluid_mass, "momentum": tuple(self.momentum), "kinetic": self.kinetic,
                "potential": self.potential, "sediment_units": self.sediment_units,
                "terrain_units": self.terrain_units, "total_units": self.total_units,
                "unit_volume": self.unit_volume, "n": self.n, "nan_particles": self.nan_particles,
                "state_hash": self.state_hash}


class SystemConfig(C.Structure):
    _fields_ = [
        ("device", C.c_int), ("particle_capacity", C.c_int64), ("key_capacity", C.c_int64),
        ("terrain_capacity", C.c_int64), ("max_scenes", C.c_int), ("tile", C.c_int), ("graph_steps", C.c_int),
        ("variant", C.c_int), ("hbm_budget", C.c_int64),
    ]


class Request(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("particles", C.c_int32), ("terrain_side", C.c_int32), ("steps", C.c_int32),
                ("coverage", C.c_float), ("amplitude", C.c_float), ("arrival_s", C.c_double)]


class Result(C.Structure):
    _fields_ = [("ticket", C.c_int64), ("seed", C.c_uint64), ("particles", C.c_int32), ("steps", C.c_int32),
                ("arrival_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double),
                ("total_units", C.c_int64), ("sediment_units", C.c_int64), ("nan_particles", C.c_int32),
                ("status", C.c_int32), ("kinetic", C.c_double), ("state_hash", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("wall_s", C.c_double), ("particle_steps", C.c_double),
                ("throughput", C.c_double), ("p50_s", C.c_double), ("p99_s", C.c_double), ("max_s", C.c_double),
                ("peak_bytes", C.c_int64), ("peak_active", C.c_int32), ("chunks", C.c_int32),
                ("peak_particles", C.c_int64), ("admit_s", C.c_double), ("prepare_s", C.c_double),
                ("gpu_wait_s", C.c_double), ("retire_s", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("tile", C.c_int), ("cell_mult", C.c_float), ("chunk_steps", C.c_int),
                ("hbm_budget", C.c_int64), ("max_active_particles", C.c_int64), ("max_scenes", C.c_int),
                ("base", Params), ("policy", C.c_int), ("variant", C.c_int)]


class TuneResult(C.Structure):
    _fields_ = [("tile", C.c_int), ("cell_mult", C.c_float), ("variant", C.c_int), ("ms_per_step", C.c_float),
                ("n_tried", C.c_int), ("tiles", C.c_int * 64), ("cell_mults", C.c_float * 64),
                ("variants", C.c_int * 64), ("ms", C.c_float * 64)]

    def as_dict(self):
        return {"tile": self.tile, "cell_mult": self.cell_mult, "variant": self.variant,
                "ms_per_step": self.ms_per_step,
                "tried": [(self.tiles[i], self.cell_mults[i], self.variants[i], self.ms[i])
                          for i in range(self.n_tried)]}


_lib = None
SIGNATURES = {
    "sph_system_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(TuneResult)]),
    "sph_scene_traversal_stats": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "sph_scene_save": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p]),
    "sph_scene_load": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p]),
    "sph_scene_load_heightfield_u8": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_float]),
    "sph_last_error": (C.c_char_p, []),
    "sph_params_default": (None, [C.POINTER(Params)]),
    "sph_system_config_default": (None, [C.POINTER(SystemConfig)]),
    "sph_system_create": (C.c_int, [C.POINTER(SystemConfig), C.POINTER(C.c_void_p)]),
    "sph_system_destroy": (C.c_int, [C.c_void_p]),
    "sph_system_step": (C.c_int, [C.c_void_p, C.c_int]),
    "sph_system_sync": (C.c_int, [C.c_void_p]),
    "sph_system_time_steps": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_float)]),
    "sph_system_profile_stages": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "sph_system_memory": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "sph_scene_create": (C.c_int, [C.c_void_p, C.POINTER(Params), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "sph_scene_destroy": (C.c_int, [C.c_void_p, C.c_int]),
    "sph_scene_set_params": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Params)]),
    "sph_scene_get_params": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Params)]),
    "sph_scene_set_steps": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "sph_scene_get_steps": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "sph_scene_set_particles": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "sph_scene_add_lattice": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_int)]),
    "sph_scene_count": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "sph_scene_get_particles": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sph_scene_get_particle": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(Particle)]),
    "sph_scene_get_records": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "sph_scene_diag": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Diag)]),
    "sph_scenes_diag": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(Diag)]),
    "sph_scene_set_terrain": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    "sph_scene_gen_terrain": (C.c_int, [C.c_void_p, C.c_int, C.c_uint64, C.c_int, C.c_float, C.c_float, C.c_float,
                                        C.c_int]),
    "sph_scene_get_terrain": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "sph_scene_terrain_dims": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sph_scene_debug_sort": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "sph_scene_neighbour_counts": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "sph_neighbour_list_capacity": (C.c_int, []),
    "sph_scene_grid_dims": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "sph_density_static": (C.c_int, [C.POINTER(Params), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sph_scene_from_request": (C.c_int, [C.c_void_p, C.POINTER(Params), C.POINTER(Request), C.POINTER(C.c_int)]),
    "sph_server_config_default": (None, [C.POINTER(ServerConfig)]),
    "sph_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "sph_server_destroy": (C.c_int, [C.c_void_p]),
    "sph_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_int64)]),
    "sph_server_poll": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sph_server_run_trace": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.POINTER(ServerStats)]),
    "sph_scene_get_particles_async": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p]),
    "sph_host_alloc": (C.c_int, [C.c_int64, C.POINTER(C.c_void_p)]),
    "sph_system_trim": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "sph_host_free": (C.c_int, [C.c_void_p]),
    "sph_grid_collision_u8": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p]),
}


def requests_array(reqs):
    """A ctypes array of Request from dicts or Request objects."""
    arr = (Request * len(reqs))()
    for i, r in enumerate(reqs):
        if isinstance(r, Request):
            arr[i] = r
        else:
            arr[i] = Request(int(r["seed"]), int(r["particles"]), int(r["terrain_side"]), int(r.get("steps", 0)),
                             float(r.get("coverage", 0.0)), float(r.get("amplitude", 0.0)),
                             float(r.get("arrival_s", 0.0)))
    return arr


class Server:
    """Continuous-batching request server (include/sph_erosion.h)."""

    def __init__(self, base: Params = None, tile=256, cell_mult=0.5, chunk_steps=16, hbm_budget=0,
                 max_active_particles=0, max_scenes=0, device=0, policy=0, variant=0):
        cfg = ServerConfig()
        lib().sph_server_config_default(C.byref(cfg))
        cfg.device, cfg.tile, cfg.cell_mult, cfg.chunk_steps = device, tile, cell_mult, chunk_steps
        cfg.policy = policy
        cfg.variant = variant or 0
        if hbm_budget:
            cfg.hbm_budget = hbm_budget
        cfg.max_active_particles = max_active_particles
        if max_scenes:
            cfg.max_scenes = max_scenes
        if base is not None:
            cfg.base = base
        h = C.c_void_p()
        _ck(lib().sph_server_create(C.byref(cfg), C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().sph_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run_trace(self, reqs):
        arr = requests_array(reqs)
        res = (Result * len(arr))()
        st = ServerStats()
        _ck(lib().sph_server_run_trace(self.h, arr, len(arr), res, C.byref(st)))
        return list(res), st.as_dict()

    def submit(self, req) -> int:
        arr = requests_array([req])
        t = C.c_int64()
        _ck(lib().sph_server_submit(self.h, C.byref(arr[0]), C.byref(t)))
        return t.value

    def poll(self, cap=64):
        out = (Result * cap)()
        n, active = C.c_int(), C.c_int()
        _ck(lib().sph_server_poll(self.h, out, cap, C.byref(n), C.byref(active)))
        return list(out[: n.value]), active.value


def lib():
    """Load libsph_gb300.so; raise if it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built; run build() first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ck(rc: int):
    if rc != 0:
        raise SphError(rc, lib().sph_last_error().decode())


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def pinned_empty(shape, dtype=np.float32):
    """A numpy array in pinned host memory (freed with the array)."""
    import weakref

    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    ptr = C.c_void_p()
    _ck(lib().sph_host_alloc(max(n, 1), C.byref(ptr)))
    buf = (C.c_byte * max(n, 1)).from_address(ptr.value)
    weakref.finalize(buf, lib().sph_host_free, ptr.value)
    return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)


def grid_collision(hmap, dims, cur, nxt, vel):
    """Grid::collision (Erosion/grid.h:462-805) for a batch of queries on the
    GPU.  hmap: 512 x 512 uint8 map indexed [x, z]; dims: (m_DimX, m_DimZ) or
    the Grid's (x, y, z) dims; cur/nxt/vel: (n, 3) float32.  Returns
    (hit bool[n], contact (n, 3), normal (n, 3))."""
    m = np.ascontiguousarray(hmap, np.uint8)
    if m.size != 512 * 512:
        raise ValueError("the height map is 512 x 512")
    dx, dz = (dims[0], dims[-1])
    cur, nxt, vel = (np.ascontiguousarray(a, np.float32).reshape(-1, 3) for a in (cur, nxt, vel))
    n = cur.shape[0]
    if nxt.shape[0] != n or vel.shape[0] != n:
        raise ValueError("cur, nxt and vel need the same number of queries")
    cp = np.zeros((n, 3), np.float32)
    nr = np.zeros((n, 3), np.float32)
    hit = np.zeros(n, np.int32)
    _ck(lib().sph_grid_collision_u8(_p(m), int(dx), int(dz), n, _p(cur), _p(nxt), _p(vel), _p(cp), _p(nr),
                                    _p(hit)))
    return hit.astype(bool), cp, nr


def neighbour_list_capacity() -> int:
    """Entries one particle's neighbour list holds, self included."""
    return lib().sph_neighbour_list_capacity()


def default_params(**overrides) -> Params:
    """Reference defaults (fluid_system.h:460-479) with keyword overrides;
    vector fields take 3-sequences."""
    p = Params()
    lib().sph_params_default(C.byref(p))
    for k, v in overrides.items():
        if k in ("gravity", "box_center", "box_half"):
            getattr(p, k)[:] = [float(x) for x in v]
        elif k == "box_len":
            p.box_half[:] = [float(v)] * 3
        else:
            setattr(p, k, v)
    return p


def params_dict(p: Params) -> dict:
    d = {}
    for name, _ in Params._fields_:
        v = getattr(p, name)
        d[name] = tuple(v) if not isinstance(v, (int, float)) else v
    return d


class System:
    def __init__(self, particle_capacity=1 << 16, key_capacity=1 << 16, terrain_capacity=1 << 12, max_scenes=1024,
                 tile=256, graph_steps=16, hbm_budget=0, device=0, variant=None):
        cfg = SystemConfig()
        lib().sph_system_config_default(C.byref(cfg))
        cfg.device, cfg.particle_capacity, cfg.key_capacity = device, particle_capacity, key_capacity
        cfg.terrain_capacity, cfg.max_scenes, cfg.tile = terrain_capacity, max_scenes, tile
        cfg.graph_steps, cfg.hbm_budget = graph_steps, hbm_budget
        if variant is not None:
            cfg.variant = variant
        h = C.c_void_p()
        _ck(lib().sph_system_create(C.byref(cfg), C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().sph_system_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def scene_from_request(self, base: Params, req) -> "Scene":
        arr = requests_array([req])
        sid = C.c_int()
        _ck(lib().sph_scene_from_request(self.h, C.byref(base), C.byref(arr[0]), C.byref(sid)))
        return Scene(self, sid.value)

    def scene(self, params: Params, capacity=0, terrain=(0, 0)) -> "Scene":
        sid = C.c_int()
        _ck(lib().sph_scene_create(self.h, C.byref(params), int(capacity), int(terrain[0]), int(terrain[1]),
                                   C.byref(sid)))
        return Scene(self, sid.value)

    def step(self, n=1):
        _ck(lib().sph_system_step(self.h, int(n)))

    def sync(self):
        _ck(lib().sph_system_sync(self.h))

    def time_steps(self, n) -> float:
        ms = C.c_float()
        _ck(lib().sph_system_time_steps(self.h, int(n), C.byref(ms)))
        return ms.value

    def profile_stages(self, n) -> np.ndarray:
        out = np.zeros(8, np.float32)
        _ck(lib().sph_system_profile_stages(self.h, int(n), _p(out)))
        return out

    def autotune(self, steps=8) -> dict:
        r = TuneResult()
        _ck(lib().sph_system_autotune(self.h, int(steps), C.byref(r)))
        return r.as_dict()

    def trim(self) -> bool:
        """With no live scene, release the arenas' memory (back to the
        initial capacities); False when a scene is live."""
        t = C.c_int()
        _ck(lib().sph_system_trim(self.h, C.byref(t)))
        return bool(t.value)

    def diag_many(self, scenes) -> list:
        """Diagnostics of several scenes in one launch (Scene objects or ids)."""
        ids = [s.id if isinstance(s, Scene) else int(s) for s in scenes]
        if not ids:
            return []
        arr = (C.c_int * len(ids))(*ids)
        out = (Diag * len(ids))()
        _ck(lib().sph_scenes_diag(self.h, len(ids), arr, out))
        return [d.as_dict() for d in out]

    def memory(self) -> int:
        b = C.c_int64()
        _ck(lib().sph_system_memory(self.h, C.byref(b)))
        return b.value


STAGES = ["keys", "scan", "scatter", "reorder", "density", "force", "terrain", "tick"]


class Scene:
    def __init__(self, system: System, sid: int):
        self.sys = system
        self.id = sid

    @property
    def h(self):
        return self.sys.h

    def destroy(self):
        _ck(lib().sph_scene_destroy(self.h, self.id))

    def set_params(self, p: Params):
        _ck(lib().sph_scene_set_params(self.h, self.id, C.byref(p)))

    def params(self) -> Params:
        p = Params()
        _ck(lib().sph_scene_get_params(self.h, self.id, C.byref(p)))
        return p

    def set_steps(self, n):
        _ck(lib().sph_scene_set_steps(self.h, self.id, int(n)))

    def steps(self) -> int:
        v = C.c_int()
        _ck(lib().sph_scene_get_steps(self.h, self.id, C.byref(v)))
        return v.value

    def set_particles(self, pos, vel=None):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        _ck(lib().sph_scene_set_particles(self.h, self.id, len(pos), _p(pos), _p(v)))

    def add_lattice(self, n, origin=(0.0, 0.0, 0.0)) -> int:
        o = np.asarray(origin, np.float32)
        added = C.c_int()
        _ck(lib().sph_scene_add_lattice(self.h, self.id, int(n), _p(o), C.byref(added)))
        return added.value

    def count(self) -> int:
        v = C.c_int()
        _ck(lib().sph_scene_count(self.h, self.id, C.byref(v)))
        return v.value

    def get_particles(self):
        n = self.count()
        pos = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        dens = np.zeros(n, np.float32)
        sed = np.zeros(n, np.int32)
        _ck(lib().sph_scene_get_particles(self.h, self.id, _p(pos), _p(vel), _p(dens), _p(sed)))
        return dict(pos=pos, vel=vel, density=dens, sed=sed)

    def get_positions(self, out=None):
        n = self.count()
        out = np.zeros((n, 3), np.float32) if out is None else out
        _ck(lib().sph_scene_get_particles(self.h, self.id, _p(out), None, None, None))
        return out

    def get_positions_async(self, out):
        """Enqueue the positions readback into `out` (pinned, see
        pinned_empty); complete after System.sync()."""
        _ck(lib().sph_scene_get_particles_async(self.h, self.id, _p(out), None, None, None))
        return out

    def get_records(self):
        n = self.count()
        rec = np.zeros((n, 27), np.float32)
        nb = np.zeros(n, np.int32)
        _ck(lib().sph_scene_get_records(self.h, self.id, _p(rec), _p(nb)))
        return rec, nb

    def get_particle(self, pid) -> Particle:
        out = Particle()
        _ck(lib().sph_scene_get_particle(self.h, self.id, int(pid), C.byref(out)))
        return out

    def diag(self) -> dict:
        d = Diag()
        _ck(lib().sph_scene_diag(self.h, self.id, C.byref(d)))
        return d.as_dict()

    def set_terrain(self, heights):
        hgt = np.ascontiguousarray(heights, np.float32)
        d, w = hgt.shape
        _ck(lib().sph_scene_set_terrain(self.h, self.id, int(w), int(d), _p(hgt)))

    def gen_terrain(self, seed, octaves, amplitude, lacunarity=2.0, gain=0.5, kind=0):
        _ck(lib().sph_scene_gen_terrain(self.h, self.id, int(seed), int(octaves), float(amplitude),
                                        float(lacunarity), float(gain), int(kind)))

    def terrain_dims(self):
        w, d = C.c_int(), C.c_int()
        _ck(lib().sph_scene_terrain_dims(self.h, self.id, C.byref(w), C.byref(d)))
        return w.value, d.value

    def get_terrain(self):
        w, d = self.terrain_dims()
        hgt = np.zeros((d, w), np.float32)
        dl = np.zeros((d, w), np.int64)
        _ck(lib().sph_scene_get_terrain(self.h, self.id, _p(hgt), _p(dl)))
        return hgt, dl

    def debug_sort(self):
        n = self.count()
        keys = np.zeros(n, np.uint32)
        order = np.zeros(n, np.int32)
        _ck(lib().sph_scene_debug_sort(self.h, self.id, _p(keys), _p(order)))
        return keys, order

    def neighbour_counts(self):
        out = np.zeros(self.count(), np.int32)
        _ck(lib().sph_scene_neighbour_counts(self.h, self.id, _p(out)))
        return out

    def save(self, path):
        _ck(lib().sph_scene_save(self.h, self.id, str(path).encode()))

    def load(self, path):
        _ck(lib().sph_scene_load(self.h, self.id, str(path).encode()))

    def load_heightfield_u8(self, map512, metres_per_level):
        m = np.ascontiguousarray(map512, np.uint8).ravel()
        if m.size != 512 * 512:
            raise ValueError("the heightfield is 512 x 512 bytes")
        _ck(lib().sph_scene_load_heightfield_u8(self.h, self.id, _p(m), float(metres_per_level)))

    def traversal_stats(self) -> dict:
        out = np.zeros(4, np.int64)
        _ck(lib().sph_scene_traversal_stats(self.h, self.id, _p(out)))
        return {"particles": int(out[0]), "rows": int(out[1]), "candidates": int(out[2]), "in_range": int(out[3])}

    def grid_dims(self):
        out = np.zeros(4, np.int32)
        _ck(lib().sph_scene_grid_dims(self.h, self.id, _p(out)))
        return tuple(int(x) for x in out)
