"""Terrain access on the GPU: the reference's surface mesh (Grid::UpdateGrid,
genIndices) bit for bit, and the world-space mesh of an eroded scene."""
import ctypes as C

import numpy as np
import pytest

import sph_gb300 as S
import workloads as W

pytestmark = pytest.mark.gpu


def _mesh_u8(hmap, dims):
    L = S.lib()
    L.sph_terrain_mesh_u8.restype = C.c_int
    L.sph_terrain_mesh_u8.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int64,
                                      C.POINTER(C.c_int64)]
    m = np.ascontiguousarray(hmap, np.uint8)
    dx, dy, dz = dims
    ni = C.c_int64()
    assert L.sph_terrain_mesh_u8(m.ctypes.data, dx, dy, dz, None, None, 0, C.byref(ni)) == 0
    verts = np.zeros(dx * dz * 6, np.float32)
    idx = np.zeros(ni.value, np.uint32)
    assert L.sph_terrain_mesh_u8(m.ctypes.data, dx, dy, dz, verts.ctypes.data, idx.ctypes.data, ni.value,
                                 C.byref(ni)) == 0
    return verts, idx


def test_mesh_u8_matches_reference(golden):
    g = golden("ref_mesh.npz")
    verts, idx = _mesh_u8(g["hmap"], tuple(int(v) for v in g["dims"]))
    assert np.array_equal(verts, g["surface"])
    assert np.array_equal(idx, g["indices"])


@pytest.mark.parametrize("dims", [(64, 255, 64), (2, 3, 5), (512, 100, 512), (37, 700, 13)])
def test_mesh_u8_matches_oracle(golden, oracle_lib, dims):
    hm = golden("ref_mesh.npz")["hmap"]
    verts, idx = _mesh_u8(hm, dims)
    ov, oi = oracle_lib.mesh(hm, *dims)
    assert np.array_equal(verts, ov, equal_nan=True)
    assert np.array_equal(idx, oi)


def test_scene_mesh_follows_erosion():
    req = dict(seed=4242, particles=6000, terrain_side=64, steps=0)
    with S.System() as sysm:
        sc = sysm.scene_from_request(W.base_params(), req)
        L = S.lib()
        L.sph_scene_terrain_mesh.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        sysm.step(40)
        hgt, delta = sc.get_terrain()
        verts = np.zeros(64 * 64 * 6, np.float32)
        idx = np.zeros(6 * 63 * 63, np.uint32)
        assert L.sph_scene_terrain_mesh(sysm.h, sc.id, verts.ctypes.data, idx.ctypes.data) == 0
        prm = sc.params()
    v = verts.reshape(-1, 6)
    assert np.array_equal(v[:, 1], np.float32(-prm.box_half[1]) + hgt.ravel())
    n = v[:, 3:6]
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-5) and (n[:, 1] > 0).all()
    assert idx.max() < 64 * 64
    assert delta.any(), "erosion should have changed the terrain"
