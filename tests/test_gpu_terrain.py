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


def test_grid_collision_matches_reference(golden):
    """Grid::collision (grid.h:462-805) on 6000 seeded queries over a seeded
    8-bit map, against the reference's own answers: bit-exact hit flags,
    contact points and normals."""
    g = golden("ref_collision.npz")
    hit, cp, nr = S.grid_collision(g["hmap"], tuple(int(v) for v in g["dims"]), g["cur"], g["next"], g["vel"])
    want = g["hit"].astype(bool)
    assert want.sum() > 1000 and (~want).sum() > 1000
    assert np.array_equal(hit, want)
    assert np.array_equal(cp.view(np.uint32), g["contact"].view(np.uint32))
    assert np.array_equal(nr.view(np.uint32), g["normal"].view(np.uint32))


def test_grid_collision_edges(golden):
    g = golden("ref_collision.npz")
    hm = g["hmap"]
    # queries whose start or end cell lies outside [0, dim - 1) never collide (grid.h:471-473)
    cur = np.array([[-0.5, 200, 10], [10, 200, 10], [99.5, 200, 10], [10, 200, 99.2]], np.float32)
    nxt = np.array([[0.5, 0, 10], [-0.2, 0, 10], [98.7, 0, 10], [10, 0, 98.0]], np.float32)
    hit, cp, nr = S.grid_collision(hm, (100, 256, 100), cur, nxt, nxt - cur)
    assert not hit.any() and not cp.any() and not nr.any()
    # an empty batch, and maps or dims the routine cannot address
    h0, c0, n0 = S.grid_collision(hm, (100, 100), np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3)))
    assert h0.shape == (0,) and c0.shape == (0, 3)
    with pytest.raises(S.SphError):
        S.grid_collision(hm, (1, 100), cur, nxt, nxt - cur)
    with pytest.raises(S.SphError):
        S.grid_collision(hm, (100, 513), cur, nxt, nxt - cur)
    with pytest.raises(ValueError):
        S.grid_collision(hm[:100], (100, 100), cur, nxt, nxt - cur)


def test_grid_collision_known_answers():
    """Known answers derived from grid.h (and confirmed with the reference's
    own code): a particle moving down through a flat field at height H lands
    on y = H with the normal (0, 1, 0); one that stops above it has no
    contact; on the terraced field 10 + x/8 the contact is on the terrace."""
    flat = np.full((512, 512), 10, np.uint8)
    cur = np.array([[30.25, 12.0, 40.5], [30.25, 12.0, 40.5]], np.float32)
    nxt = np.array([[30.3, 9.5, 40.55], [30.3, 10.5, 40.55]], np.float32)
    hit, cp, nr = S.grid_collision(flat, (100, 256, 100), cur, nxt, (nxt - cur) / 0.01)
    assert hit.tolist() == [True, False]
    assert np.array_equal(cp[0], np.float32([30.3, 10.0, 40.55])) and np.array_equal(nr[0], [0, 1, 0])
    assert not cp[1].any() and not nr[1].any()
    x = np.arange(512)[:, None] * np.ones((1, 512))
    terraced = (10 + x // 8).astype(np.uint8)
    cur = np.array([[20.3, 13.5, 20.6]], np.float32)
    nxt = np.array([[20.35, 11.0, 20.62]], np.float32)
    hit, cp, nr = S.grid_collision(terraced, (100, 256, 100), cur, nxt, (nxt - cur) / 0.01)
    assert hit[0] and np.array_equal(cp[0], np.float32([20.35, 12.0, 20.62])) and np.array_equal(nr[0], [0, 1, 0])
