"""The plain workload at its full size (1,048,576 particles over a 1024^2
fBm terrain, cells of h/2, erosion on), checked through properties that do
not depend on size:

* sediment + terrain mass units change by exactly 0;
* every particle is present once, with a finite position;
* cell keys equal the oracle's, and the sorted order equals the oracle's
  stable counting sort (linear in the particle count, so it runs at full
  size) while the particles are still stored in id order; after stepping
  they are stored in the previous step's sorted order, so the order is
  checked to be a key-sorted permutation;
* in-range neighbour counts of sampled particles equal an exact FP32
  all-pairs count against all particles, with the reference's test
  (fluid_system.h:139-142, glm::length(r) <= h with length = sqrt(dot)).
"""
import numpy as np
import pytest

import sph_gb300 as S
import workloads as W

pytestmark = pytest.mark.gpu


def _smax(h):
    """Largest FP32 s with sqrtf(s) <= h: the squared-distance form of the
    reference's in-range test."""
    h = np.float32(h)
    s = np.float32(h * h)
    while np.sqrt(np.nextafter(s, np.float32(np.inf))) <= h:
        s = np.nextafter(s, np.float32(np.inf))
    while np.sqrt(s) > h:
        s = np.nextafter(s, np.float32(0))
    return s


def test_full_size_plain_1m_properties(oracle_lib):
    O = oracle_lib
    spec = W.plain_1m()
    spec = dict(spec, params=dict(spec["params"], cell_mult=0.5))
    n = spec["n"]
    with S.System(particle_capacity=n, key_capacity=1 << 22, terrain_capacity=1 << 21, tile=128) as sysm:
        sc = W.build_scene(sysm, spec)
        assert sc.diag()["total_units"] == 0
        keys0, order0 = sc.debug_sort()
        pos0 = sc.get_particles()["pos"]
        sysm.step(200)  # past the lattice phase: the dam is collapsing
        d = sc.diag()
        st = sc.get_particles()
        keys, order = sc.debug_sort()
        nx, ny, nz, nkeys = sc.grid_dims()
        cnt = sc.neighbour_counts()
    assert d["n"] == n and d["nan_particles"] == 0
    assert d["total_units"] == 0  # exact mass
    pos = st["pos"]
    assert pos.shape == (n, 3) and np.isfinite(pos).all()

    prm = spec["params"]
    grd = O.grid(O.make_params(box_l=prm["box_half"], h=prm["smoothing_radius"]), 0.5)
    assert (nx, ny, nz, nkeys) == (grd.nx, grd.ny, grd.nz, grd.nkeys)
    ok0 = O.cell_keys(grd, pos0)
    assert np.array_equal(keys0, ok0)
    assert np.array_equal(order0, O.stable_sort(ok0, grd.nkeys))
    ok = O.cell_keys(grd, pos)
    assert np.array_equal(keys, ok)
    assert np.array_equal(np.sort(order), np.arange(n))
    assert np.all(np.diff(ok[order].astype(np.int64)) >= 0)

    smax = _smax(prm["smoothing_radius"])
    rng = np.random.default_rng(11)
    for i in rng.choice(n, 200, replace=False):
        r = pos - pos[i]  # float32: each operation rounded as in the reference
        s = (r[:, 0] * r[:, 0] + r[:, 1] * r[:, 1]) + r[:, 2] * r[:, 2]
        assert int(np.count_nonzero(s <= smax)) - 1 == cnt[i], i
    assert 20 < cnt.mean() < 80
