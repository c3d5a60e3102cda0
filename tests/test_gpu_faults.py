"""Failure handling without any GPU fault: malformed inputs are refused on
the host with an error code, a NaN-seeded scene is reported by the FP64
diagnostic without contaminating its neighbours, and a budget that cannot
hold a scene refuses it."""
import numpy as np
import pytest

import sph_gb300 as S
import workloads as W

pytestmark = pytest.mark.gpu


def test_nan_particle_is_isolated_and_reported():
    pos = W.lattice_block(12, 6, 12, W.SPACING, (-0.12, -0.2, -0.12))
    pos[len(pos) // 2] = np.nan
    with S.System() as sysm:
        sc = sysm.scene(S.default_params(**dict(W.PHYS, box_half=(0.3, 0.3, 0.3), erosion=0)))
        sc.set_particles(pos)
        sysm.step(20)
        d = sc.diag()
        st = sc.get_particles()
    assert d["nan_particles"] == 1
    bad = ~np.isfinite(st["pos"]).all(axis=1)
    assert bad.sum() == 1 and bad[len(pos) // 2]


@pytest.mark.parametrize("req", [dict(seed=1, particles=0, terrain_side=64, steps=10),
                                 dict(seed=1, particles=1000, terrain_side=1, steps=10),
                                 dict(seed=1, particles=1000, terrain_side=64, steps=-1)])
def test_malformed_requests_are_refused(req):
    with S.Server(W.base_params(), chunk_steps=8) as srv:
        with pytest.raises(S.SphError):
            srv.submit(req)
            srv.poll()


def test_invalid_parameters_are_refused():
    with S.System() as sysm:
        for bad in (dict(smoothing_radius=0.0), dict(box_half=(0.5, -1.0, 0.5)), dict(cell_mult=0.1)):
            with pytest.raises(S.SphError):
                sysm.scene(S.default_params(**dict(W.PHYS, **bad)))


def test_budget_too_small_refuses_scene():
    with S.System(particle_capacity=512, key_capacity=4096, terrain_capacity=512, hbm_budget=8 << 20) as sysm:
        with pytest.raises(S.SphError) as e:
            sysm.scene_from_request(W.base_params(), dict(seed=3, particles=200000, terrain_side=512, steps=0))
        assert e.value.code == -4  # SPH_ERR_CAPACITY
        # the system stays usable
        sc = sysm.scene_from_request(W.base_params(), dict(seed=3, particles=2000, terrain_side=64, steps=0))
        sysm.step(2)
        assert sc.diag()["total_units"] == 0


def test_refused_grid_resize_keeps_the_scene_running():
    """A parameter change whose finer grid does not fit the budget is refused
    and the scene continues with its old parameters, bit for bit."""
    req = dict(seed=11, particles=2000, terrain_side=64, steps=0)
    cfg = dict(key_capacity=4096)  # key arena sized by the scene, so a finer grid must grow it
    with S.System(**cfg) as probe:
        sc = probe.scene_from_request(W.base_params(), req)
        need = probe.memory()
        probe.step(5)
        want = sc.get_particles()["pos"]
    with S.System(hbm_budget=need + (256 << 10), **cfg) as sysm:
        sc = sysm.scene_from_request(W.base_params(), req)
        p = sc.params()
        old = p.cell_mult
        p.cell_mult = 0.25  # 8 times the cells: at least 400 KB more keys than the 256 KB of slack
        with pytest.raises(S.SphError) as e:
            sc.set_params(p)
        assert e.value.code == -4
        assert sc.params().cell_mult == old
        sysm.step(5)
        assert np.array_equal(sc.get_particles()["pos"], want)


def test_trim_returns_arena_memory_when_idle():
    """Arenas only grow; with no live scene, trim returns their memory, so a
    request with a different size mix fits a budget again."""
    big_terrain = dict(seed=5, particles=4096, terrain_side=1024, steps=0)
    many_particles = dict(seed=6, particles=120000, terrain_side=64, steps=0)
    with S.System() as probe:
        probe.scene_from_request(W.base_params(), many_particles)
        need_b = probe.memory()
    with S.System() as probe:
        probe.scene_from_request(W.base_params(), big_terrain)
        need_a = probe.memory()
    budget = max(need_a, need_b) + (1 << 20)
    with S.System(hbm_budget=budget) as sysm:
        a = sysm.scene_from_request(W.base_params(), big_terrain)
        assert not sysm.trim()  # a scene is live
        a.destroy()
        with pytest.raises(S.SphError):
            sysm.scene_from_request(W.base_params(), many_particles)
        assert sysm.trim()
        b = sysm.scene_from_request(W.base_params(), many_particles)
        sysm.step(2)
        assert b.diag()["total_units"] == 0


def test_grid_beyond_key_limit_is_refused():
    """A box whose uniform grid would need more than 2^30 cell keys is
    refused with an error code; a coarser cell size makes it fit."""
    with S.System() as sysm:
        with pytest.raises(S.SphError) as e:
            sysm.scene(S.default_params(**dict(W.PHYS, box_half=(60.0, 60.0, 60.0))))
        assert e.value.code == -4
        sc = sysm.scene(S.default_params(**dict(W.PHYS, box_half=(10.0, 1.0, 10.0), cell_mult=1.0)))
        assert sc.grid_dims()[3] <= (1 << 30) + 1


def test_server_refuses_a_request_that_cannot_fit():
    """A request whose scene exceeds the whole HBM budget is refused when it
    is submitted, so it cannot block the queue; the server goes on serving."""
    small = dict(seed=7001, particles=2048, terrain_side=64, steps=12)
    big = dict(seed=7002, particles=262144, terrain_side=512, steps=12)
    with S.Server(W.base_params(), chunk_steps=8, hbm_budget=24 << 20) as srv:
        with pytest.raises(S.SphError) as e:
            srv.submit(big)
        assert e.value.code == -4
        (res,), stats = srv.run_trace([dict(small, arrival_s=0.0)])
    assert stats["completed"] == 1
    assert res.status == 0 and res.total_units == 0 and res.state_hash != 0


def test_server_runs_a_request_without_lists_when_only_they_do_not_fit():
    """With nothing resident, a request whose scene fits the budget but whose
    neighbour lists do not is admitted and runs without the lists; it
    completes with status 0, exact mass and the same fingerprint as with the
    lists (the per-lane passes give the same bits either way), and the next
    request is admitted only once it has retired."""
    a = dict(seed=7011, particles=40000, terrain_side=128, steps=24)
    b = dict(seed=7012, particles=2048, terrain_side=64, steps=12)
    with S.Server(W.base_params(), chunk_steps=8) as roomy:
        (ra_lists,), st = roomy.run_trace([dict(a, arrival_s=0.0)])
    # the server samples its memory when it admits, before the first step
    # allocates the lists; those are 772 B per particle of the particle
    # arena (at least 2^16 particles: 50.6 MB), so 16 MB more than that peak
    # holds everything but them
    budget = int(st["peak_bytes"]) + (16 << 20)
    with S.Server(W.base_params(), chunk_steps=8, hbm_budget=budget) as srv:
        (ra, rb), stats = srv.run_trace([dict(a, arrival_s=0.0), dict(b, arrival_s=0.0)])
    assert stats["peak_bytes"] <= budget
    assert ra.status == 0 and rb.status == 0
    assert ra.total_units == 0 and rb.total_units == 0 and ra.nan_particles == 0
    assert ra.state_hash == ra_lists.state_hash
    assert rb.admit_s >= ra.done_s  # b waited for a to retire
