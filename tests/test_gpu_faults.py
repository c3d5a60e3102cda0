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
