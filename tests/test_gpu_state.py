"""Checkpoint/restore and 8-bit heightfield ingest through the C ABI."""
import numpy as np
import pytest

import sph_gb300 as S
import workloads as W

pytestmark = pytest.mark.gpu


def _state(sc):
    st = sc.get_particles()
    hgt, dl = sc.get_terrain()
    return st["pos"], st["vel"], st["sed"], hgt, dl


def test_checkpoint_resumes_bit_for_bit(tmp_path):
    req = dict(seed=99, particles=7000, terrain_side=96, steps=0)
    path = tmp_path / "scene.sphe"
    with S.System() as a:
        sa = a.scene_from_request(W.base_params(), req)
        a.step(25)
        sa.save(path)
        a.step(25)
        want = _state(sa)
        want_diag = sa.diag()
    with S.System(tile=128) as b:
        # a scene created with other parameters and no particles: everything is replaced
        sb = b.scene(S.default_params(), terrain=(8, 8))
        sb.load(path)
        assert sb.count() == req["particles"]
        b.step(25)
        got = _state(sb)
        got_diag = sb.diag()
    for x, y in zip(got, want):
        assert np.array_equal(x, y)
    assert got_diag["total_units"] == want_diag["total_units"] == 0


def test_checkpoint_rejects_garbage(tmp_path):
    bad = tmp_path / "bad.sphe"
    bad.write_bytes(b"NOPE" + bytes(64))
    with S.System() as s:
        sc = s.scene(S.default_params())
        with pytest.raises(S.SphError):
            sc.load(bad)
        with pytest.raises(S.SphError):
            sc.load(tmp_path / "missing.sphe")


def test_load_heightfield_u8(golden):
    hm = golden("ref_mesh.npz")["hmap"]
    with S.System() as s:
        sc = s.scene(S.default_params(box_half=(2.0, 1.0, 2.0)), terrain=(4, 4))
        sc.load_heightfield_u8(hm, 0.002)
        hgt, dl = sc.get_terrain()
    assert hgt.shape == (512, 512) and not dl.any()
    # the reference indexes map[512 * x + z]; the scene stores z-major rows
    want = (hm.astype(np.float32).reshape(512, 512).T * np.float32(0.002)).astype(np.float32)
    assert np.array_equal(hgt, want)
