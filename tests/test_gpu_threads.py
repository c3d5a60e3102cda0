"""Host threads.  Calls on one system handle are not thread-safe; different
handles are: each thread's results equal the same run made alone, and a
failure's message (sph_last_error) belongs to the thread that failed."""
import threading

import numpy as np
import pytest

import sph_gb300 as S
import workloads as W

pytestmark = pytest.mark.gpu

REQS = [dict(seed=9100 + i, particles=p, terrain_side=s, steps=0)
        for i, (p, s) in enumerate([(6000, 128), (9000, 64), (4096, 256), (12000, 128)])]


def _run(req, steps):
    with S.System(tile=128) as sysm:
        sc = sysm.scene_from_request(W.base_params(), req)
        sysm.step(steps)
        st = sc.get_particles()
        return st["pos"], st["vel"], st["sed"], sc.diag()["state_hash"]


def test_threads_on_separate_systems_match_runs_alone():
    steps = 25
    alone = [_run(r, steps) for r in REQS]
    out = [None] * len(REQS)
    errs = []

    def work(k):
        try:
            out[k] = _run(REQS[k], steps)
        except Exception as e:  # reported below
            errs.append(e)

    ts = [threading.Thread(target=work, args=(k,)) for k in range(len(REQS))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errs, errs
    for a, b in zip(alone, out):
        for x, y in zip(a[:3], b[:3]):
            assert np.array_equal(x, y)
        assert a[3] == b[3]


def test_error_messages_stay_with_their_thread():
    seen = {"params": set(), "scene": set()}
    start = threading.Barrier(2)

    def bad_params(sysm):
        start.wait()
        for _ in range(200):
            with pytest.raises(S.SphError) as e:
                sysm.scene(S.default_params(cell_mult=0.01))
            seen["params"].add(str(e.value))

    def bad_scene(sysm):
        ghost = S.Scene(sysm, 12345)  # no such scene in this system
        start.wait()
        for _ in range(200):
            with pytest.raises(S.SphError) as e:
                ghost.count()
            seen["scene"].add(str(e.value))

    with S.System() as a, S.System() as b:
        ts = [threading.Thread(target=bad_params, args=(a,)), threading.Thread(target=bad_scene, args=(b,))]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
    assert len(seen["params"]) == 1 and "cell_mult" in next(iter(seen["params"]))
    assert len(seen["scene"]) == 1 and "no such scene" in next(iter(seen["scene"]))
