"""GPU parity at the configured sizes, through the C ABI.

* The plain 1M scene (1,048,576 particles over 1024 x 1024 fBm, erosion on):
  one step of the GPU against the oracle's FP32 step (the reference's
  arithmetic and its all-pairs sums in ascending index) for a seeded sample
  of particle ids, from the initial block and from a developed state after
  300 steps.  Every FluidParticle field of the sample within RTOL = 1e-4
  (normwise relative per field), NeighbId exact, sediment within one unit
  plus RTOL; the FP32 oracle's own error against the FP64 oracle is printed
  beside it.
* The 16,384-particle block after 100 steps in ordered mode: equal to the
  f32x oracle bit for bit, and every field against the reference's own
  records, with the residual that libm's powf alone causes (f32 vs f32x
  oracle, both on the CPU) stated per field.
* Reduced rainfall over carved terrain (the skewed-occupancy configuration
  at 100,000 particles): sediment + terrain units exact at every check
  through 2,000 steps; and a 5,000-particle rain shower over a shallow
  carved terrain with erosion on, ordered mode equal to the f32x oracle bit
  for bit at steps 1, 50 and 150.
"""
import numpy as np
import pytest

import sph_gb300 as S
from helpers import C1, RTOL, field_errors, oracle_params

pytestmark = pytest.mark.gpu

ORDERED = S.SPH_FLAG_RECORD | S.SPH_FLAG_ORDERED
SAMPLE = 2048


def _report(tag, errs):
    print(tag, {k: f"{v:.2e}" for k, v in errs.items()})


def _sample_check(O, op, st, base, delta, nb_prev, rec, nb, sed, ids, tag):
    """GPU records of one step (rec, nb, sed by id) against the oracle's
    sampled FP32 step from the state st that the step started from."""
    o = O.sample(op, st["pos"], st["vel"], ids, sed=st["sed"], base=base, delta=delta, nbid=nb_prev,
                 precision="f32")
    o64 = O.sample(op, st["pos"].astype(np.float64), st["vel"].astype(np.float64), ids, sed=st["sed"], base=base,
                   delta=delta, nbid=nb_prev, precision="f64")
    e = field_errors(rec[ids], o["rec"])
    _report(f"{tag}: gpu vs oracle f32", e)
    _report(f"{tag}: oracle f32 vs f64", field_errors(o["rec"], o64["rec"]))
    _report(f"{tag}: gpu vs oracle f64", field_errors(rec[ids], o64["rec"]))
    for k, v in e.items():
        assert v <= RTOL, (tag, k, v)
    assert np.array_equal(nb[ids], o["nbid"]), tag
    ds = np.abs(sed[ids].astype(np.int64) - o["sed"])
    assert ds.max() <= 1 + RTOL * max(1, np.abs(o["sed"]).max()), (tag, ds.max())


@pytest.mark.parametrize("variant", [88, 264, 163960])
def test_plain_1m_sampled_fields_vs_oracle(oracle_lib, variant):
    """Per-lane passes (88), cooperative passes (264) and per-lane passes in
    fast arithmetic with dynamically scheduled force warps (163960)."""
    import workloads as W

    O = oracle_lib
    spec = W.plain_1m()
    n = spec["n"]
    t = spec["terrain"]
    op = oracle_params(O, spec["params"], terrain=(t["w"], t["d"]))
    ids = np.sort(np.random.default_rng(42).choice(n, SAMPLE, replace=False)).astype(np.int32)
    with S.System(particle_capacity=n, key_capacity=1 << 20, terrain_capacity=1 << 21, variant=variant) as sysm:
        sc = W.build_scene(sysm, spec, flags=S.SPH_FLAG_RECORD)
        base, delta = sc.get_terrain()  # no erosion yet: the heights are the base
        assert not delta.any()
        st = sc.get_particles()
        sysm.step(1)
        rec, nb = sc.get_records()
        _sample_check(O, op, st, base, delta, np.full(n, -1, np.int32), rec, nb, sc.get_particles()["sed"], ids,
                      f"1M variant {variant} step 1")
        sysm.step(299)
        st = sc.get_particles()
        _, delta = sc.get_terrain()
        _, nb_prev = sc.get_records()
        sysm.step(1)
        rec, nb = sc.get_records()
        after = sc.get_particles()
        _sample_check(O, op, st, base, delta, nb_prev, rec, nb, after["sed"], ids, f"1M variant {variant} step 301")
        assert sc.diag()["total_units"] == 0
        # the developed state is past the lattice: the sample's neighbourhoods differ
        cnt = sc.neighbour_counts()[ids]
        print("1M step 301: in-range neighbours of the sample", cnt.min(), np.median(cnt), cnt.max())
        assert len(np.unique(cnt)) > 5


def test_plain_16384_ordered_100_steps_vs_reference(oracle_lib, golden):
    """Ordered mode is the reference's arithmetic with correctly rounded
    x^2 and x^3.  After 100 steps it equals the f32x oracle bit for bit, so
    its distance to the reference is exactly the distance between the f32x
    and f32 oracles: the rounding of glibc's powf(x, 3) (it differs from the
    correctly rounded cube on about 0.07% of inputs; powf(x, 2) never does),
    amplified by 100 steps of a chaotic flow.  Every field is within RTOL of
    the reference except the ones listed in POWF_RESIDUAL_16384, whose error is
    asserted equal to that powf residual and bounded by it."""
    O = oracle_lib
    g = golden("ref_c1_16384.npz")
    p = oracle_params(O, C1)
    with S.System(particle_capacity=len(g["pos0"])) as sysm:
        sc = sysm.scene(S.default_params(**C1, flags=ORDERED), capacity=len(g["pos0"]))
        sc.set_particles(g["pos0"])
        sysm.step(1)
        rec1, nb1 = sc.get_records()
        sysm.step(99)
        rec, nb = sc.get_records()
    assert np.array_equal(rec1, g["rec1"]) and np.array_equal(nb1, g["nb1"])
    x = O.run_grid(p, g["pos0"], nsteps=100, precision="f32x")
    assert np.array_equal(rec, x["rec"]) and np.array_equal(nb, x["nbid"])
    e_gpu = field_errors(rec, g["rec100"])
    e_powf = field_errors(x["rec"], g["rec100"])
    e64 = field_errors(rec, golden("fp64_c1_16384.npz")["rec100"])
    _report("16384 ordered step 100 vs reference", e_gpu)
    _report("16384 ordered step 100 vs fp64", e64)
    _report("16384 reference step 100 vs fp64", field_errors(g["rec100"], golden("fp64_c1_16384.npz")["rec100"]))
    assert e_gpu == e_powf
    for k, v in e_gpu.items():
        assert v <= POWF_RESIDUAL_16384.get(k, RTOL), (k, v)


# Per-field error of the f32x oracle against the reference after 100 steps
# of the 16,384-particle block, where it exceeds RTOL: the whole difference
# is glibc powf's rounding (the oracles differ in nothing else).
# Measured on the CPU: pressure force 1.474e-4; every other field below
# 1e-4 (acceleration 7.4e-5, force terms 3.8e-5 to 5.5e-5, position 9.6e-7).
POWF_RESIDUAL_16384 = {"fpress": 1.48e-4}


def _rain_shower(n=5000, seed=9):
    """A 5,000-particle rain shower: x, z uniform over a 0.8 x 0.8 m floor,
    heights uniform in the top 30% of a 0.2 m tall box (about the rest
    density), falling at 3 m/s onto 64 x 64 carved-valley terrain (amplitude
    0.06), erosion on; the drops reach the terrain within about 30 steps."""
    import workloads as W

    bh = (0.4, 0.1, 0.4)
    rng = np.random.default_rng(seed)
    pos = np.empty((n, 3), np.float32)
    s = W.SPACING
    pos[:, 0] = rng.uniform(-bh[0] + s / 2, bh[0] - s / 2, n)
    pos[:, 2] = rng.uniform(-bh[2] + s / 2, bh[2] - s / 2, n)
    pos[:, 1] = rng.uniform(bh[1] - 0.6 * bh[1], bh[1] - s / 2, n)
    vel = np.zeros_like(pos)
    vel[:, 1] = -3.0
    prm = dict(W.PHYS, box_half=bh, k_capacity=0.05)
    return prm, pos, vel


def test_rain_shower_ordered_bit_exact_with_erosion(oracle_lib):
    O = oracle_lib
    prm, pos, vel = _rain_shower()
    tw = td = 64
    heights = O.fbm(9, tw, td, 5, 0.06, kind=2)
    op = oracle_params(O, prm, terrain=(tw, td))
    with S.System(particle_capacity=len(pos)) as sysm:
        sc = sysm.scene(S.default_params(**prm, flags=ORDERED), capacity=len(pos), terrain=(tw, td))
        sc.set_terrain(heights)
        sc.set_particles(pos, vel)
        done = 0
        x = dict(pos=pos, vel=vel, nbid=None, sed=None, delta=None)
        for s in (1, 50, 150):
            sysm.step(s - done)
            x = O.run_grid(op, x["pos"], x["vel"], nsteps=s - done, nbid=x["nbid"], sed=x["sed"], base=heights,
                           delta=x["delta"], precision="f32x")
            done = s
            rec, nb = sc.get_records()
            st = sc.get_particles()
            _, dl = sc.get_terrain()
            assert np.array_equal(rec, x["rec"]), s
            assert np.array_equal(nb, x["nbid"]), s
            assert np.array_equal(st["sed"], x["sed"]) and np.array_equal(dl.ravel(), x["delta"]), s
            assert sc.diag()["total_units"] == 0
        assert (st["sed"] > 0).sum() > 100, "erosion never picked up sediment"


def test_rainfall_100k_exact_mass_through_2000_steps():
    """The skewed-occupancy configuration at 100,000 particles (its box floor
    and terrain scaled with the particle count): rain falls, reaches the
    carved valleys and pools.  Sediment + terrain units change by exactly 0
    at every one of 20 checks, every particle stays finite, and sediment is
    moving by the end."""
    import workloads as W

    spec = W.skew_rain(100_000)
    t = spec["terrain"]
    with S.System(particle_capacity=spec["n"], key_capacity=1 << 22, terrain_capacity=t["w"] * t["d"],
                  variant=88) as sysm:
        sc = W.build_scene(sysm, spec)
        moved = 0
        for _ in range(20):
            sysm.step(100)
            d = sc.diag()
            assert d["total_units"] == 0 and d["nan_particles"] == 0 and d["n"] == spec["n"]
            moved = max(moved, abs(d["sediment_units"]))
        st = sc.get_particles()
    assert np.isfinite(st["pos"]).all()
    assert moved > 0, "no sediment moved in 2,000 steps"
    # pooled: particles per 0.25 m x 0.25 m column of the floor, against the
    # uniform rain they started as
    bh = spec["params"]["box_half"]

    def columns(p):
        ix = np.clip(((p[:, 0] + bh[0]) / 0.25).astype(int), 0, int(2 * bh[0] / 0.25))
        iz = np.clip(((p[:, 2] + bh[2]) / 0.25).astype(int), 0, int(2 * bh[2] / 0.25))
        c = np.bincount(ix * 1000 + iz)
        return c[c > 0]

    c0, c1 = columns(spec["pos"]), columns(st["pos"])
    print("column occupancy max/mean: start", c0.max() / c0.mean(), "after 2000 steps", c1.max() / c1.mean())
    assert c1.max() / c1.mean() > 1.2 * c0.max() / c0.mean()


@pytest.mark.parametrize("variant", [88, 164088])
def test_batched_scenes_sampled_fields_vs_oracle(oracle_lib, variant):
    """The batched form against the oracle: eight of the seeded batched
    scenes (4,532 to 47,055 particles, terrain sides 64 to 512) stepped
    together in one system for 60 steps, then one more step of each checked
    on 512 sampled particles against the oracle's FP32 step from that
    scene's own state: every field within RTOL, NeighbId exact, sediment
    within one unit.  Exact (88) and fast-arithmetic (164088) kernels."""
    import workloads as W

    O = oracle_lib
    reqs = W.batched_requests(256)[:8]
    base = S.default_params(**dict(W.PHYS, cell_mult=0.5, flags=S.SPH_FLAG_RECORD))
    total = sum(r["particles"] for r in reqs)
    with S.System(particle_capacity=total + 512 * len(reqs), key_capacity=1 << 22, terrain_capacity=1 << 20,
                  variant=variant) as sysm:
        scenes = [sysm.scene_from_request(base, r) for r in reqs]
        bases = [sc.get_terrain()[0] for sc in scenes]  # before any erosion: the base heights
        sysm.step(60)
        states = []
        for sc in scenes:
            st = sc.get_particles()
            _, dl = sc.get_terrain()
            _, nb = sc.get_records()
            states.append((st, dl, nb))
        sysm.step(1)
        for k, (sc, (st, dl, nb_prev), hb) in enumerate(zip(scenes, states, bases)):
            n = sc.count()
            rec, nb = sc.get_records()
            after = sc.get_particles()
            prm = S.params_dict(sc.params())
            tw, td = sc.terrain_dims()
            op = oracle_params(O, prm, terrain=(tw, td))
            ids = np.sort(np.random.default_rng(k).choice(n, min(512, n), replace=False)).astype(np.int32)
            _sample_check(O, op, st, hb, dl, nb_prev, rec, nb, after["sed"], ids,
                          f"batched scene {k} ({n} particles, {tw}x{td}) variant {variant}")
            assert sc.diag()["total_units"] == 0
