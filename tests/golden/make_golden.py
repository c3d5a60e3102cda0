"""Generates the golden vectors in this directory from the reference's own
code (Erosion/fluid_system.h and Erosion/grid.h, built headless by
oracle/Makefile `ref`).  Run where the reference sources exist:

    python tests/golden/make_golden.py [/path/to/reference]

Every input is seeded; the files are small float32/int npz archives.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "sph-erosion_gb300"))

import oracle as O  # noqa: E402
import workloads as W  # noqa: E402

C1_REF = dict(g=(0.0, -9.81, 0.0), dt=1e-3, p0=1000.0, mass=float(np.float32(W.PHYS["mass"])), visc=0.1,
              surf_tens=0.0728, k=3.0, cr=0.5, h=0.04, len=0.5)


def rec_fields(rec):
    return {name: rec[:, sl] for name, sl in O.FIELDS.items()}


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"{name}: {os.path.getsize(path)} bytes")


def run_ref(params, pos, steps, vel=None):
    R = O.Reference()
    R.set_params(**params)
    R.set_particles(pos, vel)
    out = {}
    done = 0
    for s in steps:
        R.run(s - done)
        done = s
        rec, ids, nb = R.get()
        out[s] = (rec.copy(), nb.copy(), R.neighbour_counts())
    R.close()
    return out


def fp64_fixture():
    """FP64 oracle records of the 16,384-particle block after 100 steps
    (rounded to float32), the yardstick of the reference's own rounding
    error."""
    spec = W.plain_small(erosion=False, terrain=False)
    p = O.make_params(box_l=(0.5, 0.5, 0.5), **{k: v for k, v in C1_REF.items() if k != "len"})
    out = O.run(p, spec["pos"], nsteps=100, precision="f64")
    save("fp64_c1_16384.npz", rec100=out["rec"].astype(np.float32))


def c1_16384_fixture():
    """The full 16,384-particle plain-small block (32 x 16 x 32), no terrain
    (the reference has none): records after 1 and after 100 steps."""
    spec = W.plain_small(erosion=False, terrain=False)
    res = run_ref(C1_REF, spec["pos"], [1, 100])
    save("ref_c1_16384.npz", pos0=spec["pos"], rec1=res[1][0], nb1=res[1][1], cnt1=res[1][2].astype(np.int16),
         rec100=res[100][0], nb100=res[100][1], cnt100=res[100][2].astype(np.int16))


def collision_fixture():
    """Grid::collision (grid.h:462-805) on seeded queries over a seeded 8-bit
    heightfield: particles above the surface moving through it, in cells that
    keep every lookup of the routine inside the map."""
    import ctypes as C

    rng = np.random.default_rng(17)
    hm = np.clip(O.fbm(17, 512, 512, 4, 60.0) + 40.0 + rng.uniform(0, 3, (512, 512)), 0, 255).astype(np.uint8)
    dims = (100, 256, 100)
    L = O.Reference().L
    g = L.ref_grid_new(*dims)
    L.ref_grid_load(g, np.ascontiguousarray(hm.ravel()))
    nq = 6000
    cur = np.zeros((nq, 3), np.float32)
    nxt = np.zeros((nq, 3), np.float32)
    vel = np.zeros((nq, 3), np.float32)
    for q in range(nq):
        x, z = rng.uniform(3.0, 95.0, 2)
        h = float(hm.ravel()[int(x) * 512 + int(z)])
        cur[q] = (x, h + rng.uniform(0.05, 3.0), z)
        step = np.array([rng.uniform(-1.2, 1.2), -rng.uniform(0.1, 5.0), rng.uniform(-1.2, 1.2)])
        if q % 5 == 0:
            step[1] = rng.uniform(-0.5, 0.5)  # grazing motion
        nxt[q] = cur[q] + step
        vel[q] = step / 0.01
    cp = np.zeros((nq, 3), np.float32)
    nr = np.zeros((nq, 3), np.float32)
    hit = np.zeros(nq, np.int32)
    for q in range(nq):
        a, b = np.zeros(3, np.float32), np.zeros(3, np.float32)
        hit[q] = L.ref_grid_collision(g, np.ascontiguousarray(cur[q]), np.ascontiguousarray(nxt[q]),
                                      np.ascontiguousarray(vel[q]), a, b)
        cp[q], nr[q] = a, b
    L.ref_grid_free(g)
    print("collision hits:", int(hit.sum()), "of", nq)
    save("ref_collision.npz", hmap=hm, dims=np.array(dims, np.int32), cur=cur, next=nxt, vel=vel, contact=cp,
         normal=nr, hit=hit)


def main(ref_root):
    assert O.build_ref(ref_root), "reference harness did not build"

    # 1. The reference's own default scene: Initialize(1000), dt = 0.01
    #    (the value the F key sets, Erosion/main.cpp:476-485).
    R = O.Reference()
    R.initialize(1000)
    pos0 = R.get()[0][:, 0:3].copy()
    R.close()
    dflt = dict(O.REFERENCE_DEFAULTS, dt=0.01)
    res = run_ref(dflt, pos0, [1, 10, 50])
    save("ref_default_1000.npz", pos0=pos0,
         rec1=res[1][0], nb1=res[1][1], cnt1=res[1][2].astype(np.int16),
         rec10=res[10][0], nb10=res[10][1],
         pos50=res[50][0][:, 0:6], nb50=res[50][1])

    # 2. Plain-small layout at reduced size: 16 x 8 x 16 = 2048 particles,
    #    no terrain (the reference has none), 1 and 100 steps.
    s = W.SPACING
    pos = W.lattice_block(16, 8, 16, s, (-0.5 + s / 2, -0.28, -0.5 + s / 2))
    res = run_ref(C1_REF, pos, [1, 100])
    save("ref_c1_2048.npz", pos0=pos, rec1=res[1][0], nb1=res[1][1], cnt1=res[1][2].astype(np.int16),
         rec100=res[100][0], nb100=res[100][1], cnt100=res[100][2].astype(np.int16))

    # 3. The full 16,384-particle plain-small block.
    c1_16384_fixture()

    # 4. Edge cases: coincident particles (AddParticles at the same origin,
    #    fluid_system.h:232-251), a lone particle in free fall, particles
    #    placed outside each box face, and an empty step.
    R = O.Reference()
    R.set_params(**dflt)
    R.initialize(27)
    R.add_particles(8)
    R.add_particles(8)
    coinc0 = R.get()[0][:, 0:3].copy()
    R.run(1)
    rc1, _, nbc1 = R.get()
    R.run(4)
    rc5, _, nbc5 = R.get()
    R.close()
    lone = np.array([[0.01, 0.05, -0.02]], np.float32)
    rl = run_ref(dflt, lone, [1, 3])
    walls = np.array([[0.25, 0.0, 0.0], [-0.21, 0.05, 0.0], [0.0, 0.23, 0.01], [0.0, -0.3, 0.0],
                      [0.02, 0.0, 0.205], [0.0, 0.01, -0.26], [0.21, 0.21, 0.0], [0.3, 0.3, 0.3]], np.float32)
    wv = np.array([[1.0, 0.0, 0.0], [-1.0, 0.5, 0.0], [0.0, 2.0, 0.0], [0.1, -3.0, 0.0],
                   [0.0, 0.0, 1.0], [0.0, 0.0, -2.0], [1.0, 1.0, 0.0], [0.5, 0.5, 0.5]], np.float32)
    rw = run_ref(dflt, walls, [1], vel=wv)
    save("ref_edge.npz", coinc0=coinc0, coinc_rec1=rc1, coinc_nb1=nbc1, coinc_rec5=rc5, coinc_nb5=nbc5,
         lone0=lone, lone_rec1=rl[1][0], lone_rec3=rl[3][0], walls0=walls, walls_vel0=wv, walls_rec1=rw[1][0])

    # 5. Terrain surface mesh of Grid::UpdateGrid on a seeded 8-bit map at
    #    the dims the front end uses (Grid(50,255,50), main.cpp:100-105).
    rng = np.random.default_rng(7)
    hm = (O.fbm(7, 512, 512, 4, 200.0) + rng.uniform(0, 20, (512, 512))).astype(np.uint8)
    import ctypes as C
    L = O.Reference().L
    g = L.ref_grid_new(50, 255, 50)
    L.ref_grid_load(g, np.ascontiguousarray(hm.ravel()))
    L.ref_grid_update(g, 50, 255, 50)
    ns, ni = L.ref_grid_surface_size(g), L.ref_grid_indices_size(g)
    surf = np.zeros(ns, np.float32)
    idx = np.zeros(ni, np.uint32)
    L.ref_grid_surface(g, surf)
    L.ref_grid_indices(g, idx)
    L.ref_grid_free(g)
    save("ref_mesh.npz", hmap=hm, dims=np.array([50, 255, 50], np.int32), surface=surf, indices=idx)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if "--c1-16384-only" in sys.argv:
        O.build_ref(args[0] if args else "/root/reference")
        c1_16384_fixture()
        fp64_fixture()
        sys.exit(0)
    if "--collision-only" in sys.argv:
        O.build_ref(args[0] if args else "/root/reference")
        collision_fixture()
        sys.exit(0)
    if "--fp64-only" not in sys.argv:
        main(args[0] if args else "/root/reference")
        collision_fixture()
    fp64_fixture()
