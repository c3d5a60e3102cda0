"""The C++ drop-in (FluidSystemSPH and Grid over the C ABI).

CPU: the front-end-style program compiles and links against the library.
GPU: it runs like the reference's front end and its records, mesh and
counts match the reference's golden vectors (fast mode within RTOL after 1
and 10 steps; ordered mode bit for bit after the first step; the mesh bit
for bit).
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG, ROOT
from helpers import RTOL, field_errors

SRC = os.path.join(ROOT, "tests", "shim", "shim_main.cpp")


SRC_EROSION = os.path.join(ROOT, "tests", "shim", "shim_erosion.cpp")
GLM = "/root/reference/vendor/glm"


def _build(tmp_path, src=SRC, glm=None):
    import build

    lib = build.build()
    exe = str(tmp_path / (os.path.splitext(os.path.basename(src))[0] + ("_glm" if glm else "")))
    flags = [f"-I{glm}"] if glm else ["-DSPH_SHIM_NO_GLM"]
    cmd = ["g++", "-std=c++17", "-O2", *flags, f"-I{ROOT}/include", f"-I{PKG}/host", src, "-o", exe,
           f"-L{PKG}", "-lsph_gb300", f"-Wl,-rpath,{PKG}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert os.path.exists(lib)
    return exe


def test_shim_compiles_and_links(tmp_path):
    for src in (SRC, SRC_EROSION):
        exe = _build(tmp_path, src)
        assert os.access(exe, os.X_OK)


def test_shim_compiles_against_glm(tmp_path):
    """With the reference's own glm the drop-in's vector type is glm::vec3,
    so the front end's `glm::vec3* gr = fluidsph.GetGrav();`
    (Erosion/main.cpp:283) and `SetOrigin(glm::vec3(0.0))` (:170) compile
    unchanged."""
    if not os.path.isdir(GLM):
        pytest.skip("the reference's glm is not present here")
    exe = _build(tmp_path, SRC, glm=GLM)
    assert os.access(exe, os.X_OK)
    exe = _build(tmp_path, SRC_EROSION, glm=GLM)
    assert os.access(exe, os.X_OK)


def _read(path):
    b = open(path, "rb").read()
    off = 0

    def take(dt, n):
        nonlocal off
        a = np.frombuffer(b, dt, n, off)
        off += a.nbytes
        return a

    out = {}
    for tag in ("s1", "s10"):
        n = int(take(np.int32, 1)[0])
        raw = take(np.uint8, n * 28 * 4).reshape(n, 28 * 4)
        out[tag] = raw[:, :108].copy().view(np.float32).reshape(n, 27), raw[:, 108:].copy().view(np.int32).ravel()
    ns = int(take(np.int32, 1)[0])
    out["surface"] = take(np.float32, ns).copy()
    ni = int(take(np.int32, 1)[0])
    out["indices"] = take(np.uint32, ni).copy()
    out["count"] = int(take(np.int32, 1)[0])
    if off < len(b):
        nq = int(take(np.int32, 1)[0])
        raw = take(np.uint8, nq * 28).reshape(nq, 28)
        out["hit"] = raw[:, :4].copy().view(np.int32).ravel()
        out["contact_normal"] = raw[:, 4:].copy().view(np.float32).reshape(nq, 6)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("ordered", [False, True])
def test_shim_front_end_session_matches_reference(tmp_path, golden, ordered):
    exe = _build(tmp_path)
    g = golden("ref_default_1000.npz")
    m = golden("ref_mesh.npz")
    hm = tmp_path / "hm.bin"
    hm.write_bytes(np.ascontiguousarray(m["hmap"], np.uint8).tobytes())
    out = tmp_path / "out.bin"
    # Grid::collision through the drop-in, one call per query, on a slice of
    # the reference's collision vectors
    c = golden("ref_collision.npz")
    cm = tmp_path / "cm.bin"
    cm.write_bytes(np.ascontiguousarray(c["hmap"], np.uint8).tobytes())
    nq = 600
    q = np.concatenate([c["cur"][:nq], c["next"][:nq], c["vel"][:nq]], axis=1).astype(np.float32)
    qf = tmp_path / "q.bin"
    qf.write_bytes(np.array([c["dims"][0], c["dims"][2], nq], np.int32).tobytes() + q.tobytes())
    args = [exe, str(out), str(hm), "ordered" if ordered else "fast", str(cm), str(qf)]
    subprocess.run(args, check=True, timeout=120)
    r = _read(str(out))
    rec1, nb1 = r["s1"]
    rec10, nb10 = r["s10"]
    if ordered:
        assert np.array_equal(rec1, g["rec1"])
    assert max(field_errors(rec1, g["rec1"]).values()) <= RTOL
    assert max(field_errors(rec10, g["rec10"]).values()) <= RTOL
    assert np.array_equal(nb1, g["nb1"]) and np.array_equal(nb10, g["nb10"])
    assert np.array_equal(r["surface"], m["surface"])
    assert np.array_equal(r["indices"], m["indices"])
    assert r["count"] == 1000 + 125
    assert np.array_equal(r["hit"], c["hit"][:nq])
    want = np.concatenate([c["contact"][:nq], c["normal"][:nq]], axis=1)
    assert np.array_equal(r["contact_normal"].view(np.uint32), want.view(np.uint32))


def _read_erosion(path):
    b = open(path, "rb").read()
    off = 0

    def take(dt, n):
        nonlocal off
        a = np.frombuffer(b, dt, n, off)
        off += a.nbytes
        return a

    out = {}
    for k, dt in (("s0", np.float32), ("s1", np.float32), ("i0", np.uint32), ("i1", np.uint32)):
        n = int(take(np.int32, 1)[0])
        out[k] = take(dt, n).copy()
    out["total"], out["sediment"] = (int(x) for x in take(np.int64, 2))
    out["n"], out["nan"], out["mat"] = (int(x) for x in take(np.int32, 3))
    return out


@pytest.mark.gpu
def test_shim_erodes_the_front_ends_grid(tmp_path, golden):
    """The drop-in with the terrain coupling on, driven like the front end
    (Grid(dimX, 255, dimZ) + LoadHeightfield + UpdateGrid, FluidSystemSPH
    Initialize + Run(grid)): after 200 steps the grid's surface mesh, from
    the same UpdateGrid / GetSurfaceParts calls, is the eroded terrain: its
    heights changed where the fluid flowed, its x and z and indices did not,
    sediment + terrain units are conserved exactly and sediment is carried."""
    exe = _build(tmp_path, SRC_EROSION)
    m = golden("ref_mesh.npz")
    hm = tmp_path / "hm.bin"
    hm.write_bytes(np.ascontiguousarray(m["hmap"], np.uint8).tobytes())
    out = tmp_path / "out.bin"
    subprocess.run([exe, str(out), str(hm), "200"], check=True, timeout=120)
    r = _read_erosion(str(out))
    s0, s1 = r["s0"].reshape(-1, 6), r["s1"].reshape(-1, 6)
    assert len(s0) == 48 * 40 and np.array_equal(r["i0"], r["i1"])
    assert np.array_equal(s0[:, [0, 2]], s1[:, [0, 2]])  # same vertices along x and z
    dh = s1[:, 1] - s0[:, 1]
    assert np.isfinite(s1).all()
    # the uneroded heights come back to within float rounding of the grey
    # levels; erosion moves them by whole fractions of a level
    print("eroded vertices", int((np.abs(dh) > 1e-2).sum()), "min/max change", dh.min(), dh.max())
    assert (np.abs(dh) > 1e-2).sum() > 10, "the surface did not change"
    assert dh.min() < -1e-2  # eroded somewhere
    assert r["total"] == 0 and r["sediment"] > 0
    assert r["n"] == 1000 and r["nan"] == 0
    assert r["mat"] == 48 * 40  # UpdateGrid marks the eroded surface voxels
