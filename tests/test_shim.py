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


def _build(tmp_path):
    import build

    lib = build.build()
    exe = str(tmp_path / "shim_main")
    cmd = ["g++", "-std=c++17", "-O2", "-DSPH_SHIM_NO_GLM", f"-I{ROOT}/include", f"-I{PKG}/host", SRC, "-o", exe,
           f"-L{PKG}", "-lsph_gb300", f"-Wl,-rpath,{PKG}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    assert os.path.exists(lib)
    return exe


def test_shim_compiles_and_links(tmp_path):
    exe = _build(tmp_path)
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
