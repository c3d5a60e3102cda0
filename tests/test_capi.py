"""CPU tests of the C-ABI boundary: the library loads without a GPU and
exports exactly what include/sph_erosion.h declares.  No compute call is
made here."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import PKG, ROOT


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"SPH_API\s+[\w\s\*]+?\b(sph_\w+)\s*\(", txt))
    return names


@pytest.fixture(scope="module")
def built_lib():
    import sph_gb300 as S

    if not os.path.exists(S.LIB_PATH):
        import build

        build.build()
    return S


def test_header_declares_entry_points():
    names = _declared()
    for must in ("sph_system_create", "sph_system_step", "sph_scene_create", "sph_scene_set_particles",
                 "sph_scene_add_lattice", "sph_scene_get_particle", "sph_scene_diag", "sph_scene_set_terrain"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    declared = _declared()
    assert declared <= exported, declared - exported
    # nothing else leaks out under the sph_ prefix
    assert {e for e in exported if e.startswith("sph_")} == declared


def test_library_loads_and_binds(built_lib):
    L = built_lib.lib()
    for name in _declared():
        assert hasattr(L, name)


def test_param_defaults_are_reference_members(built_lib):
    p = built_lib.default_params()
    assert tuple(p.gravity) == pytest.approx((0.0, -9.82, 0.0))
    assert p.dt == 0.0
    assert p.rest_density == pytest.approx(998.29)
    assert p.mass == pytest.approx(0.02)
    assert p.viscosity == pytest.approx(3.5)
    assert p.surface_tension == pytest.approx(0.0728)
    assert p.gas_stiffness == pytest.approx(3.0)
    assert p.smoothing_radius == pytest.approx(0.0457)
    assert tuple(p.box_half) == pytest.approx((0.2, 0.2, 0.2))


def test_errors_are_status_codes(built_lib):
    L = built_lib.lib()
    assert L.sph_system_step(None, 1) == -1
    assert b"null" in L.sph_last_error()
    assert L.sph_scene_create(None, None, 0, 0, 0, None) == -1
