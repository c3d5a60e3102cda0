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


FRAME_LOOP_C = r"""
#include <stddef.h>
#include "sph_erosion.h"
static void draw_instances(const float* p, int n) { (void)p; (void)n; }
int frame_loop(int running) {
    sph_system_config cfg; sph_system_config_default(&cfg);
    sph_system* sys; if (sph_system_create(&cfg, &sys) != SPH_OK) return 1;
    sph_params prm; sph_params_default(&prm);
    prm.dt = 0.01f;
    int sc; sph_scene_create(sys, &prm, 1000, 0, 0, &sc);
    float origin[3] = {0, 0, 0}; int added;
    sph_scene_add_lattice(sys, sc, 1000, origin, &added);
    float* pos[2];
    sph_host_alloc((int64_t)added * 12, (void**)&pos[0]);
    sph_host_alloc((int64_t)added * 12, (void**)&pos[1]);
    for (int frame = 0; frame < running; ++frame) {
        sph_scene_set_params(sys, sc, &prm);
        sph_system_step(sys, 1);
        sph_scene_get_particles_async(sys, sc, pos[frame & 1], NULL, NULL, NULL);
        sph_system_sync(sys);
        draw_instances(pos[frame & 1], added);
    }
    sph_host_free(pos[0]); sph_host_free(pos[1]);
    return sph_system_destroy(sys);
}
int main(void) { return 0; }  /* linked, not run: frame_loop needs a GPU */
"""


def test_frame_loop_example_compiles_as_c_and_links(built_lib, tmp_path):
    """The per-frame loop shown for front ends compiles as C99 against the
    header and links against the library."""
    src = tmp_path / "loop.c"
    src.write_text(FRAME_LOOP_C)
    exe = tmp_path / "loop"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", f"-I{ROOT}/include", str(src), "-o", str(exe),
                        f"-L{PKG}", "-lsph_gb300", f"-Wl,-rpath,{PKG}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


SERVER_LOOP_C = r"""
#include <stddef.h>
#include <stdio.h>
#include "sph_erosion.h"
static void report(const char* msg) { fprintf(stderr, "%s\n", msg); }
static void deliver(const sph_result* r) { (void)r; }
int serve_one(void) {
    sph_server_config scfg; sph_server_config_default(&scfg);
    scfg.hbm_budget = (int64_t)120 << 30;
    scfg.policy = 1;
    sph_server* srv; if (sph_server_create(&scfg, &srv) != SPH_OK) return 1;
    sph_request r = {0};
    r.seed = 42; r.particles = 65536; r.terrain_side = 256; r.steps = 500;
    int64_t ticket;
    if (sph_server_submit(srv, &r, &ticket) != SPH_OK)
        report(sph_last_error());
    sph_result out[64]; int n, active;
    do {
        sph_server_poll(srv, out, 64, &n, &active);
        for (int i = 0; i < n; ++i)
            if (out[i].status == SPH_OK) deliver(&out[i]);
    } while (active > 0);
    return sph_server_destroy(srv);
}
int main(void) { return 0; }  /* linked, not run: serving needs a GPU */
"""


def test_server_example_compiles_as_c_and_links(built_lib, tmp_path):
    """The serving loop shown for C callers compiles as C99 against the
    header and links against the library."""
    src = tmp_path / "serve.c"
    src.write_text(SERVER_LOOP_C)
    exe = tmp_path / "serve"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", f"-I{ROOT}/include", str(src), "-o", str(exe),
                        f"-L{PKG}", "-lsph_gb300", f"-Wl,-rpath,{PKG}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_ctypes_mirrors_match_the_header_layout(tmp_path):
    """Every public struct's size and field offsets, as the C compiler lays
    them out from include/sph_erosion.h, equal the Python binding's ctypes
    mirrors."""
    import sph_gb300 as S

    pairs = {"sph_params": S.Params, "sph_particle": S.Particle, "sph_diag": S.Diag,
             "sph_system_config": S.SystemConfig, "sph_tune_result": S.TuneResult, "sph_request": S.Request,
             "sph_server_config": S.ServerConfig, "sph_result": S.Result, "sph_server_stats": S.ServerStats}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "sph_erosion.h"', "int main(void) {"]
    want = []
    for cname, cls in pairs.items():
        lines.append(f'    printf("%zu\\n", sizeof({cname}));')
        want.append(C.sizeof(cls))
        for fname, *_ in cls._fields_:
            lines.append(f'    printf("%zu\\n", offsetof({cname}, {fname}));')
            want.append(getattr(cls, fname).offset)
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", f"-I{ROOT}/include", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == want
