"""The allocation-free density pass, sph_density_static, through the C ABI.

It exists for callers that cannot allocate device memory (an application
owning the GPU through its own pool, a real-time loop that cannot take
cudaMalloc's implicit synchronisation, a plugin where allocation is not
allowed): its scratch is a fixed device array inside the library.  Here it
must give the same densities and pressures as the ordinary path (a scene
stepped once, whose step computes pass 1 from the same positions), on two
calls in a row that reuse the shared array.  The test owns the device
buffers (allocated through torch), as such a caller would.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import sph_gb300 as S
from helpers import C1, RTOL

pytestmark = pytest.mark.gpu


def _scene_density(params, pos):
    with S.System(particle_capacity=len(pos)) as sysm:
        sc = sysm.scene(params)
        sc.set_particles(pos)
        sysm.step(1)  # the step's pass 1 reads the initial positions
        return sc.get_particles()["density"]


def _static_density(params, pos):
    import torch  # the caller-side buffers: a GPU run without torch fails here instead of skipping
    dev_pos = torch.from_numpy(np.ascontiguousarray(pos, np.float32).ravel()).cuda()
    dens = torch.full((len(pos),), -1.0, dtype=torch.float32, device="cuda")
    pres = torch.full((len(pos),), -1.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = S.lib().sph_density_static(C.byref(params), len(pos), C.c_void_p(dev_pos.data_ptr()),
                                    C.c_void_p(dens.data_ptr()), C.c_void_p(pres.data_ptr()), C.c_void_p(stream))
    assert rc == 0, S.lib().sph_last_error().decode()
    return dens.cpu().numpy(), pres.cpu().numpy()


def test_static_density_matches_scene_path_twice(golden):
    g = golden("ref_c1_2048.npz")
    params = S.default_params(**C1)
    first = golden("ref_c1_16384.npz")["pos0"]
    second = g["rec100"][:, 0:3]  # a different (compressed) set on the second call
    for pos in (first, second):
        want = _scene_density(params, pos)
        got, pres = _static_density(params, pos)
        err = np.abs(got.astype(np.float64) - want).max() / np.abs(want).max()
        assert err <= RTOL, err
        assert np.array_equal(got, want)  # same kernels, same order: identical bits
        k = np.float32(C1["gas_stiffness"])
        assert np.array_equal(pres, k * (got - np.float32(C1["rest_density"])))


def test_static_density_rejects_oversize():
    """Sizes beyond the fixed scratch fail with a clear error before any
    device access (the pointers are never touched)."""
    params = S.default_params(**C1)
    n = 32768 + 1
    assert S.lib().sph_density_static(C.byref(params), n, C.c_void_p(1), C.c_void_p(1), None, None) == -4
    assert b"exceed" in S.lib().sph_last_error()
    big = S.default_params(**dict(C1, box_half=(2.0, 2.0, 2.0)))  # 100^3 cells: 1.6M keys
    assert S.lib().sph_density_static(C.byref(big), 10, C.c_void_p(1), C.c_void_p(1), None, None) == -4
    assert b"keys" in S.lib().sph_last_error()


def test_static_density_refuses_a_capturing_stream():
    """Every call ends by synchronising its stream, which a stream being
    captured into a CUDA graph cannot do: on such a stream the call returns
    SPH_ERR_INVALID before touching it, and the capture stays usable."""
    import torch

    params = S.default_params(**C1)
    pos = torch.zeros(30, dtype=torch.float32, device="cuda")
    dens = torch.zeros(10, dtype=torch.float32, device="cuda")
    x = torch.zeros(1, dtype=torch.float32, device="cuda")
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side):
        x.add_(1.0)
        rc = S.lib().sph_density_static(C.byref(params), 10, C.c_void_p(pos.data_ptr()), C.c_void_p(dens.data_ptr()),
                                        None, C.c_void_p(side.cuda_stream))
    assert rc == -1
    assert b"captured" in S.lib().sph_last_error()
    graph.replay()
    torch.cuda.synchronize()
    assert x.item() == 1.0
