"""The allocation-free extrapolation entry point, called through the C ABI on device
buffers, against the allocating entry point ffgpu_extrapolate (bit-identical results),
on two calls in a row so that scratch left behind by the first call cannot leak into the
second.  Collected last on purpose: a failure here leaves every other test already run."""
import ctypes

import numpy as np
import pytest

import gpu_api as G
import oracle_api as O
from ffengine_gb300 import load_library, scenes

pytestmark = pytest.mark.gpu


def _noalloc(grid_dev, valid_dev, shape, layers, stream_ptr):
    d, h, w = shape
    f = load_library().ffgpu_extrapolate_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_void_p]
    f.restype = None
    err = ctypes.c_int(1)
    f(w, h, d, grid_dev.data_ptr(), valid_dev.data_ptr(), layers, stream_ptr, ctypes.byref(err))
    if not err.value:
        m = load_library().CBindings_get_error_message
        m.restype = ctypes.c_char_p
        raise RuntimeError(m().decode())


def _case(n, seed):
    pos, vel = scenes.dam_break_particles(n, 0.5, 0.6, seed=seed, velocity_sigma=1.0)
    (u, vu), _, _ = O.p2g(n, 1.0 / n, pos, vel)
    return u, vu


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    layers = O.layers(5)
    for n, seed in ((24, 0), (40, 1)):            # two calls in a row, different sizes and data
        u, vu = _case(n, seed)
        ref = G.extrapolate(u, vu, layers)
        gd = torch.from_numpy(np.ascontiguousarray(u)).cuda()
        vd = torch.from_numpy(np.ascontiguousarray(vu)).cuda()
        torch.cuda.synchronize()
        _noalloc(gd, vd, u.shape, layers, stream.cuda_stream)
        stream.synchronize()
        got = gd.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_noalloc_rejects_grids_over_the_limit():
    torch = pytest.importorskip("torch")
    g = torch.zeros(8, device="cuda")
    v = torch.zeros(8, dtype=torch.uint8, device="cuda")
    with pytest.raises(RuntimeError, match="at most 4194304 cells"):
        _noalloc(g, v, (256, 128, 129), 3, None)
