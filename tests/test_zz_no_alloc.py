"""The no-allocation render entry point (muon_gpu_render_noalloc).

It exists for callers that may not allocate device memory while rendering —
an application whose own allocator holds the GPU's memory, or a real-time
loop that allocates nothing after start-up. It must produce the film that
muon_gpu_render_device produces for the same scene and settings, on repeated
calls, using only its fixed static buffer. This file is collected last on
purpose.
"""
import ctypes as C

import numpy as np
import pytest

import muon_gb300 as m
from conftest import GOLDEN
from muon_gb300 import native
from muon_gb300.native import check, load


def _device_film(h, w):
    torch = pytest.importorskip("torch")
    return (torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
            torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
            torch.zeros((h, w), dtype=torch.int32, device="cuda"))


def _render(fn, scene, params, film):
    s, q, n = film
    check(fn(scene._h, C.byref(params), C.c_void_p(s.data_ptr()), C.c_void_p(q.data_ptr()),
             C.c_void_p(n.data_ptr())))
    return s.cpu().numpy(), q.cpu().numpy(), n.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["pathtracer", "normals"])
def test_noalloc_render_matches_the_allocating_entry_point(lib, integrator):
    fx = np.load(f"{GOLDEN}/pt_cornell.npz")
    scene = m.Scene.from_string(str(fx["scene"]))
    h, w = scene.height, scene.width
    params = scene.params(integrator=integrator, pixel_samples=64, seed=11)
    ref = _render(load().muon_gpu_render_device, scene, params, _device_film(h, w))
    for _ in range(2):  # two calls in a row share the static buffer
        got = _render(load().muon_gpu_render_noalloc, scene, params, _device_film(h, w))
        assert np.array_equal(got[2], ref[2])
        assert np.allclose(got[0], ref[0], rtol=1e-12, atol=0)
        assert np.allclose(got[1], ref[1], rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_noalloc_render_leaves_free_device_memory_unchanged(lib):
    """The property the entry point exists for: once the scene exists (its
    creation placed the static buffer on the device) and the kernels have
    run once, rendering through it changes the device's free memory by
    nothing, on the first call and on the next."""
    torch = pytest.importorskip("torch")
    fx = np.load(f"{GOLDEN}/pt_cornell.npz")
    scene = m.Scene.from_string(str(fx["scene"]))
    h, w = scene.height, scene.width
    params = scene.params(pixel_samples=16, seed=5)
    films = [_device_film(h, w) for _ in range(3)]
    # loads the rendering kernels (the allocating entry point, its own film)
    _render(load().muon_gpu_render_device, scene, params, films[0])
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    fn = load().muon_gpu_render_noalloc
    for s, q, n in films[1:]:
        check(fn(scene._h, C.byref(params), C.c_void_p(s.data_ptr()), C.c_void_p(q.data_ptr()),
                 C.c_void_p(n.data_ptr())))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    assert torch.equal(films[1][2], films[0][2]) and torch.equal(films[2][2], films[0][2])
    assert torch.allclose(films[1][0], films[0][0], rtol=1e-12, atol=0)
    assert torch.allclose(films[2][0], films[0][0], rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_noalloc_rejects_waves_beyond_its_buffer(lib):
    fx = np.load(f"{GOLDEN}/pt_cornell.npz")
    scene = m.Scene.from_string(str(fx["scene"]))
    params = scene.params(pixel_samples=4, wave_paths=native.NOALLOC_SCRATCH_BYTES)
    film = _device_film(scene.height, scene.width)
    with pytest.raises(m.MuonError) as e:
        _render(load().muon_gpu_render_noalloc, scene, params, film)
    assert e.value.code == 1 and "scratch" in str(e.value)
