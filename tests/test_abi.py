"""The C ABI library builds, loads and exports every declared entry point."""
import re

from conftest import ROOT


def _declared_functions():
    text = open(f"{ROOT}/include/muon_gpu.h").read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(muon_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = _declared_functions()
    for required in ["muon_gpu_scene_create", "muon_gpu_render", "muon_gpu_intersect", "muon_gpu_occluded",
                     "muon_gpu_stats", "muon_gpu_scene_destroy", "muon_gpu_last_error", "muon_parse_scene_file"]:
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    from muon_gb300 import native

    for name in _declared_functions():
        assert hasattr(lib, name), name
        assert name in native.SIGNATURES, f"{name} missing from the ctypes signatures"


def test_errors_are_status_codes(lib):
    import ctypes as C

    from muon_gb300 import native

    h = C.c_void_p()
    rc = lib.muon_parse_scene_file(b"/nonexistent/scene.muon", C.byref(h))
    assert rc == 5
    assert b"cannot open" in lib.muon_gpu_last_error()
    assert lib.muon_gpu_scene_create(None, C.byref(h)) == 1
    assert lib.muon_gpu_render(None, None, None) == 1
    assert lib.muon_gpu_stats(None, None) == 1
    assert native.MUON_OK == 0


def test_guide_and_cache_entry_points_without_a_device(lib):
    """Null handles are argument errors (no device needed), and releasing the
    work-array cache is safe when nothing was ever cached."""
    import ctypes as C

    assert lib.muon_gpu_guide_create(None, None, C.byref(C.c_void_p())) == 1
    assert lib.muon_gpu_guide_sample(None, None, None, 4, None, None) == 1
    assert lib.muon_gpu_guide_forward(None, None, 4, None) == 1
    assert lib.muon_gpu_guide_train(None, 1, None) == 1
    lib.muon_gpu_release_cached()


def test_scene_without_camera_is_a_parse_error(lib):
    import pytest

    import muon_gb300 as m

    with pytest.raises(m.MuonError) as e:
        m.parse_string("film_size 4 4\nsphere 0 0 0 1\n")
    assert e.value.code == 5


def test_header_compiles_and_links_as_c(lib, tmp_path):
    """include/muon_gpu.h is a C ABI: a C99 program includes it, links
    against libmuon_gpu.so and runs the host-only parsing calls."""
    import os
    import shutil
    import subprocess

    if shutil.which("gcc") is None:
        import pytest
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.join(root, "muon_gb300", "lib")
    src = tmp_path / "t.c"
    src.write_text(r"""
#include <stdio.h>
#include <string.h>
#include "muon_gpu.h"
int main(void) {
  const char *text = "film_size 8 4\nintegrator pathtracer\ncamera 0 0 5  0 0 0  0 1 0  45\n"
                     "quad_light -1 3 -1  0 0 2  2 0 0  5 5 5\nsphere 0 0 0 1\n";
  MuonParsedScene *ps = NULL;
  MuonSceneDesc desc;
  MuonRenderParams params;
  if (muon_parse_scene_string(text, ".", &ps) != MUON_OK) return 1;
  if (muon_parsed_scene_desc(ps, &desc, &params) != MUON_OK) return 2;
  if (desc.width != 8 || desc.height != 4 || desc.num_spheres != 1 || desc.num_lights != 1) return 3;
  if (params.integrator != MUON_INTEGRATOR_PATHTRACER) return 4;
  muon_parsed_scene_free(ps);
  if (muon_gpu_render(NULL, NULL, NULL) != MUON_ERR_INVALID_ARG) return 5;
  if (strlen(muon_gpu_last_error()) == 0) return 6;
  puts("ok");
  return 0;
}
""")
    exe = tmp_path / "t"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", str(src), "-I", os.path.join(root, "include"),
                    "-L", libdir, "-lmuon_gpu", "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.returncode
    assert out.stdout.strip() == "ok"
