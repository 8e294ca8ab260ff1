"""The `load` scene command (muon/parser.cc:465-561): a mesh file read from
the scene file's directory adds vertices, and triangles under the current
material and transform, exactly like the same mesh written inline with
start_mesh / vertex / tri. Every supported format (PLY ascii and binary in
both byte orders, STL ascii and binary, OBJ) must give the same triangles."""
import struct

import numpy as np
import pytest

import muon_gb300 as m
from muon_gb300 import scenes

HEADER = """camera 0 0 5  0 0 0  0 1 0  45
film_size 32 32
integrator normals
diffuse 0.5 0.4 0.3
push_transform
translate 0.1 0.2 0.3
scale 1.5 1.5 1.5
"""


def mesh():
    V, F = scenes.icosphere(1)
    return V.astype(np.float32), F.astype(np.int32)


def write_ply_ascii(path, V, F):
    with open(path, "w") as f:
        f.write(f"ply\nformat ascii 1.0\nelement vertex {len(V)}\nproperty float x\nproperty float y\n"
                f"property float z\nproperty float nx\nelement face {len(F)}\n"
                "property list uchar int vertex_indices\nend_header\n")
        for v in V:
            f.write(" ".join(format(float(x), ".9g") for x in v) + " 0\n")
        for t in F:
            f.write("3 %d %d %d\n" % tuple(t))


def write_ply_binary(path, V, F, big):
    e = ">" if big else "<"
    with open(path, "wb") as f:
        f.write((f"ply\nformat binary_{'big' if big else 'little'}_endian 1.0\nelement vertex {len(V)}\n"
                 "property float x\nproperty float y\nproperty float z\nelement face {0}\n"
                 "property list uchar int vertex_indices\nend_header\n").replace("{0}", str(len(F))).encode())
        for v in V:
            f.write(struct.pack(e + "3f", *v))
        for t in F:
            f.write(struct.pack(e + "B3i", 3, *t))


def write_stl_binary(path, V, F):
    with open(path, "wb") as f:
        f.write(b"\0" * 80 + struct.pack("<I", len(F)))
        for t in F:
            f.write(struct.pack("<3f", 0, 0, 0))
            for k in t:
                f.write(struct.pack("<3f", *V[k]))
            f.write(b"\0\0")


def write_stl_ascii(path, V, F):
    with open(path, "w") as f:
        f.write("solid s\n")
        for t in F:
            f.write(" facet normal 0 0 0\n  outer loop\n")
            for k in t:
                f.write("   vertex " + " ".join(format(float(x), ".9g") for x in V[k]) + "\n")
            f.write("  endloop\n endfacet\n")
        f.write("endsolid s\n")


def write_obj(path, V, F):
    with open(path, "w") as f:
        for v in V:
            f.write("v " + " ".join(format(float(x), ".9g") for x in v) + "\n")
        for t in F:
            f.write("f %d/1/1 %d//2 %d\n" % tuple(t + 1))


def triangles(text, base):
    p = m.parse_string(text, base)
    d = p.desc
    n = d.num_triangles
    out = [(tuple(tuple(r) for r in d.triangles[i].v), tuple(tuple(r) for r in d.triangles[i].n),
            d.triangles[i].transform, d.triangles[i].material, d.triangles[i].smooth) for i in range(n)]
    return out, p.warnings


def inline_text(V, F, smooth):
    lines = [HEADER, f"compute_vertex_normals {'on' if smooth else 'off'}", "start_mesh"]
    lines += ["vertex " + " ".join(format(float(x), ".9g") for x in v) for v in V]
    lines += ["tri %d %d %d" % tuple(t) for t in F]
    lines += ["end_mesh", "pop_transform"]
    return "\n".join(lines) + "\n"


WRITERS = {"ascii.ply": write_ply_ascii, "le.ply": lambda p, V, F: write_ply_binary(p, V, F, False),
           "be.ply": lambda p, V, F: write_ply_binary(p, V, F, True), "bin.stl": write_stl_binary,
           "ascii.stl": write_stl_ascii, "mesh.obj": write_obj}


@pytest.mark.parametrize("name", sorted(WRITERS))
@pytest.mark.parametrize("smooth", [False, True])
def test_load_equals_inline_mesh(lib, tmp_path, name, smooth):
    V, F = mesh()
    WRITERS[name](str(tmp_path / name), V, F)
    text = HEADER + f"compute_vertex_normals {'on' if smooth else 'off'}\nload {name}\npop_transform\n"
    got, warn = triangles(text, str(tmp_path))
    want, _ = triangles(inline_text(V, F, smooth), str(tmp_path))
    assert warn == 0
    assert len(got) == len(F)
    assert got == want


def test_missing_or_malformed_file_is_skipped_with_a_warning(lib, tmp_path):
    (tmp_path / "bad.ply").write_text("ply\nformat ascii 1.0\nelement vertex 1\nproperty float x\nend_header\n1\n")
    (tmp_path / "oob.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 9\n")
    for f in ("missing.ply", "bad.ply", "oob.obj", "mesh.xyz"):
        got, warn = triangles(HEADER + f"load {f}\n", str(tmp_path))
        assert got == [] and warn == 1
