"""Seeded synthetic scenes for the benchmark workloads, emitted as .muon text.

The same text is rendered by the GPU path and by the CPU oracle, so both see
identical input. Numbers are written with 9 significant digits, which
round-trips float32 exactly through the reference parser's `istream >> float`.

Small geometry is authored at a large object-space scale and shrunk with a
`scale` transform: the reference rejects any triangle whose object-space
unnormalised normal is shorter than 1e-4 (muon/objects.cc:104-108), which
would make small triangles authored directly invisible.
"""
from __future__ import annotations

import numpy as np


def _f(x: float) -> str:
    return format(float(np.float32(x)), ".9g")


def _v(*xs) -> str:
    return " ".join(_f(x) for x in xs)


# Unit cube vertices and outward-facing triangles (counter-clockwise seen from
# outside).
_CUBE_V = [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]
_CUBE_T = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4), (3, 7, 6), (3, 6, 2),
           (0, 4, 7), (0, 7, 3), (1, 2, 6), (1, 6, 5)]


def _cube(lines: list[str]) -> None:
    lines.append("start_mesh")
    for v in _CUBE_V:
        lines.append("vertex " + _v(*v))
    for t in _CUBE_T:
        lines.append("tri %d %d %d" % t)
    lines.append("end_mesh")


def _quad(lines: list[str], a, b, c, d) -> None:
    """Two triangles a-b-c, a-c-d (normal (b-a)x(c-a))."""
    lines.append("start_mesh")
    for v in (a, b, c, d):
        lines.append("vertex " + _v(*v))
    lines.append("tri 0 1 2")
    lines.append("tri 0 2 3")
    lines.append("end_mesh")


def cornell(width: int = 256, height: int = 256, spp: int = 16, max_depth: int = 5, seed: int = 1,
            integrator: str = "pathtracer", nee: str = "mis") -> str:
    """Cornell box: five walls of the box [-1,1]x[0,2]x[-1,1] (2 triangles each,
    facing inwards; left (0.63,0.065,0.05), right (0.14,0.45,0.09), others 0.73),
    two rotated boxes (12 triangles each, Lambertian 0.73), a 0.25x0.25 ceiling
    quad light with emission (17,12,4); pinhole camera with 40 degree FOV."""
    L = ["# Cornell box: 5 walls, 2 rotated boxes, one 0.25x0.25 ceiling light",
         f"random_seed {seed}",
         f"film_size {width} {height}",
         f"integrator {integrator}",
         f"pixel_samples {spp}",
         f"max_depth {max_depth}",
         f"next_event_estimation {nee}",
         "importance_sampling brdf",
         "russian_roulette off",
         "camera 0 1 3.9  0 1 0  0 1 0  40",
         "quad_light -0.125 1.999 -0.125  0 0 0.25  0.25 0 0  17 12 4",
         "brdf lambertian",
         "ambient 0 0 0",
         "specular 0 0 0",
         "emission 0 0 0"]
    grey = (0.73, 0.73, 0.73)
    walls = [
        ("floor", grey, (-1, 0, -1), (-1, 0, 1), (1, 0, 1), (1, 0, -1)),
        ("ceiling", grey, (-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1)),
        ("back", grey, (-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1)),
        ("left", (0.63, 0.065, 0.05), (-1, 0, -1), (-1, 2, -1), (-1, 2, 1), (-1, 0, 1)),
        ("right", (0.14, 0.45, 0.09), (1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1)),
    ]
    for name, kd, a, b, c, d in walls:
        L.append(f"# {name}")
        L.append("diffuse " + _v(*kd))
        _quad(L, a, b, c, d)
    L.append("diffuse " + _v(*grey))
    for (tx, ty, tz, ang, sx, sy, sz) in ((0.33, 0.3, 0.35, -18.0, 0.3, 0.3, 0.3),
                                          (-0.35, 0.6, -0.3, 22.0, 0.3, 0.6, 0.3)):
        L += ["push_transform", f"translate {_v(tx, ty, tz)}", f"rotate 0 1 0 {_f(ang)}", f"scale {_v(sx, sy, sz)}"]
        _cube(L)
        L.append("pop_transform")
    return "\n".join(L) + "\n"


def sphere_field(width: int = 512, height: int = 512, spp: int = 64, max_depth: int = 8, n_spheres: int = 512,
                 seed: int = 1, nee: str = "mis") -> str:
    """Random sphere field: centres U[-10,10]^3, radii U[0.2,1.0]; material
    uniform over {Lambertian albedo U[0.1,0.9]^3; Phong kd U[0,0.5]^3,
    ks U[0,0.5]^3, shininess 10^U[0,3]; GGX roughness U[0.05,0.6], F0
    U[0.02,0.9], diffuse 0}; a ground quad below the field and one 2x2 quad
    light of emission 10 above it. numpy PCG64 stream seeded with `seed`."""
    rng = np.random.default_rng(seed)
    L = ["# random sphere field",
         f"random_seed {seed}",
         f"film_size {width} {height}",
         "integrator pathtracer",
         f"pixel_samples {spp}",
         f"max_depth {max_depth}",
         f"next_event_estimation {nee}",
         "importance_sampling brdf",
         "russian_roulette off",
         "gamma 2.2",
         "camera 0 6 34  0 0 0  0 1 0  45",
         "quad_light -1 12 -1  0 0 2  2 0 0  10 10 10",
         "ambient 0 0 0",
         "emission 0 0 0",
         "brdf lambertian",
         "diffuse 0.5 0.5 0.5",
         "specular 0 0 0"]
    _quad(L, (-30, -11, -30), (-30, -11, 30), (30, -11, 30), (30, -11, -30))
    centres = rng.uniform(-10.0, 10.0, size=(n_spheres, 3))
    radii = rng.uniform(0.2, 1.0, size=n_spheres)
    kinds = rng.integers(0, 3, size=n_spheres)
    for i in range(n_spheres):
        k = kinds[i]
        if k == 0:
            L += ["brdf lambertian", "diffuse " + _v(*rng.uniform(0.1, 0.9, 3)), "specular 0 0 0"]
        elif k == 1:
            L += ["brdf phong", "diffuse " + _v(*rng.uniform(0.0, 0.5, 3)), "specular " + _v(*rng.uniform(0.0, 0.5, 3)),
                  "shininess " + _f(10.0 ** rng.uniform(0.0, 3.0))]
        else:
            f0 = rng.uniform(0.02, 0.9)
            L += ["brdf ggx", "diffuse 0 0 0", "specular " + _v(f0, f0, f0), "roughness " + _f(rng.uniform(0.05, 0.6))]
        L.append("sphere " + _v(*centres[i], radii[i]))
    return "\n".join(L) + "\n"


def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: 12 + 30 (4^level - 1) / 3 * ... vertices, 20 * 4^level
    triangles (counter-clockwise seen from outside). Returns (V float64, F int32)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    V = np.array(v, dtype=np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array(f, dtype=np.int64)
    for _ in range(level):
        # midpoint of every edge, shared between its two triangles
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (len(V) + 1) + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // (len(V) + 1), uniq % (len(V) + 1)
        mid = V[a] + V[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1).T + len(V)
        V = np.concatenate([V, mid])
        F = np.concatenate([np.stack([F[:, 0], m[:, 0], m[:, 2]], 1), np.stack([F[:, 1], m[:, 1], m[:, 0]], 1),
                            np.stack([F[:, 2], m[:, 2], m[:, 1]], 1), m])
    return V, F.astype(np.int32)


def value_noise(p: np.ndarray, seed: int, freq: float = 3.0) -> np.ndarray:
    """Seeded 3-D value noise in [-1, 1]: trilinear blend of random lattice values."""
    rng = np.random.default_rng(seed)
    lattice = rng.uniform(-1.0, 1.0, size=(64, 64, 64))
    q = (p + 2.0) * freq
    i0 = np.floor(q).astype(np.int64)
    f = q - i0
    f = f * f * (3.0 - 2.0 * f)
    out = np.zeros(len(p))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = (f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * (f[:, 2] if dz else 1 - f[:, 2])
                out += w * lattice[(i0[:, 0] + dx) % 64, (i0[:, 1] + dy) % 64, (i0[:, 2] + dz) % 64]
    return out


def _mesh(lines: list[str], V: np.ndarray, F: np.ndarray) -> None:
    lines.append("start_mesh")
    lines.extend("vertex " + _v(*v) for v in V)
    lines.extend("tri %d %d %d" % tuple(t) for t in F)
    lines.append("end_mesh")


def feature_mix(width: int = 128, height: int = 128, spp: int = 1, integrator: str = "normals",
                nee: str = "mis", max_depth: int = 5) -> str:
    """Cornell room exercising every primitive path: rotated/scaled triangles, a
    mirrored (negative-scale) box, a non-uniformly scaled sphere, a plain
    sphere, a smooth-shaded icosphere (compute_vertex_normals), Phong and GGX
    materials, two quad lights and a point light."""
    L = ["# feature coverage scene", "random_seed 7", f"film_size {width} {height}", f"integrator {integrator}",
         f"pixel_samples {spp}", f"max_depth {max_depth}", f"next_event_estimation {nee}",
         "importance_sampling brdf", "russian_roulette off", "camera 0 1 3.9  0 1 0  0 1 0  40",
         "quad_light -0.125 1.999 -0.125  0 0 0.25  0.25 0 0  17 12 4",
         "quad_light -0.99 1.2 -0.3  0 0.3 0  0 0 0.6  4 4 6",
         "point_light 0.5 1.5 0.5  1 1 1", "ambient 0 0 0", "emission 0 0 0", "brdf lambertian", "specular 0 0 0"]
    walls = [((0.73, 0.73, 0.73), (-1, 0, -1), (-1, 0, 1), (1, 0, 1), (1, 0, -1)),
             ((0.73, 0.73, 0.73), (-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1)),
             ((0.73, 0.73, 0.73), (-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1)),
             ((0.63, 0.065, 0.05), (-1, 0, -1), (-1, 2, -1), (-1, 2, 1), (-1, 0, 1)),
             ((0.14, 0.45, 0.09), (1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1))]
    for kd, a, b, c, d in walls:
        L.append("diffuse " + _v(*kd))
        _quad(L, a, b, c, d)
    L += ["brdf phong", "diffuse 0.5 0.45 0.4", "specular 0.3 0.3 0.3", "shininess 40",
          "push_transform", "translate -0.5 0.25 -0.4", "rotate 0.2 1 0.1 30", "scale 0.25 0.25 0.25"]
    _cube(L)
    L += ["pop_transform", "push_transform", "translate 0.55 0.2 -0.5", "rotate 0 1 0 -15", "scale -0.2 0.2 0.2"]
    _cube(L)
    L += ["pop_transform", "brdf ggx", "diffuse 0.1 0.1 0.1", "specular 0.8 0.6 0.3", "roughness 0.2",
          "push_transform", "translate 0.45 0.75 0.1", "rotate 1 0 1 40", "scale 0.3 0.15 0.2",
          "sphere 0 0 0 1", "pop_transform", "roughness 0.05", "specular 0.9 0.9 0.9",
          "sphere -0.45 0.9 0.25 0.22", "brdf lambertian", "diffuse 0.2 0.5 0.8", "specular 0 0 0",
          "compute_vertex_normals on", "push_transform", "translate -0.1 0.3 0.45", "scale 0.002 0.002 0.002"]
    V, F = icosphere(2)
    _mesh(L, V * 100.0, F)
    L += ["pop_transform"]
    return "\n".join(L) + "\n"


def _mesh_fast(lines: list[str], V: np.ndarray, F: np.ndarray) -> None:
    """A mesh block for large meshes (vectorised number formatting)."""
    lines.append("start_mesh")
    v32 = V.astype(np.float32)
    lines.extend("vertex " + " ".join(row) for row in np.char.mod("%.9g", v32).tolist())
    lines.extend(("tri %d %d %d" % (a, b, c)) for a, b, c in F.tolist())
    lines.append("end_mesh")


def dense_mesh(width: int = 1024, height: int = 1024, spp: int = 256, max_depth: int = 10, level: int = 8,
               clutter: int = 10000, seed: int = 1) -> str:
    """Dense mesh in the Cornell box: a subdivided icosphere (level 8:
    1,310,720 triangles) with seeded value-noise radial displacement of
    amplitude 0.1, GGX roughness 0.15, smooth vertex normals, radius 0.5 at
    (0, 0.75, 0); plus `clutter` random small triangles (edges U[0.01, 0.05])
    inside the box. Both are authored at 1000x object scale under a `scale`
    transform so that no triangle falls under the reference's 1e-4 rejection."""
    rng = np.random.default_rng(seed)
    L = cornell(width, height, spp, max_depth, seed, "pathtracer", "mis").splitlines()
    V, F = icosphere(level)
    V = V * (1.0 + 0.1 * value_noise(V, seed, freq=3.0))[:, None]
    L += ["brdf ggx", "diffuse 0.1 0.1 0.1", "specular 0.6 0.6 0.6", "roughness 0.15",
          "compute_vertex_normals on", "push_transform", "translate 0 0.75 0", "scale 0.0005 0.0005 0.0005"]
    _mesh_fast(L, V * 1000.0, F)
    L += ["pop_transform", "compute_vertex_normals off", "brdf lambertian", "specular 0 0 0",
          "diffuse 0.6 0.5 0.4", "push_transform", "scale 0.001 0.001 0.001"]
    centres = rng.uniform([-0.95, 0.05, -0.95], [0.95, 1.95, 0.95], size=(clutter, 3))
    edge = rng.uniform(0.01, 0.05, size=clutter)
    d1 = rng.normal(size=(clutter, 3))
    d1 /= np.linalg.norm(d1, axis=1, keepdims=True)
    d2 = rng.normal(size=(clutter, 3))
    d2 -= (d2 * d1).sum(1, keepdims=True) * d1
    d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
    a = centres
    b = centres + d1 * edge[:, None]
    c = centres + (0.5 * d1 + 0.866 * d2) * edge[:, None]
    CV = np.stack([a, b, c], axis=1).reshape(-1, 3) * 1000.0
    CF = np.arange(3 * clutter, dtype=np.int64).reshape(-1, 3)
    _mesh_fast(L, CV, CF)
    L.append("pop_transform")
    return "\n".join(L) + "\n"


def whitted(width: int = 128, height: int = 128, spp: int = 1, max_depth: int = 5, seed: int = 1,
            integrator: str = "raytracer", nee: str = "off") -> str:
    """Scene for the ray tracer and analytic direct lighting: 24 seeded
    spheres (every third one an ellipsoid under a push_transform), Phong
    materials with and without specular colour (mirror chains up to
    max_depth), a slightly specular ground quad, ambient terms, two attenuated
    point lights, a directional light and one quad light (a quad light adds a
    specular term in the ray tracer and is the only light analytic direct
    lighting uses)."""
    rng = np.random.default_rng(seed)
    L = ["# spheres and lights for the ray tracer",
         f"random_seed {seed}",
         f"film_size {width} {height}",
         f"integrator {integrator}",
         f"pixel_samples {spp}",
         f"max_depth {max_depth}",
         f"next_event_estimation {nee}",
         "camera 0 3 12  0 0.5 0  0 1 0  50",
         "attenuation 1 0.05 0.01",
         "point_light 4 6 4  12 11 10",
         "point_light -5 3 2  4 5 7",
         "directional_light 0.3 1 0.4  0.15 0.15 0.12",
         "quad_light -1 5.5 -1  2 0 0  0 0 2  6 6 6",
         "brdf phong",
         "emission 0 0 0",
         "ambient 0.03 0.03 0.03",
         "diffuse 0.5 0.5 0.45",
         "specular 0.2 0.2 0.2",
         "shininess 40"]
    _quad(L, (-12, 0, -12), (-12, 0, 12), (12, 0, 12), (12, 0, -12))
    for k in range(24):
        c = rng.uniform([-5.0, 0.3, -5.0], [5.0, 2.5, 3.0])
        r = rng.uniform(0.3, 0.9)
        kd = rng.uniform(0.05, 0.8, 3)
        mirror = rng.uniform() < 0.4
        ks = rng.uniform(0.3, 0.9, 3) if mirror else np.zeros(3)
        L += ["diffuse " + _v(*kd), "specular " + _v(*ks), "shininess " + _f(10 ** rng.uniform(0.5, 2.5)),
              "ambient " + _v(*(0.1 * kd))]
        if k % 3 == 2:
            sx, sy, sz = rng.uniform(0.5, 1.5, 3)
            L += ["push_transform", "translate " + _v(*c), "rotate 0 1 0 " + _f(rng.uniform(0, 180)),
                  "scale " + _v(sx, sy, sz), "sphere 0 0 0 " + _f(r), "pop_transform"]
        else:
            L.append("sphere " + _v(*c, r))
    return "\n".join(L) + "\n"


def batch_scene(index: int, seed: int = 1, max_tris: int = 500_000, resolutions=(128, 256, 512, 1024),
                spp_range=(4, 64), depth_range=(4, 10)) -> str:
    """Scene `index` of the batched workload: the Cornell box with a displaced
    icosphere of a log-uniform triangle count in [1000, max_tris] (the nearest
    icosphere level at or below the count, the rest as small clutter
    triangles), one material drawn from Lambertian / Phong / GGX, resolution
    drawn from `resolutions` (square), spp uniform in spp_range, max depth
    uniform in depth_range, NEE with MIS. Seeded by (seed, index)."""
    rng = np.random.default_rng([seed, index])
    target = int(round(np.exp(rng.uniform(np.log(1000), np.log(max_tris)))))
    level = 0
    while 20 * 4 ** (level + 1) <= target:
        level += 1
    clutter = max(0, target - 20 * 4 ** level)
    res = int(rng.choice(resolutions))
    spp = int(rng.integers(spp_range[0], spp_range[1] + 1))
    depth = int(rng.integers(depth_range[0], depth_range[1] + 1))
    L = cornell(res, res, spp, depth, int(rng.integers(1, 1 << 30)), "pathtracer", "mis").splitlines()
    kind = int(rng.integers(0, 3))
    if kind == 0:
        L += ["brdf lambertian", "diffuse " + _v(*rng.uniform(0.2, 0.8, 3)), "specular 0 0 0"]
    elif kind == 1:
        L += ["brdf phong", "diffuse " + _v(*rng.uniform(0.1, 0.5, 3)), "specular " + _v(*rng.uniform(0.1, 0.5, 3)),
              "shininess " + _f(10 ** rng.uniform(0.5, 2.5))]
    else:
        L += ["brdf ggx", "diffuse " + _v(*rng.uniform(0.0, 0.3, 3)), "specular " + _v(*rng.uniform(0.2, 0.9, 3)),
              "roughness " + _f(rng.uniform(0.05, 0.5))]
    V, F = icosphere(level)
    V = V * (1.0 + 0.1 * value_noise(V, seed * 1000 + index, freq=3.0))[:, None]
    c = rng.uniform([-0.4, 0.5, -0.4], [0.4, 1.1, 0.4])
    r = rng.uniform(0.25, 0.45)
    L += ["push_transform", "translate " + _v(*c), "scale " + _v(r / 1000, r / 1000, r / 1000)]
    _mesh_fast(L, V * 1000.0, F)
    L.append("pop_transform")
    if clutter:
        L += ["push_transform", "scale 0.001 0.001 0.001"]
        centres = rng.uniform([-0.95, 0.05, -0.95], [0.95, 1.95, 0.95], size=(clutter, 3))
        edge = rng.uniform(0.01, 0.05, size=clutter)
        d1 = rng.normal(size=(clutter, 3))
        d1 /= np.linalg.norm(d1, axis=1, keepdims=True)
        d2 = rng.normal(size=(clutter, 3))
        d2 -= (d2 * d1).sum(1, keepdims=True) * d1
        d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
        tri = np.stack([centres, centres + d1 * edge[:, None], centres + (0.5 * d1 + 0.866 * d2) * edge[:, None]], 1)
        _mesh_fast(L, tri.reshape(-1, 3) * 1000.0, np.arange(3 * clutter, dtype=np.int64).reshape(-1, 3))
        L.append("pop_transform")
    return "\n".join(L) + "\n"


def slit_room(width: int = 1024, height: int = 1024, spp: int = 16, max_depth: int = 10, level: int = 8,
              clutter: int = 10000, seed: int = 1, roughness: float | None = None) -> str:
    """Guiding workload: the dense-mesh icosphere and clutter inside a closed
    room [-1,1]x[0,2]x[-1,1] whose only opening is a 0.05-wide slit across the
    ceiling (x in [-0.025, 0.025]); a 1x1 quad light of emission 50 outside,
    0.5 above the slit, lights the room through it. Every object (each wall,
    the icosphere, the clutter) has its own GGX material with alpha
    U[0.05, 0.5] (or `roughness` for all). Camera inside the room. NEE with
    MIS, BRDF sampling."""
    rng = np.random.default_rng(seed)
    L = ["# closed room lit through a ceiling slit",
         f"random_seed {seed}",
         f"film_size {width} {height}",
         "integrator pathtracer",
         f"pixel_samples {spp}",
         f"max_depth {max_depth}",
         "next_event_estimation mis",
         "importance_sampling brdf",
         "russian_roulette off",
         "camera 0 1.1 0.95  0 0.7 -1  0 1 0  60",
         "quad_light -0.5 2.5 -0.5  0 0 1  1 0 0  50 50 50",
         "emission 0 0 0",
         "ambient 0 0 0"]

    def ggx(kd):
        return ["brdf ggx", "diffuse " + _v(*kd), "specular 0.04 0.04 0.04",
                "roughness " + _f(rng.uniform(0.05, 0.5) if roughness is None else roughness)]

    h = 0.025
    walls = [
        ((0.6, 0.6, 0.6), [((-1, 0, -1), (-1, 0, 1), (1, 0, 1), (1, 0, -1))]),                       # floor
        ((0.6, 0.6, 0.6), [((-1, 2, -1), (-h, 2, -1), (-h, 2, 1), (-1, 2, 1)),                       # ceiling
                           ((h, 2, -1), (1, 2, -1), (1, 2, 1), (h, 2, 1))]),
        ((0.6, 0.6, 0.6), [((-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1))]),                     # back
        ((0.6, 0.6, 0.6), [((-1, 0, 1), (-1, 2, 1), (1, 2, 1), (1, 0, 1))]),                         # front
        ((0.63, 0.065, 0.05), [((-1, 0, -1), (-1, 2, -1), (-1, 2, 1), (-1, 0, 1))]),                 # left
        ((0.14, 0.45, 0.09), [((1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1))]),                      # right
    ]
    for kd, quads in walls:
        L += ggx(kd)
        for a, b, c, d in quads:
            _quad(L, a, b, c, d)
    V, F = icosphere(level)
    V = V * (1.0 + 0.1 * value_noise(V, seed, freq=3.0))[:, None]
    L += ggx((0.5, 0.45, 0.4))
    L += ["push_transform", "translate 0 0.6 -0.2", "scale 0.0005 0.0005 0.0005"]
    _mesh_fast(L, V * 1000.0, F)
    L.append("pop_transform")
    if clutter:
        L += ggx((0.3, 0.4, 0.6))
        L += ["push_transform", "scale 0.001 0.001 0.001"]
        centres = rng.uniform([-0.95, 0.05, -0.95], [0.95, 1.95, 0.95], size=(clutter, 3))
        edge = rng.uniform(0.01, 0.05, size=clutter)
        d1 = rng.normal(size=(clutter, 3))
        d1 /= np.linalg.norm(d1, axis=1, keepdims=True)
        d2 = rng.normal(size=(clutter, 3))
        d2 -= (d2 * d1).sum(1, keepdims=True) * d1
        d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
        tri = np.stack([centres, centres + d1 * edge[:, None], centres + (0.5 * d1 + 0.866 * d2) * edge[:, None]], 1)
        _mesh_fast(L, tri.reshape(-1, 3) * 1000.0, np.arange(3 * clutter, dtype=np.int64).reshape(-1, 3))
        L.append("pop_transform")
    return "\n".join(L) + "\n"


WORKLOADS = {
    "cornell": cornell,
    "sphere_field": sphere_field,
    "feature_mix": feature_mix,
    "dense_mesh": dense_mesh,
    "slit_room": slit_room,
}
