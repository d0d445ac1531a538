"""Synthetic FacetRT scenes, band optics and hemisphere sample tables.

Every scene is seeded (numpy default_rng) and Y-up like the reference
(facetrtcore.cpp:485-486, :496).  Vertex arrays are (3F, 6) float32
[px, py, pz, nx, ny, nz] with the three vertices of a facet consecutive and
sharing the unit normal normalize((b-a) x (c-a)) (appendTriangle,
facetrtcore.cpp:287-306).  Object facets come first, ground facets last
(facetrtcore.cpp:2998-3004), and `leaf_count` is the number of object facets.

Named workloads:
  config1  10 x 10 m soil (32 x 32 quads = 2,048 triangles) + 2,048 leaf
           triangles (edge 0.05 m, centres in [-5,5]^2 x [0.2,1.5], normals on
           the upper hemisphere): 4,096 facets.
  config2  60 trees (64-triangle trunk cylinder r = 0.15 m, h ~ U(4,8); crown
           sphere r ~ U(1.5,3) of 3,000 leaves, edge 0.08 m, normals on the
           sphere) on a 50 x 50 m soil of 20,000 triangles: 203,840 facets.
  config3  the same forest with 150 trees on 80 x 80 m: 479,600 facets.
  c5_scenes  32 scenes with facet counts log-uniform in [20k, 400k], cycling
           row crops (0.75 m rows of 0.3 m-wide leaf hedges), forests (the
           config-2 tree) and urban blocks (5-40 m boxes, faces subdivided
           into 0.5 m cells), each on its own soil.
"""
import math

import numpy as np


class Scene:
    def __init__(self, vertices, leaf_count, name, trunk_count=0, walls=False):
        self.vertices = np.ascontiguousarray(vertices, np.float32)
        self.leaf_count = int(leaf_count)
        self.trunk_count = int(trunk_count)
        self.walls = bool(walls)  # object facets are building walls and roofs
        self.name = name

    @property
    def facet_count(self):
        return len(self.vertices) // 3

    @property
    def surface_count(self):
        return 2 * self.facet_count

    def bounds(self):
        p = self.vertices[:, :3]
        return p.min(0), p.max(0)

    def normals(self):
        return self.vertices[0::3, 3:6]


def _triangles_to_vertices(a, b, c):
    """(F,3) corner arrays -> (3F,6) vertex array with facet normals."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    c = np.asarray(c, np.float64)
    n = np.cross(b - a, c - a)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    keep = ln[:, 0] > 1e-12
    n = n[keep] / ln[keep]
    F = int(keep.sum())
    v = np.empty((F, 3, 6), np.float64)
    v[:, 0, :3] = a[keep]
    v[:, 1, :3] = b[keep]
    v[:, 2, :3] = c[keep]
    v[:, :, 3:] = n[:, None, :]
    return v.reshape(-1, 6).astype(np.float32)


def _orthonormal(n):
    helper = np.where(np.abs(n[:, 1:2]) < 0.9, [[0.0, 1.0, 0.0]], [[1.0, 0.0, 0.0]])
    t = np.cross(helper, n)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    b = np.cross(n, t)
    return t, b


def equilateral(centres, normals, edge, rng):
    """Equilateral triangles (counter-clockwise around `normals`)."""
    centres = np.asarray(centres, np.float64)
    normals = np.asarray(normals, np.float64)
    normals = normals / np.linalg.norm(normals, axis=1, keepdims=True)
    t, b = _orthonormal(normals)
    theta = rng.uniform(0, 2 * np.pi, len(centres))[:, None]
    R = edge / math.sqrt(3.0)
    corners = []
    for k in range(3):
        ang = theta + 2 * np.pi * k / 3
        corners.append(centres + R * (np.cos(ang) * t + np.sin(ang) * b))
    return corners


def uniform_sphere(n, rng):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def soil_grid(x0, x1, z0, z1, nx, nz, y=0.0):
    xs = np.linspace(x0, x1, nx + 1)
    zs = np.linspace(z0, z1, nz + 1)
    X0, Z0 = np.meshgrid(xs[:-1], zs[:-1], indexing="ij")
    X1, Z1 = np.meshgrid(xs[1:], zs[1:], indexing="ij")
    X0, Z0, X1, Z1 = (q.ravel() for q in (X0, Z0, X1, Z1))
    Y = np.full_like(X0, y)
    a = np.stack([X0, Y, Z0], 1)
    b1 = np.stack([X0, Y, Z1], 1)
    c1 = np.stack([X1, Y, Z1], 1)
    d1 = np.stack([X1, Y, Z0], 1)
    # both triangles face +Y: (a, b1, c1) and (a, c1, d1)
    A = np.concatenate([a, a])
    B = np.concatenate([b1, c1])
    C = np.concatenate([c1, d1])
    return A, B, C


def cylinder(base, radius, height, segments=32):
    ang = np.linspace(0, 2 * np.pi, segments + 1)[:-1]
    ang2 = np.roll(ang, -1)
    p0 = np.stack([np.cos(ang), np.zeros_like(ang), np.sin(ang)], 1) * radius
    p1 = np.stack([np.cos(ang2), np.zeros_like(ang2), np.sin(ang2)], 1) * radius
    up = np.array([0.0, height, 0.0])
    base = np.asarray(base, np.float64)
    # outward normals: (p0, p0+up, p1) and (p1, p0+up, p1+up)
    A = np.concatenate([base + p0, base + p1])
    B = np.concatenate([base + p0 + up, base + p0 + up])
    C = np.concatenate([base + p1, base + p1 + up])
    return A, B, C


def quad_grid(origin, u, v, nu, nv):
    """Triangles of the parallelogram origin + s u + t v (s, t in [0, 1]) in
    nu x nv cells, facing u x v."""
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    i = i.ravel()[:, None].astype(np.float64)
    j = j.ravel()[:, None].astype(np.float64)
    o = np.asarray(origin, np.float64)
    du = np.asarray(u, np.float64) / nu
    dv = np.asarray(v, np.float64) / nv
    p00 = o + i * du + j * dv
    return (np.concatenate([p00, p00]), np.concatenate([p00 + du, p00 + du + dv]),
            np.concatenate([p00 + du + dv, p00 + dv]))


def box(x0, z0, w, d, h, cell=0.5):
    """Roof and four walls of a w x d x h box (outward normals), every face
    subdivided into cells of about `cell` metres."""
    n = lambda length: max(1, int(math.ceil(length / cell)))
    faces = [((x0, h, z0), (0, 0, d), (w, 0, 0), n(d), n(w)),          # roof, +y
             ((x0, 0, z0), (0, 0, d), (0, h, 0), n(d), n(h)),          # -x
             ((x0 + w, 0, z0), (0, h, 0), (0, 0, d), n(h), n(d)),      # +x
             ((x0, 0, z0), (0, h, 0), (w, 0, 0), n(h), n(w)),          # -z
             ((x0, 0, z0 + d), (w, 0, 0), (0, h, 0), n(w), n(h))]      # +z
    parts = [quad_grid(*f) for f in faces]
    return tuple(np.concatenate([p[k] for p in parts]) for k in range(3))


def row_crops(target, seed=0, leaf_edge=0.05, spacing=0.75, width=0.3):
    """Hedge rows along x, `spacing` m apart and `width` m wide, of leaf
    triangles (normals on the upper hemisphere) over a soil plane; about
    `target` facets (10 % soil)."""
    rng = np.random.default_rng(seed)
    nq = max(8, int(round(math.sqrt(0.05 * target))))
    leaves = max(1, target - 2 * nq * nq)
    L = float(np.clip(math.sqrt(leaves) / 12.0, 4.0, 60.0))
    rows = max(2, int(L / spacing))
    row_z = -L / 2 + spacing / 2 + spacing * rng.integers(0, rows, leaves)
    height = rng.uniform(0.4, 0.9, rows)[((row_z + L / 2 - spacing / 2) / spacing).round().astype(int)]
    centres = np.stack([rng.uniform(-L / 2, L / 2, leaves), rng.uniform(0.05, 1.0, leaves) * height,
                        row_z + rng.uniform(-width / 2, width / 2, leaves)], 1)
    nrm = uniform_sphere(leaves, rng)
    nrm[:, 1] = np.abs(nrm[:, 1])
    leaf = _triangles_to_vertices(*equilateral(centres, nrm, leaf_edge, rng))
    soil = _triangles_to_vertices(*soil_grid(-L / 2, L / 2, -L / 2, L / 2, nq, nq))
    return Scene(np.concatenate([leaf, soil]), len(leaf) // 3, f"crops({target}, seed={seed})")


def forest_of(target, seed=0):
    """The config-2 tree (3,000 leaves and a 64-triangle trunk) repeated to
    about `target` facets over a soil of about 10 % of them."""
    soil_quads = max(64, int(0.05 * target))
    trees = max(1, int(round((target - 2 * soil_quads) / 3064)))
    extent = 10.0 + 6.0 * math.sqrt(trees)
    return forest(trees, extent, soil_quads, seed, name=f"forest({target}, seed={seed})")


def urban(target, seed=0, cell=0.5):
    """5-40 m boxes on 50 m plots until about `target` facets, on a soil of
    about 5 % of them."""
    rng = np.random.default_rng(seed)
    nq = max(8, int(round(math.sqrt(0.025 * target))))
    parts = []
    count = 2 * nq * nq
    k = 0
    while count < target or not parts:
        w, d, h = rng.uniform(5.0, 40.0, 3)
        b = box(50.0 * (k % 8) + rng.uniform(0, 50 - w), 50.0 * (k // 8) + rng.uniform(0, 50 - d),
                w, d, h, cell)
        parts.append(_triangles_to_vertices(*b))
        count += len(parts[-1]) // 3
        k += 1
    walls = np.concatenate(parts)
    p = walls[:, :3]
    x0, z0 = p[:, 0].min() - 10, p[:, 2].min() - 10
    x1, z1 = p[:, 0].max() + 10, p[:, 2].max() + 10
    soil = _triangles_to_vertices(*soil_grid(x0, x1, z0, z1, nq, nq))
    return Scene(np.concatenate([walls, soil]), len(walls) // 3, f"urban({target}, seed={seed})",
                 walls=True)


def c5_scenes(count=32, seed=0, lo=20000, hi=400000):
    """Scenes of uneven size: facet counts log-uniform in [lo, hi], kinds
    cycling crops, forest, urban."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(lo), math.log(hi), count)).astype(int)
    makers = (row_crops, forest_of, urban)
    return [makers[i % 3](int(n), seed + 1 + i) for i, n in enumerate(sizes)]


def config1(seed=0, leaves=2048, grid=32):
    rng = np.random.default_rng(seed)
    centres = np.stack([rng.uniform(-5, 5, leaves), rng.uniform(0.2, 1.5, leaves),
                        rng.uniform(-5, 5, leaves)], 1)
    n = uniform_sphere(leaves, rng)
    n[:, 1] = np.abs(n[:, 1])
    leaf = _triangles_to_vertices(*equilateral(centres, n, 0.05, rng))
    soil = _triangles_to_vertices(*soil_grid(-5, 5, -5, 5, grid, grid))
    return Scene(np.concatenate([leaf, soil]), len(leaf) // 3, f"config1(seed={seed})")


def forest(trees, extent, soil_quads, seed=0, leaves_per_crown=3000, leaf_edge=0.08,
           name="forest"):
    rng = np.random.default_rng(seed)
    half = extent / 2.0
    parts = []
    trunk_parts = []
    for _ in range(trees):
        x, z = rng.uniform(-half + 3, half - 3, 2)
        h = rng.uniform(4.0, 8.0)
        r = rng.uniform(1.5, 3.0)
        trunk_parts.append(_triangles_to_vertices(*cylinder((x, 0.0, z), 0.15, h)))
        # uniform points in the crown sphere
        d = uniform_sphere(leaves_per_crown, rng)
        rad = r * rng.uniform(0, 1, leaves_per_crown) ** (1.0 / 3.0)
        centres = np.array([x, h, z]) + d * rad[:, None]
        centres[:, 1] = np.maximum(centres[:, 1], 0.3)
        normals = uniform_sphere(leaves_per_crown, rng)
        parts.append(_triangles_to_vertices(*equilateral(centres, normals, leaf_edge, rng)))
    leaves = np.concatenate(parts)
    trunks = np.concatenate(trunk_parts)
    nq = int(round(math.sqrt(soil_quads)))
    soil = _triangles_to_vertices(*soil_grid(-half, half, -half, half, nq, nq))
    verts = np.concatenate([leaves, trunks, soil])
    obj = (len(leaves) + len(trunks)) // 3
    return Scene(verts, obj, name, trunk_count=len(trunks) // 3)


def config2(seed=0):
    return forest(60, 50.0, 10000, seed, name=f"config2(seed={seed})")


def config3(seed=0):
    return forest(150, 80.0, 10000, seed, name=f"config3(seed={seed})")


# ---- directions and optics ------------------------------------------------
def sun_direction(zenith_deg, azimuth_deg):
    """facetrtcore.cpp:491-498, evaluated by the library's C++ host code so
    that it rounds exactly as the reference's (C library cos/sin)."""
    from . import facetcu
    return facetcu.sun_direction(zenith_deg, azimuth_deg)


def hemisphere_directions(count=40):
    """facetrtcore.cpp:475-489 (golden-spiral upper hemisphere), evaluated by
    the library's C++ host code."""
    from . import facetcu
    return facetcu.hemisphere_directions(count)


def direct_geometry(scene, sunlit, sun):
    """sunlit_s * max(0, n_s . sun) per side (the D of makeOptics without the beam)."""
    n = scene.normals().astype(np.float32)
    c = n @ np.asarray(sun, np.float32)
    cos = np.empty(2 * len(n), np.float32)
    cos[0::2] = np.maximum(c, 0)
    cos[1::2] = np.maximum(-c, 0)
    return (np.asarray(sunlit, np.float32) * cos).astype(np.float32)


def band_optics(scene, bands=64, leaf=(0.04, 0.48), soil=(0.12, 0.30), leaf_tau_ratio=0.4,
                wall=(0.20, 0.30)):
    """Per-band reflectance/transmittance (bands, S): leaf rho ramps leaf[0] ->
    leaf[1] with tau = leaf_tau_ratio * rho, soil rho soil[0] -> soil[1] and
    tau = 0; trunk facets take the leaf reflectance with tau = 0; walls (urban
    scenes) ramp wall[0] -> wall[1] with tau = 0.  Both sides of a facet share
    its material."""
    if scene.walls:
        F = scene.facet_count
        t = np.linspace(0.0, 1.0, bands) if bands > 1 else np.zeros(1)
        material = np.full(2 * F, 1, np.intp)
        material[:2 * scene.leaf_count] = 0
        rho_t = np.stack([wall[0] + (wall[1] - wall[0]) * t,
                          soil[0] + (soil[1] - soil[0]) * t], 1).astype(np.float32)
        return rho_t[:, material], np.zeros((bands, 2 * F), np.float32)
    F = scene.facet_count
    t = np.linspace(0.0, 1.0, bands, dtype=np.float64) if bands > 1 else np.zeros(1)
    lr = leaf[0] + (leaf[1] - leaf[0]) * t
    sr = soil[0] + (soil[1] - soil[0]) * t
    nleaf = scene.leaf_count - scene.trunk_count
    # material per side: 0 leaf, 1 trunk, 2 soil; one (bands, 3) table each
    material = np.full(2 * F, 2, np.intp)
    material[:2 * nleaf] = 0
    material[2 * nleaf:2 * scene.leaf_count] = 1
    rho_t = np.stack([lr, lr, sr], 1).astype(np.float32)
    tau_t = np.stack([leaf_tau_ratio * lr, np.zeros(bands), np.zeros(bands)], 1).astype(np.float32)
    return rho_t[:, material], tau_t[:, material]


def thermal_optics(scene, temperature, wavelength_nm=11000.0, leaf_eps=0.97, ground_eps=0.95):
    """One thermal band: rho = 1 - eps, tau = 0, emission eps * Planck(T) per
    side (W m-2 sr-1 um-1), leaf emissivity for leaf and trunk facets, the
    ground one for soil and walls; temperature per facet (K)."""
    F = scene.facet_count
    eps_f = np.full(F, ground_eps)
    if not scene.walls:
        eps_f[:scene.leaf_count] = leaf_eps
    # Planck's law in W m-2 sr-1 um-1 (c1 = 2 h c^2, c2 = h c / k in um K)
    um = wavelength_nm / 1000.0
    t = np.maximum(1.0, np.asarray(temperature, np.float64))
    planck = 1.1910439340652e8 / (um ** 5 * np.expm1(14388.291040407 / (t * um)))
    eps = np.repeat(eps_f, 2)
    rho = (1.0 - eps).astype(np.float32)
    return rho, np.zeros_like(rho), (eps * np.repeat(planck, 2)).astype(np.float32)


def reference_optics(scene, sunlit, sun, beam=700.0, leaf_rho=0.10, leaf_tau=0.05,
                     ground_rho=0.20, ground_tau=0.0):
    """makeOptics (facetrtcore.cpp:500-522) with its constants as arguments."""
    F = scene.facet_count
    o = np.zeros((2 * F, 4), np.float32)
    leaf = np.arange(F) < scene.leaf_count
    o[:, 0] = np.repeat(np.where(leaf, leaf_rho, ground_rho), 2)
    o[:, 1] = np.repeat(np.where(leaf, leaf_tau, ground_tau), 2)
    o[:, 3] = direct_geometry(scene, sunlit, sun) * np.float32(beam)
    return o


def hemisphere_samples(rays, sets=32, seed=1234):
    """Per-set sample tables for the hemisphere ray caster.

    uv: (sets, rays, 2) barycentric weights of vertices b and c (origin =
    a + u (b - a) + v (c - a)), strictly inside the triangle;
    dirs: (sets, rays, 3) cosine-distributed unit directions in the side's
    local frame (z along the side normal).  Stratified: a rotated
    golden-ratio lattice per set (Cranley-Patterson shift), mapped with
    Malley's method; computed in float64 and stored as float32."""
    rng = np.random.default_rng(seed)
    j = np.arange(rays, dtype=np.float64)
    phi = (math.sqrt(5.0) - 1.0) / 2.0
    uv = np.empty((sets, rays, 2), np.float32)
    dirs = np.empty((sets, rays, 3), np.float32)
    for p in range(sets):
        s1, s2, s3, s4 = rng.uniform(0, 1, 4)
        u1 = np.mod((j + 0.5) / rays + s1, 1.0)
        u2 = np.mod(j * phi + s2, 1.0)
        r = np.sqrt(u1)
        a = 2 * np.pi * u2
        d = np.stack([r * np.cos(a), r * np.sin(a), np.sqrt(np.maximum(1.0 - u1, 0.0))], 1)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        dirs[p] = d
        w1 = 0.02 + 0.96 * np.mod(j * phi + s3, 1.0)
        w2 = 0.02 + 0.96 * np.mod((j + 0.5) / rays + s4, 1.0)
        su = np.sqrt(w1)
        uv[p, :, 0] = su * (1.0 - w2)
        uv[p, :, 1] = su * w2
    return uv, dirs


def energy_site(seed=0, leaves=1500, soil_cells=16):
    """A small FacetEB site: a leaf crown, a building, a tilted PV array and
    a soil plane (objects first, soil last, as loadProjectScene orders them).
    Returns (scene, material_indices, kinds) where kinds names the material
    slots: 0 leaf, 1 wall, 2 PV, 3-5 soils (force-restore, 0.35 Rn, dry
    1.5 x force-restore); index 99 marks facets without a material."""
    rng = np.random.default_rng(seed)
    centres = rng.normal(0.0, 1.0, (leaves, 3))
    centres *= (1.4 * rng.uniform(0, 1, leaves) ** (1 / 3) /
                np.linalg.norm(centres, axis=1))[:, None]
    centres += np.array([-2.0, 2.6, 0.0])
    leaf = _triangles_to_vertices(*equilateral(centres, uniform_sphere(leaves, rng), 0.08, rng))
    wall = _triangles_to_vertices(*box(1.0, -2.5, 2.5, 2.0, 3.0, cell=0.6))
    tilt = np.array([0.0, 0.55, -0.85])
    panel = _triangles_to_vertices(*quad_grid((-3.0, 0.8, 3.0), (3.0, 0.0, 0.0), tilt, 8, 2))
    soil = _triangles_to_vertices(*soil_grid(-6, 6, -6, 6, soil_cells, soil_cells))
    objects = len(leaf) // 3 + len(wall) // 3 + len(panel) // 3
    vertices = np.concatenate([leaf, wall, panel, soil])
    F = len(vertices) // 3
    nl, nw, npv = len(leaf) // 3, len(wall) // 3, len(panel) // 3
    mi = np.empty(F, np.uint32)
    mi[:nl] = np.where(rng.uniform(0, 1, nl) < 0.9, 0, 99)
    mi[nl:nl + nw] = 1
    mi[nl + nw:objects] = 2
    mi[objects:] = rng.choice([3, 4, 5, 99], F - objects, p=[0.4, 0.25, 0.25, 0.1])
    return Scene(vertices, objects, f"energy_site(seed={seed})", walls=False), mi, (
        "leaf", "wall", "pv", "soil", "soil_storage_035", "dry_soil")
