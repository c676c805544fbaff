"""Seeded synthetic scenes and ray sets (the workloads of the render hot path).

Every generator computes in float64 and casts once to float32, so the same
seed gives the same bits on any host.  Layouts are the ones the C ABI takes:
de-indexed triangles float32[ntri, 9] (the form cr::registry::register_model
stores after persist_and_expand, src/render/entities/registry.cpp:51-97), a
per-primitive material index, and a crg_material table.

  box_scene()        — the "box" scene: 5 wall quads of a unit cube (open
                       towards the camera), two boxes rotated +-17 deg about y,
                       one 0.25 x 0.25 ceiling light of radiance 17; 36 triangles.
  soup(), soup_rays()— 1,048,576-triangle random soup and its primary/shadow rays.
  displaced_scene()  — fBm-displaced icosphere on a ground quad with per-triangle
                       Lambert / GGX / glass materials, a sphere light and a
                       constant environment.
"""
from __future__ import annotations

import math
import os

import numpy as np

from ._abi import MATERIAL_DTYPE, RAY_DTYPE, SHADE_GLASS, SHADE_METAL, SHADE_SMOOTH


def material_table(rows):
    """rows: list of dicts with crg_material fields; defaults follow
    cr::material::information (src/render/material/material.h:31-41)."""
    m = np.zeros(len(rows), MATERIAL_DTYPE)
    for i, r in enumerate(rows):
        m[i]["shade_type"] = r.get("shade_type", SHADE_SMOOTH)
        m[i]["ior"] = r.get("ior", 1.5)
        m[i]["roughness"] = r.get("roughness", 0.5)
        m[i]["reflectiveness"] = r.get("reflectiveness", 1.0)
        m[i]["emission"] = r.get("emission", 0.0)
        m[i]["colour"] = r.get("colour", (1.0, 1.0, 1.0, 1.0))
        m[i]["tex"] = r.get("tex", -1)
    return m


def _quad(corners, normal):
    """Two triangles of a planar quad, wound so cross(v1-v0, v2-v0) points along normal."""
    a, b, c, d = (np.asarray(p, np.float64) for p in corners)
    if np.dot(np.cross(b - a, c - a), np.asarray(normal, np.float64)) < 0:
        a, b, c, d = a, d, c, b
    return [np.concatenate([a, b, c]), np.concatenate([a, c, d])]


def _box(size, base_centre, angle_deg):
    """12 outward-wound triangles of a box standing on y=0, rotated about y."""
    sx, sy, sz = size
    th = math.radians(angle_deg)
    cth, sth = math.cos(th), math.sin(th)

    def P(x, y, z):
        # Ry(theta) applied to the local corner, then translated
        return (base_centre[0] + x * cth + z * sth, y, base_centre[2] - x * sth + z * cth)

    hx, hz = sx / 2, sz / 2
    c = {
        (i, j, k): P((2 * i - 1) * hx, j * sy, (2 * k - 1) * hz) for i in (0, 1) for j in (0, 1) for k in (0, 1)
    }
    centre = np.array([base_centre[0], sy / 2, base_centre[2]])
    faces = [
        [c[0, 0, 0], c[1, 0, 0], c[1, 1, 0], c[0, 1, 0]],
        [c[0, 0, 1], c[1, 0, 1], c[1, 1, 1], c[0, 1, 1]],
        [c[0, 0, 0], c[0, 0, 1], c[0, 1, 1], c[0, 1, 0]],
        [c[1, 0, 0], c[1, 0, 1], c[1, 1, 1], c[1, 1, 0]],
        [c[0, 0, 0], c[1, 0, 0], c[1, 0, 1], c[0, 0, 1]],
        [c[0, 1, 0], c[1, 1, 0], c[1, 1, 1], c[0, 1, 1]],
    ]
    tris = []
    for f in faces:
        fc = np.mean(np.asarray(f), axis=0)
        tris += _quad(f, fc - centre)
    return tris


def box_scene():
    """The 36-triangle box scene (Lambertian only; sun off; no skybox).

    Returns dict(verts float32[36,9], mat_idx uint32[36], mats, camera dict)."""
    tris, mids = [], []

    def add(ts, m):
        tris.extend(ts)
        mids.extend([m] * len(ts))

    add(_quad([(0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0)], (0, 1, 0)), 0)  # floor
    add(_quad([(0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)], (0, -1, 0)), 0)  # ceiling
    add(_quad([(0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1)], (0, 0, -1)), 0)  # back wall
    add(_quad([(0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)], (1, 0, 0)), 1)  # left wall (red)
    add(_quad([(1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0)], (-1, 0, 0)), 2)  # right wall (green)
    add(_box((0.3, 0.3, 0.3), (0.68, 0.0, 0.33), -17.0), 0)  # short box
    add(_box((0.3, 0.6, 0.3), (0.32, 0.0, 0.67), 17.0), 0)  # tall box
    y = 1.0 - 1e-3
    add(_quad([(0.375, y, 0.375), (0.625, y, 0.375), (0.625, y, 0.625), (0.375, y, 0.625)], (0, -1, 0)), 3)  # light
    verts = np.asarray(tris, np.float64).astype(np.float32)
    mats = material_table(
        [
            {"colour": (0.73, 0.73, 0.73, 1.0)},
            {"colour": (0.63, 0.065, 0.05, 1.0)},
            {"colour": (0.14, 0.45, 0.09, 1.0)},
            {"colour": (1.0, 1.0, 1.0, 1.0), "emission": 17.0},
        ]
    )
    camera = dict(position=(0.5, 0.5, -1.4), rotation=(0.0, 0.0, 0.0), fov=40.0, mode=0, scale=1.0)
    return dict(verts=np.ascontiguousarray(verts), mat_idx=np.asarray(mids, np.uint32), mats=mats, camera=camera)


def textured_box(seed=5):
    """The box scene with per-corner texture coordinates and four textures
    (cr::image entities referenced by material `tex`):
      0  a 16x16 two-tone checker on the floor, ceiling and back wall;
      1  a 32x32 texture on both inner boxes whose alpha is zero in a grid of
         holes (pass-through texels, renderer.cpp:37-41);
      2  an 8x8 colour gradient on the light (a textured emitter);
      3  a 4x4 noise texture on the left wall.
    Coordinates are the corner positions projected on the two axes of the
    face's plane, scaled so textures repeat across a face."""
    sc = box_scene()
    v = sc["verts"].reshape(-1, 3, 3).astype(np.float64)
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    ax = np.argmax(np.abs(n), axis=1)
    uvs = np.zeros((len(v), 3, 2))
    for t in range(len(v)):
        a, b = [k for k in range(3) if k != ax[t]]
        uvs[t, :, 0] = v[t, :, a] * 2.0
        uvs[t, :, 1] = v[t, :, b] * 2.0
    r = np.random.default_rng(seed)
    ii, jj = np.meshgrid(np.arange(16), np.arange(16), indexing="ij")
    checker = np.where(((ii // 4 + jj // 4) % 2 == 0)[..., None], [0.8, 0.8, 0.75, 1.0], [0.3, 0.35, 0.6, 1.0])
    holes = np.tile([0.9, 0.7, 0.3, 1.0], (32, 32, 1))
    hi, hj = np.meshgrid(np.arange(32), np.arange(32), indexing="ij")
    holes[(hi % 8 < 3) & (hj % 8 < 3), 3] = 0.0
    gi, gj = np.meshgrid(np.linspace(0.4, 1.0, 8), np.linspace(0.5, 1.0, 8), indexing="ij")
    grad = np.stack([gi, gj, np.full_like(gi, 0.8), np.ones_like(gi)], -1)
    noise = np.concatenate([r.uniform(0.2, 0.8, (4, 4, 3)), np.ones((4, 4, 1))], -1)
    mats = material_table(
        [
            {"colour": (0.73, 0.73, 0.73, 1.0), "tex": 0},
            {"colour": (0.63, 0.065, 0.05, 1.0), "tex": 3},
            {"colour": (0.14, 0.45, 0.09, 1.0)},
            {"colour": (1.0, 1.0, 1.0, 1.0), "emission": 17.0, "tex": 2},
            {"colour": (0.73, 0.73, 0.73, 1.0), "tex": 1},
        ]
    )
    mat_idx = sc["mat_idx"].copy()
    mat_idx[10:34] = 4  # the two inner boxes
    textures = [t.astype(np.float32) for t in (checker, holes, grad, noise)]
    return dict(sc, mats=mats, mat_idx=mat_idx, uvs=uvs.reshape(-1, 6).astype(np.float32), textures=textures)


def affine(translate=(0.0, 0.0, 0.0), rotate_deg=(0.0, 0.0, 0.0), scale=(1.0, 1.0, 1.0)):
    """4x4 row-major T * Ry * Rx * Rz * S (float32)."""
    ax, ay, az = np.radians(np.asarray(rotate_deg, np.float64))
    rx = np.array([[1, 0, 0], [0, np.cos(ax), -np.sin(ax)], [0, np.sin(ax), np.cos(ax)]])
    ry = np.array([[np.cos(ay), 0, np.sin(ay)], [0, 1, 0], [-np.sin(ay), 0, np.cos(ay)]])
    rz = np.array([[np.cos(az), -np.sin(az), 0], [np.sin(az), np.cos(az), 0], [0, 0, 1]])
    m = np.eye(4)
    m[:3, :3] = ry @ rx @ rz @ np.diag(np.asarray(scale, np.float64))
    m[:3, 3] = translate
    return m.astype(np.float32)


def instanced_box():
    """Three instances of the box scene's mesh (cr::entity::instances): the
    identity, a copy moved right, turned 30 degrees about y and scaled
    non-uniformly, and a copy moved left and up, tilted 10 degrees about x;
    the camera is pulled back to see all three."""
    sc = box_scene()
    inst = np.stack([affine(),
                     affine((1.25, 0.0, 0.35), (0.0, 30.0, 0.0), (0.8, 1.1, 0.9)),
                     affine((-1.2, 0.25, 0.2), (10.0, 0.0, 0.0), (1.0, 1.0, 1.0))])
    camera = dict(position=(0.5, 0.65, -3.2), rotation=(0.0, 0.0, 0.0), fov=45.0, mode=0, scale=1.0)
    return dict(sc, instances=inst, camera=camera)


def merge_models(models, camera=None):
    """A scene of several models (cr::registry entities, each with its own mesh,
    materials and instance list): `models` is a list of dicts {verts, mat_idx,
    mats[, uvs][, instances]} with model-local material indices.  Returns the
    scene dict with the merged arrays the library holds after
    crg_scene_add_model (primitives in model order, material indices rebased)
    and the list itself under "models"."""
    verts = np.concatenate([np.asarray(m["verts"], np.float32).reshape(-1, 9) for m in models])
    mats = np.concatenate([np.asarray(m["mats"]) for m in models])
    base = np.cumsum([0] + [len(m["mats"]) for m in models])
    mat_idx = np.concatenate([np.asarray(m["mat_idx"], np.uint32) + np.uint32(base[k]) for k, m in enumerate(models)])
    out = dict(verts=np.ascontiguousarray(verts), mat_idx=mat_idx.astype(np.uint32), mats=mats, models=list(models))
    if any(m.get("uvs") is not None for m in models):
        out["uvs"] = np.concatenate([np.asarray(m["uvs"], np.float32).reshape(-1, 6) if m.get("uvs") is not None
                                     else np.zeros((len(np.asarray(m["verts"]).reshape(-1, 9)), 6), np.float32)
                                     for m in models])
    if camera is not None:
        out["camera"] = camera
    return out


def multi_model_box(duplicate=False):
    """Three models with their own instance lists (cr::entity::instances per
    entity, components.h:18-21):
      0  the box room (walls and the ceiling light), no list (one identity instance);
      1  the short box with a metal, a glass and a Lambert material, three instances;
      2  the tall box plus a small emissive quad on its top, two instances.
    duplicate=True adds model 3, a second copy of model 1's mesh with one
    identity instance, so some hits of different models tie exactly (the earlier
    model must win)."""
    sc = box_scene()
    room = dict(verts=np.concatenate([sc["verts"][:10], sc["verts"][34:]]),
                mat_idx=np.concatenate([sc["mat_idx"][:10], sc["mat_idx"][34:]]), mats=sc["mats"])
    short = np.asarray(_box((0.3, 0.3, 0.3), (0.0, 0.0, 0.0), 0.0), np.float64).astype(np.float32)
    m1 = dict(verts=short, mat_idx=np.array([0, 0, 1, 1, 2, 2, 0, 0, 1, 1, 2, 2], np.uint32),
              mats=material_table([{"colour": (0.8, 0.6, 0.3, 1.0), "shade_type": SHADE_METAL, "roughness": 0.2},
                                   {"colour": (0.9, 0.95, 1.0, 1.0), "shade_type": SHADE_GLASS, "ior": 1.5},
                                   {"colour": (0.3, 0.5, 0.8, 1.0)}]),
              instances=np.stack([affine((0.68, 0.0, 0.33), (0.0, -17.0, 0.0)),
                                  affine((0.25, 0.0, 0.25), (0.0, 40.0, 0.0), (0.6, 0.5, 0.6)),
                                  affine((0.75, 0.45, 0.7), (15.0, 10.0, 5.0), (0.4, 0.4, 0.4))]))
    tall = _box((0.3, 0.6, 0.3), (0.0, 0.0, 0.0), 0.0)
    y = 0.6 + 2e-3
    lamp = _quad([(-0.05, y, -0.05), (0.05, y, -0.05), (0.05, y, 0.05), (-0.05, y, 0.05)], (0, 1, 0))
    m2 = dict(verts=np.asarray(tall + lamp, np.float64).astype(np.float32),
              mat_idx=np.array([0] * 12 + [1, 1], np.uint32),
              mats=material_table([{"colour": (0.7, 0.7, 0.7, 1.0)},
                                   {"colour": (1.0, 0.8, 0.6, 1.0), "emission": 6.0}]),
              instances=np.stack([affine((0.32, 0.0, 0.67), (0.0, 17.0, 0.0)),
                                  affine((0.85, 0.0, 0.8), (0.0, -30.0, 0.0), (0.5, 0.8, 0.5))]))
    models = [room, m1, m2]
    if duplicate:
        models.append(dict(m1, instances=None))
        models[1] = dict(m1, instances=np.concatenate([np.eye(4, dtype=np.float32)[None], m1["instances"]]))
    camera = dict(position=(0.5, 0.5, -1.4), rotation=(0.0, 0.0, 0.0), fov=40.0, mode=0, scale=1.0)
    return merge_models(models, camera)


def soup(n=1 << 20, seed=1, sigma=0.01):
    """Random triangle soup: centroids U[0,1]^3, vertex offsets N(0, sigma^2) per axis."""
    rng = np.random.default_rng(seed)
    cen = rng.random((n, 1, 3))
    off = rng.normal(0.0, sigma, (n, 3, 3))
    return np.ascontiguousarray((cen + off).reshape(n, 9).astype(np.float32))


def soup_rays(n, seed, shadow=False):
    """Rays from uniform points on the sphere around the unit cube (centre 0.5,
    radius sqrt(3)/2) towards U[0,1]^3 targets.  Primary rays: tmax = +inf;
    shadow rays: tmax ~ U[0.1, 1].  tmin = 1e-5 as src/objects/model.cpp:22."""
    rng = np.random.default_rng(seed)
    g = rng.normal(size=(n, 3))
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    org = 0.5 + g * (math.sqrt(3.0) / 2.0)
    tgt = rng.random((n, 3))
    d = tgt - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros(n, RAY_DTYPE)
    r["org"] = org.astype(np.float32)
    r["dir"] = d.astype(np.float32)
    r["tmin"] = np.float32(1e-5)
    r["tmax"] = rng.uniform(0.1, 1.0, n).astype(np.float32) if shadow else np.float32(np.inf)
    return r


def closed_box(albedo=0.5, emission=1.0):
    """Furnace scene: the six inward-facing faces of the unit cube, every face
    Lambertian with the given albedo and emission, camera inside.  Every path
    of the reference estimator hits a wall at every segment, so one sample is
    exactly sum_{k=1..B} albedo^k * emission (renderer.cpp:310-311)."""
    tris = []
    tris += _quad([(0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0)], (0, 1, 0))
    tris += _quad([(0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)], (0, -1, 0))
    tris += _quad([(0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1)], (0, 0, -1))
    tris += _quad([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)], (0, 0, 1))
    tris += _quad([(0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)], (1, 0, 0))
    tris += _quad([(1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0)], (-1, 0, 0))
    verts = np.asarray(tris, np.float64).astype(np.float32)
    mats = material_table([{"colour": (albedo, albedo, albedo, 1.0), "emission": emission}])
    camera = dict(position=(0.5, 0.5, 0.3), rotation=(0.0, 0.0, 0.0), fov=60.0)
    return dict(verts=np.ascontiguousarray(verts), mat_idx=np.zeros(12, np.uint32), mats=mats, camera=camera)


# ----------------------------------------------------------------------------- displaced scene
_ICO_V = None


def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                  (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
                  (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)
    return v, f


def geodesic_grid(freq: int):
    """Grid points of a unit geodesic icosphere: each icosahedron face split
    into a freq x freq triangular grid projected onto the sphere.  Returns
    (points [20, P, 3] float64, local triangles [freq^2, 3] indices into a
    face's points)."""
    v, f = _icosahedron()
    i, j = np.meshgrid(np.arange(freq + 1), np.arange(freq + 1), indexing="ij")
    keep = (i + j) <= freq
    i, j = i[keep], j[keep]
    lut = -np.ones((freq + 1, freq + 1), np.int64)
    lut[i, j] = np.arange(i.size)
    # grid triangles: up (i,j),(i+1,j),(i,j+1); down (i+1,j),(i+1,j+1),(i,j+1)
    ui, uj = np.meshgrid(np.arange(freq), np.arange(freq), indexing="ij")
    up = (ui + uj) <= freq - 1
    dn = (ui + uj) <= freq - 2
    tri_up = np.stack([lut[ui[up], uj[up]], lut[ui[up] + 1, uj[up]], lut[ui[up], uj[up] + 1]], 1)
    tri_dn = np.stack([lut[ui[dn] + 1, uj[dn]], lut[ui[dn] + 1, uj[dn] + 1], lut[ui[dn], uj[dn] + 1]], 1)
    local = np.concatenate([tri_up, tri_dn])
    pts = np.empty((len(f), i.size, 3))
    for k, (a, b, c) in enumerate(f):
        A, B, C = v[a], v[b], v[c]
        P = A + np.outer(i / freq, B - A) + np.outer(j / freq, C - A)
        pts[k] = P / np.linalg.norm(P, axis=1, keepdims=True)
    return pts, local


def grid_triangles(pts, local):
    """De-indexed triangles [20 * len(local), 3, 3] wound away from the origin."""
    T = pts[:, local].reshape(-1, 3, 3)
    n = np.cross(T[:, 1] - T[:, 0], T[:, 2] - T[:, 0])
    flip = np.einsum("ij,ij->i", n, T.mean(axis=1)) < 0
    T[flip] = T[flip][:, [0, 2, 1]]
    return T


def geodesic_sphere(freq: int):
    """Unit geodesic icosphere, 20 * freq^2 triangles wound outward, float64 [n, 3, 3]."""
    return grid_triangles(*geodesic_grid(freq))


def _lattice_value(ix, iy, iz, seed):
    """Hash of integer lattice points to [-1, 1] (splitmix64-style finaliser)."""
    h = (ix.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)) ^ (iy.astype(np.uint64) * np.uint64(0xC2B2AE3D27D4EB4F)) \
        ^ (iz.astype(np.uint64) * np.uint64(0x165667B19E3779F9)) ^ np.uint64(seed * 0x27D4EB2F165667C5 & 0xFFFFFFFFFFFFFFFF)
    h ^= h >> np.uint64(30)
    h *= np.uint64(0xBF58476D1CE4E5B9)
    h ^= h >> np.uint64(27)
    h *= np.uint64(0x94D049BB133111EB)
    h ^= h >> np.uint64(31)
    return (h >> np.uint64(11)).astype(np.float64) / float(1 << 53) * 2.0 - 1.0


def value_noise(p, seed):
    """Trilinear value noise with smoothstep weights, in [-1, 1]."""
    with np.errstate(over="ignore"):
        fl = np.floor(p)
        f = p - fl
        w = f * f * (3.0 - 2.0 * f)
        i0 = fl.astype(np.int64)
        acc = 0.0
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    val = _lattice_value(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz, seed)
                    wx = w[:, 0] if dx else 1.0 - w[:, 0]
                    wy = w[:, 1] if dy else 1.0 - w[:, 1]
                    wz = w[:, 2] if dz else 1.0 - w[:, 2]
                    acc = acc + val * wx * wy * wz
    return acc


def fbm(p, octaves=6, seed=7, base=2.0):
    """Sum of octaves of value noise, gain 1/2, lacunarity 2, normalised to [-1, 1]."""
    total, norm, amp, freq = 0.0, 0.0, 1.0, base
    for o in range(octaves):
        total = total + amp * value_noise(p * freq, seed + 101 * o)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def displaced_scene(freq=458, amplitude=0.05, seed=7, light_freq=8, n_materials=1024):
    """The displaced-mesh scene: a geodesic icosphere (20 * freq^2 triangles;
    freq = 458 gives 4,195,280, the icosphere count nearest 4,194,304) displaced
    radially by fBm (6 octaves, amplitude 0.05, seed 7), on a 2-triangle
    ground quad; per-triangle materials drawn by seed from a palette (60%
    Lambert albedo U[0.1, 0.9], 25% GGX metal roughness U[0.05, 0.5], 15%
    dielectric IOR 1.5); one emissive sphere light (tessellated, centre
    (2.5, 3.0, -1.5), radius 0.5, radiance 20 x (1, 0.95, 0.9)); constant
    environment of radiance 1 (a 1x1 skybox)."""
    cache = _cache_path("displaced", freq, amplitude, seed, light_freq, n_materials)
    if cache and os.path.exists(cache):
        with np.load(cache) as z:
            out = {k: z[k] for k in ("verts", "mat_idx", "mats", "skybox")}
        out.update(camera=dict(position=(0.0, 0.25, -3.4), rotation=(0.0, 0.0, 0.0), fov=45.0),
                   width=1920, height=1080, spp=256, max_bounces=16)
        return out
    rng = np.random.default_rng(seed)
    pts, local = geodesic_grid(freq)  # displacement on the unique grid points
    flat = pts.reshape(-1, 3)
    flat = flat * (1.0 + amplitude * fbm(flat, 6, seed))[:, None]
    sphere = grid_triangles(flat.reshape(pts.shape), local).reshape(-1, 9)
    ground = np.asarray(_quad([(-12, -1.1, -12), (12, -1.1, -12), (12, -1.1, 12), (-12, -1.1, 12)], (0, 1, 0)))
    L = geodesic_sphere(light_freq).reshape(-1, 3) * 0.5 + np.array([2.5, 3.0, -1.5])
    light = L.reshape(-1, 9)
    verts = np.concatenate([sphere, ground, light]).astype(np.float32)
    # palette: Lambert, GGX metal, glass; then ground and light materials
    n_l, n_g = int(n_materials * 0.6), int(n_materials * 0.25)
    n_d = n_materials - n_l - n_g
    rows = []
    for _ in range(n_l):
        rows.append({"colour": tuple(rng.uniform(0.1, 0.9, 3)) + (1.0,)})
    for _ in range(n_g):
        rows.append({"shade_type": SHADE_METAL, "roughness": float(rng.uniform(0.05, 0.5)),
                     "colour": tuple(rng.uniform(0.5, 1.0, 3)) + (1.0,)})
    for _ in range(n_d):
        rows.append({"shade_type": SHADE_GLASS, "ior": 1.5, "colour": (1.0, 1.0, 1.0, 1.0)})
    ground_m = len(rows)
    rows.append({"colour": (0.5, 0.5, 0.5, 1.0)})
    light_m = len(rows)
    rows.append({"colour": (1.0, 0.95, 0.9, 1.0), "emission": 20.0})
    mats = material_table(rows)
    ns = sphere.shape[0]
    u = rng.random(ns)
    cat = np.where(u < 0.6, 0, np.where(u < 0.85, 1, 2))
    pick = rng.random(ns)
    base = np.array([0, n_l, n_l + n_g])
    size = np.array([n_l, n_g, n_d])
    mat_idx = np.concatenate([
        (base[cat] + np.minimum((pick * size[cat]).astype(np.int64), size[cat] - 1)).astype(np.uint32),
        np.full(2, ground_m, np.uint32),
        np.full(light.shape[0], light_m, np.uint32),
    ])
    camera = dict(position=(0.0, 0.25, -3.4), rotation=(0.0, 0.0, 0.0), fov=45.0)
    sky = np.ones((1, 1, 4), np.float32)
    out = dict(verts=np.ascontiguousarray(verts), mat_idx=mat_idx, mats=mats, camera=camera, skybox=sky,
               width=1920, height=1080, spp=256, max_bounces=16)
    if cache:
        os.makedirs(os.path.dirname(cache), exist_ok=True)
        tmp = cache + f".{os.getpid()}.npz"
        np.savez(tmp, verts=out["verts"], mat_idx=mat_idx, mats=mats, skybox=sky)
        os.replace(tmp, cache)
    return out


def _cache_path(*key):
    """Scenes are pure functions of their parameters; a generated one may be
    kept under $CRG_SCENE_CACHE (default /tmp/crg_scene_cache) for reuse by
    later processes.  CRG_SCENE_CACHE="" disables the cache."""
    root = os.environ.get("CRG_SCENE_CACHE", "/tmp/crg_scene_cache")
    if not root:
        return None
    return os.path.join(root, "_".join(str(k) for k in key) + ".npz")


def batch_views(n=64, seed=3):
    """The batched-render workload: n views, each drawing its scene from
    {box, displaced}, its resolution from {128^2, 256^2, 512^2, 1024x768,
    1920x1080} and its spp from {16, 64, 256}, with the camera on a seeded orbit
    (box: an arc in front of the open face; displaced: around the sphere).
    Returns [(scene_index, camera dict, dict(width, height, spp, max_bounces))];
    scene 0 = box_scene(), 1 = displaced_scene()."""
    rng = np.random.default_rng(seed)
    res = [(128, 128), (256, 256), (512, 512), (1024, 768), (1920, 1080)]
    spps = [16, 64, 256]
    out = []
    for _ in range(n):
        scene = int(rng.integers(2))
        w, h = res[int(rng.integers(len(res)))]
        spp = spps[int(rng.integers(len(spps)))]
        a = float(rng.uniform(-25.0, 25.0)) if scene == 0 else float(rng.uniform(-180.0, 180.0))
        b = float(rng.uniform(-6.0, 6.0)) if scene == 0 else float(rng.uniform(-20.0, 10.0))
        ra, rb = math.radians(a), math.radians(b)
        fwd = np.array([math.sin(ra) * math.cos(rb), -math.sin(rb), math.cos(ra) * math.cos(rb)])
        if scene == 0:
            pos = np.array([0.5, 0.5, 0.5]) - 1.9 * fwd
            cam = dict(position=tuple(pos), rotation=(a, b, 0.0), fov=40.0)
            mb = 8
        else:
            pos = -3.4 * fwd
            cam = dict(position=tuple(pos), rotation=(a, b, 0.0), fov=45.0)
            mb = 16
        out.append((scene, cam, dict(width=w, height=h, spp=spp, max_bounces=mb)))
    return out


def inverse_box(albedo=None, light_colour=None):
    """Inverse-rendering scene: the box scene with one material per
    non-emitting triangle (34 albedos, RGB) and one light material of emission
    17 whose colour sets the radiance (17 x colour; the emitter's colour is
    also its albedo, as in the reference).  With no arguments the parameters
    are the box scene's true ones; `albedo` [34, 3] and `light_colour` [3]
    override them (the optimisation starts from albedo 0.5 and radiance 10,
    i.e. light colour 10/17)."""
    base = box_scene()
    true_alb = base["mats"]["colour"][base["mat_idx"][:34], :3].astype(np.float64)
    alb = true_alb if albedo is None else np.asarray(albedo, np.float64).reshape(34, 3)
    lc = np.ones(3) if light_colour is None else np.asarray(light_colour, np.float64).reshape(3)
    rows = [{"colour": tuple(alb[i]) + (1.0,)} for i in range(34)]
    rows.append({"colour": tuple(lc) + (1.0,), "emission": 17.0})
    mat_idx = np.concatenate([np.arange(34, dtype=np.uint32), np.full(2, 34, np.uint32)])
    return dict(verts=base["verts"], mat_idx=mat_idx, mats=material_table(rows), camera=base["camera"],
                true_albedo=true_alb, true_light=np.ones(3))
