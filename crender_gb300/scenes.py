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
