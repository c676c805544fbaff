"""A second, independent restatement of the EXTENDED estimator, in FP64 numpy
from its published methods: emissive-triangle next-event estimation with a
power-proportional emitter pick (Walker's alias table, Vose's construction),
uniform points on the picked triangle, two-sided emitters and power-heuristic
MIS (Veach 1997) against BSDF sampling; cosine-weighted Lambert sampling in the
Duff et al. (2017) frame of the geometric normal (the reference scatters into that
hemisphere, src/render/renderer.cpp:93-97); GGX metal with visible-normal
sampling (Heitz 2018), Smith G and Schlick F; a dielectric choosing reflection
by the exact Fresnel term; Russian roulette from a set depth with survival
min(max(throughput), 0.95).  It draws the oracle's random numbers (group 1 + 2i:
BSDF u1, u2, the Fresnel choice, roulette; group 2 + 2i: emitter column, point
on the triangle, alias test), so every one-sample pixel of the oracle's film
must equal it up to FP32 rounding, except where a branch decision sits within
rounding of its threshold."""
import numpy as np
import pytest

from crender_gb300 import api, scenes
from test_faithful_restatement_cpu import closest, reflect
from test_oracle import _camera_f64, pcg4d_py

TMIN = 1e-5


def alias_table(w):
    """Vose's alias construction with last-in-first-out worklists filled in index order."""
    n = len(w)
    q = [wi * n / sum(w) for wi in w]
    prob, alias = [1.0] * n, list(range(n))
    small = [i for i in range(n) if q[i] < 1.0]
    large = [i for i in range(n) if q[i] >= 1.0]
    while small and large:
        s, g = small.pop(), large.pop()
        prob[s], alias[s] = q[s], g
        q[g] = (q[g] + q[s]) - 1.0
        (small if q[g] < 1.0 else large).append(g)
    return np.float32(prob), alias


def frame(n):
    """Duff et al. 2017: (t, b) completing n to a right-handed orthonormal basis."""
    s = -1.0 if n[2] < 0 else 1.0
    a = -1.0 / (s + n[2])
    b = n[0] * n[1] * a
    return np.array([1 + s * n[0] * n[0] * a, s * b, -s * n[0]]), np.array([b, s + n[1] * n[1] * a, -n[1]])


def ggx_d(nh, a):
    return a * a / (np.pi * (nh * nh * (a * a - 1) + 1) ** 2)


def ggx_lambda(w, a):
    return 0.5 * (np.sqrt(1 + a * a * (w[0] ** 2 + w[1] ** 2) / w[2] ** 2) - 1)


def schlick(f0, c):
    return f0 + (1 - f0) * (1 - np.clip(c, 0, 1)) ** 5


def vndf(wo, a, u1, u2):
    """Heitz 2018, "Sampling the GGX Distribution of Visible Normals"."""
    vh = np.array([a * wo[0], a * wo[1], wo[2]])
    vh /= np.linalg.norm(vh)
    l2 = vh[0] ** 2 + vh[1] ** 2
    t1v = np.array([-vh[1], vh[0], 0.0]) / np.sqrt(l2) if l2 > 0 else np.array([1.0, 0, 0])
    t2v = np.cross(vh, t1v)
    r, phi = np.sqrt(u1), 2 * np.pi * u2
    t1, t2 = r * np.cos(phi), r * np.sin(phi)
    sw = 0.5 * (1 + vh[2])
    t2 = (1 - sw) * np.sqrt(1 - t1 * t1) + sw * t2
    nh = t1 * t1v + t2 * t2v + np.sqrt(max(0.0, 1 - t1 * t1 - t2 * t2)) * vh
    h = np.array([a * nh[0], a * nh[1], max(0.0, nh[2])])
    return h / np.linalg.norm(h)


def fresnel(ci, eta):
    ci = min(max(ci, 0.0), 1.0)
    st2 = eta * eta * (1 - ci * ci)
    if st2 >= 1:
        return 1.0, st2
    ct = np.sqrt(1 - st2)
    rs = (eta * ci - ct) / (eta * ci + ct)
    rp = (ci - eta * ct) / (ci + eta * ct)
    return 0.5 * (rs * rs + rp * rp), st2


class Lights:
    def __init__(self, V, mats, mi):
        lum = {}
        for k, m in enumerate(mats):
            if m["emission"] > 0:
                c = m["colour"].astype(np.float64) * float(m["emission"])
                lum[k] = 0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2]
        self.prim = [p for p in range(len(V)) if int(mi[p]) in lum]
        area = [0.5 * np.linalg.norm(np.cross(V[p, 1] - V[p, 0], V[p, 2] - V[p, 0])) for p in self.prim]
        w = [a * lum[int(mi[p])] for a, p in zip(area, self.prim)]
        total = sum(w)
        self.prob, self.alias = alias_table(w)
        self.area_pdf = {k: v / total for k, v in lum.items()}  # pick probability / area, per material

    def pick(self, u1, u2):
        n = len(self.prim)
        j = min(int(np.float32(u1) * np.float32(n)), n - 1)
        return j if u2 < self.prob[j] else self.alias[j]


def occluded(o, d, tmax, V):
    t, _ = closest(o, d, V)
    return t < tmax


def nee(ctx, i, p, n, T, bsdf, V):
    sc, L, (pix, s, seed) = ctx["sc"], ctx["lights"], ctx["key"]
    g = pcg4d_py([pix, s, 2 + 2 * i, seed])
    prim = L.prim[L.pick(g[0], g[3])]
    a, b, c = V[prim]
    su = np.sqrt(g[1])
    pl = a * (1 - su) + b * (su * (1 - g[2])) + c * (su * g[2])
    po = p + n * 1e-4
    w = pl - po
    d2 = w @ w
    dist = np.sqrt(d2)
    wi = w / dist
    cos_s = wi @ n
    if cos_s <= 0:
        return np.zeros(3)
    ng = np.cross(b - a, c - a)
    cos_l = abs((ng / np.linalg.norm(ng)) @ wi)
    if cos_l <= 0 or occluded(po, wi, dist * 0.999, V):
        return np.zeros(3)
    m = sc["mats"][sc["mat_idx"][prim]]
    Le = m["colour"][:3].astype(np.float64) * float(m["emission"])
    p_light = L.area_pdf[int(sc["mat_idx"][prim])] * d2 / cos_l
    if bsdf["kind"] == "lambert":
        f, p_bsdf, cos_i = bsdf["albedo"] / np.pi, cos_s / np.pi, cos_s
    else:
        t_, b_, wol, al = bsdf["t"], bsdf["b"], bsdf["wol"], bsdf["alpha"]
        wil = np.array([wi @ t_, wi @ b_, wi @ n])
        if wil[2] <= 0:
            return np.zeros(3)
        h = (wol + wil) / np.linalg.norm(wol + wil)
        D = ggx_d(h[2], al)
        lo, li = ggx_lambda(wol, al), ggx_lambda(wil, al)
        f = schlick(bsdf["f0"], wol @ h) * D / (1 + lo + li) / (4 * wol[2] * wil[2])
        p_bsdf, cos_i = D / (1 + lo) / (4 * wol[2]), wil[2]
    w_mis = p_light ** 2 / (p_light ** 2 + p_bsdf ** 2)
    return T * f * Le * cos_i * w_mis / p_light


def sample(sc, st, px, py, s, env):
    W, H = st.width, st.height
    pix = py * W + px
    V = sc["verts"].astype(np.float64).reshape(-1, 3, 3)
    mats, mi = sc["mats"], sc["mat_idx"]
    ctx = dict(sc=sc, lights=sc["_lights"], key=(pix, s, st.seed))
    g0 = pcg4d_py([pix, s, 0, st.seed])
    o, d = _camera_f64(sc["camera"], (px + g0[0]) / W, (py + g0[1]) / H, st.aspect)
    T, L = np.ones(3), np.zeros(3)
    prev_pdf, prev_delta = 0.0, True
    for i in range(st.max_bounces):
        t, prim = closest(o, d, V)
        if prim < 0:
            L = L + T * env
            break
        p = o + t * d
        a, b, c = V[prim]
        ng = np.cross(b - a, c - a)
        ng /= np.linalg.norm(ng)
        m = mats[mi[prim]]
        rgb = m["colour"][:3].astype(np.float64)
        cos_nd = ng @ d
        n = ng if cos_nd < 0 else -ng
        if m["emission"] > 0:
            Le = rgb * float(m["emission"])
            if prev_delta:
                L = L + T * Le
            else:
                pl = ctx["lights"].area_pdf[int(mi[prim])] * t * t / abs(cos_nd)
                L = L + T * Le * prev_pdf ** 2 / (prev_pdf ** 2 + pl ** 2)
        g = pcg4d_py([pix, s, 1 + 2 * i, st.seed])
        more = i + 1 < st.max_bounces
        if m["shade_type"] == scenes.SHADE_SMOOTH:
            tt, bb = frame(ng)
            if more:
                L = L + nee(ctx, i, p, ng, T, dict(kind="lambert", albedo=rgb), V)
            r, phi = np.sqrt(g[0]), 2 * np.pi * g[1]
            lz = np.sqrt(max(0.0, 1 - g[0]))
            d = tt * r * np.cos(phi) + bb * r * np.sin(phi) + ng * lz
            o = p + ng * 1e-4
            prev_pdf, prev_delta = lz / np.pi, False
            T = T * rgb
        elif m["shade_type"] == scenes.SHADE_METAL:
            f0, al = rgb * float(m["reflectiveness"]), float(m["roughness"])
            tt, bb = frame(n)
            wo = -d
            wol = np.array([wo @ tt, wo @ bb, wo @ n])
            if wol[2] <= 0:
                break
            if more:
                L = L + nee(ctx, i, p, n, T, dict(kind="ggx", f0=f0, t=tt, b=bb, wol=wol, alpha=al), V)
            h = vndf(wol, al, g[0], g[1])
            woh = wol @ h
            wil = 2 * woh * h - wol
            if wil[2] <= 0:
                break
            lo, li = ggx_lambda(wol, al), ggx_lambda(wil, al)
            T = T * schlick(f0, woh) * (1 + lo) / (1 + lo + li)
            prev_pdf, prev_delta = ggx_d(h[2], al) / (1 + lo) / (4 * wol[2]), False
            d = tt * wil[0] + bb * wil[1] + n * wil[2]
            o = p + n * 1e-4
        else:
            eta = 1 / float(m["ior"]) if cos_nd < 0 else float(m["ior"])
            ci = -(d @ n)
            F, st2 = fresnel(ci, eta)
            if g[2] < F:
                d, o = reflect(d, n), p + n * 1e-4
            else:
                d = d * eta + n * (eta * min(max(ci, 0.0), 1.0) - np.sqrt(1 - st2))
                o = p - n * 1e-4
            T = T * rgb
            prev_delta = True
        if st.rr_depth > 0 and i + 1 >= st.rr_depth:
            q = min(T.max(), 0.95)
            if g[3] >= q:
                break
            T = T / q
    return L


def scene(kind):
    sc = scenes.box_scene()
    if kind == "materials":
        mats = scenes.material_table([
            {"colour": (0.73, 0.73, 0.73, 1.0)},
            {"colour": (0.63, 0.065, 0.05, 1.0)},
            {"colour": (0.14, 0.45, 0.09, 1.0)},
            {"colour": (1.0, 1.0, 1.0, 1.0), "emission": 17.0},
            {"colour": (1.0, 1.0, 1.0, 1.0), "shade_type": scenes.SHADE_GLASS, "ior": 1.5},
            {"colour": (0.9, 0.8, 0.5, 1.0), "shade_type": scenes.SHADE_METAL, "roughness": 0.3},
        ])
        mi = sc["mat_idx"].copy()
        mi[10:22] = 4
        mi[22:34] = 5
        v = sc["verts"].copy().reshape(-1, 3, 3)
        v[10:34, :, 1] += np.float32(1e-3)  # off the floor: no coplanar ties (see the faithful restatement)
        sc = dict(sc, verts=np.ascontiguousarray(v.reshape(-1, 9)), mats=mats, mat_idx=mi)
    V = sc["verts"].astype(np.float64).reshape(-1, 3, 3)
    return dict(sc, _lights=Lights(V, sc["mats"], sc["mat_idx"]))


@pytest.mark.parametrize("kind,rr,seed,env", [("plain", 3, 11, 0.0), ("plain", 0, 12, 0.25),
                                              ("materials", 3, 13, 0.0), ("materials", 2, 14, 0.4)])
def test_oracle_samples_equal_the_extended_restatement(orc, kind, rr, seed, env):
    sc = scene(kind)
    W, H = 24, 16
    st = api.make_settings(W, H, 1, 8, rr, 1, seed, W / H)
    sky = np.full((1, 1, 4), env, np.float32) if env else None
    desc = {k: v for k, v in sc.items() if not k.startswith("_")}
    film = orc.render(desc, sc["camera"], st, skybox=sky)["sum64"].reshape(H, W, 3)
    close, lit = 0, 0
    for py in range(H):
        for px in range(W):
            want = sample(sc, st, px, py, 0, env)
            got = film[H - 1 - py, W - 1 - px]
            lit += bool(want.any())
            close += bool(np.allclose(got, want, rtol=1e-4, atol=1e-6))
    assert lit > W * H // 3
    assert close >= 0.98 * W * H, f"{W * H - close} of {W * H} pixels differ"
