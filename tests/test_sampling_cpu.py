"""The estimators' sampling helpers, as the oracle computes them, against their
published definitions: the uniform sphere of cr::sampling::sphere
(src/util/sampling.h:156-166), the orthonormal frame of cr::sampling::build_local
(sampling.h:21-33, Duff et al. 2017), the GGX distribution of specular_d
(sampling.h:93-106) with the Smith Lambda of the same distribution, visible-normal
sampling (Heitz 2018) and the exact dielectric Fresnel equations.  The library's
kernels use the same expressions, and their renders equal the oracle's bit for bit,
so these checks pin both."""
import numpy as np
import pytest
from scipy import integrate

F3 = np.zeros(3, np.float32)


def sphere(orc, u1, u2):
    orc.lib().orc_sample_sphere(float(u1), float(u2), F3.ctypes.data)
    return F3.astype(np.float64)


def test_sphere_covers_the_sphere_uniformly(orc):
    n = 64
    u = (np.arange(n) + 0.5) / n
    pts = np.array([sphere(orc, a, b) for a in u for b in u])
    assert np.allclose(np.linalg.norm(pts, axis=1), 1.0, atol=1e-6)
    # the polar coordinate is 2 u1 - 1 exactly (Archimedes: uniform in height)
    assert np.array_equal(pts[:, 1].reshape(n, n)[:, 0].astype(np.float32), (2 * u - 1).astype(np.float32))
    assert np.abs(pts.mean(axis=0)).max() < 1e-3
    octant = (pts[:, 0] > 0) * 4 + (pts[:, 1] > 0) * 2 + (pts[:, 2] > 0)
    assert np.allclose(np.bincount(octant, minlength=8) / len(pts), 1 / 8, atol=0.01)


def test_build_local_is_orthonormal_and_right_handed(orc):
    r = np.random.default_rng(1)
    ns = r.normal(size=(2000, 3))
    ns = np.concatenate([ns, [[0, 0, 1], [0, 0, -1], [1e-4, 0, -1], [0, 1e-4, 1], [1, 0, 0], [0, -1, 0]]])
    ns = (ns / np.linalg.norm(ns, axis=1, keepdims=True)).astype(np.float32)
    t, b = np.zeros(3, np.float32), np.zeros(3, np.float32)
    for n in ns:
        n = np.ascontiguousarray(n)
        orc.lib().orc_build_local(n.ctypes.data, t.ctypes.data, b.ctypes.data)
        T, B, N = t.astype(np.float64), b.astype(np.float64), n.astype(np.float64)
        for v in (T, B):
            assert abs(np.linalg.norm(v) - 1) < 2e-6
        assert max(abs(T @ N), abs(B @ N), abs(T @ B)) < 2e-6
        assert np.cross(T, B) @ N > 0.999999


def ggx_d64(mu, a):
    """Trowbridge-Reitz / GGX normal distribution for cos(theta_h) = mu."""
    a2 = a * a
    return a2 / (np.pi * (mu * mu * (a2 - 1) + 1) ** 2)


def ggx_lambda64(w, a):
    """Smith Lambda of the GGX distribution: (-1 + sqrt(1 + a^2 tan^2 theta)) / 2."""
    t2 = (w[0] ** 2 + w[1] ** 2) / w[2] ** 2
    return 0.5 * (np.sqrt(1 + a * a * t2) - 1)


@pytest.mark.filterwarnings("ignore::scipy.integrate.IntegrationWarning")  # float32 integrand: roundoff-limited
@pytest.mark.parametrize("alpha", [0.05, 0.2, 0.5, 1.0])
def test_ggx_d_matches_definition_and_is_normalised(orc, alpha):
    mus = np.linspace(0.0, 1.0, 201, dtype=np.float32)
    got = np.array([orc.lib().orc_ggx_d(float(m), alpha) for m in mus])
    want = ggx_d64(mus.astype(np.float64), np.float64(np.float32(alpha)))
    # the reference's form (mu a^2 - mu) mu + 1 cancels to a^2 near mu = 1: float error ~ eps / a^2
    assert np.allclose(got, want, rtol=max(2e-6, 4e-7 / alpha ** 2), atol=0)
    # projected-area normalisation: 2 pi * integral_0^1 D(mu) mu dmu = 1
    val, _ = integrate.quad(lambda m: orc.lib().orc_ggx_d(m, alpha) * m, 0.0, 1.0, points=[1 - alpha * alpha],
                            limit=400, epsabs=1e-9)
    assert abs(2 * np.pi * val - 1) < 1e-4


def test_smith_lambda_matches_definition(orc):
    r = np.random.default_rng(2)
    for _ in range(500):
        a = float(np.float32(r.uniform(0.02, 1.0)))
        w = r.normal(size=3)
        w[2] = abs(w[2]) + 1e-3
        w = (w / np.linalg.norm(w)).astype(np.float32)
        got = orc.lib().orc_ggx_lambda(np.ascontiguousarray(w).ctypes.data, a)
        want = ggx_lambda64(w.astype(np.float64), a)
        assert abs(got - want) <= 1e-5 * max(1.0, want)
    up = np.array([0, 0, 1], np.float32)
    assert orc.lib().orc_ggx_lambda(up.ctypes.data, 0.3) == 0.0


def vndf_pdf(h, wo, a):
    """Distribution of visible normals: G1(wo) max(0, wo.h) D(h) / wo.z."""
    g1 = 1 / (1 + ggx_lambda64(wo, a))
    return g1 * np.maximum(0.0, h @ wo) * ggx_d64(h[..., 2], a) / wo[2]


def moment(f, wo, a):
    """integral of f(h) * vndf(h) over the upper hemisphere, in (theta, phi)."""
    def integrand(phi, th):
        h = np.array([np.sin(th) * np.cos(phi), np.sin(th) * np.sin(phi), np.cos(th)])
        return f(h) * vndf_pdf(h, wo, a) * np.sin(th)
    return integrate.dblquad(integrand, 0, np.pi / 2, 0, 2 * np.pi, epsabs=1e-7, epsrel=1e-6)[0]


@pytest.mark.parametrize("alpha,theta_o", [(0.3, 0.2), (0.6, 1.2), (0.15, 1.45)])
def test_vndf_samples_follow_the_visible_normal_distribution(orc, alpha, theta_o):
    a = float(np.float32(alpha))
    wo = np.array([np.sin(theta_o) * np.cos(0.7), np.sin(theta_o) * np.sin(0.7), np.cos(theta_o)], np.float32)
    wo64 = wo.astype(np.float64)
    assert abs(moment(lambda h: 1.0, wo64, a) - 1) < 1e-4  # the density itself integrates to 1
    u = np.random.default_rng(3).random((40_000, 2)).astype(np.float32)
    hs = np.zeros((len(u), 3))
    h3 = np.zeros(3, np.float32)
    for i, (u1, u2) in enumerate(u):
        orc.lib().orc_sample_vndf(wo.ctypes.data, a, float(u1), float(u2), h3.ctypes.data)
        hs[i] = h3
    assert np.allclose(np.linalg.norm(hs, axis=1), 1, atol=2e-6)
    assert (hs[:, 2] >= 0).all()
    assert (hs @ wo64 > -1e-6).all()  # only normals facing the viewer are sampled
    for f in (lambda h: h[..., 0], lambda h: h[..., 1], lambda h: h[..., 2], lambda h: h[..., 2] ** 2,
              lambda h: h[..., 0] * h[..., 2]):
        vals = f(hs)
        se = vals.std() / np.sqrt(len(vals))
        assert abs(vals.mean() - moment(f, wo64, a)) < 5 * se + 1e-6


def fresnel64(ci, eta):
    """Unpolarised dielectric reflectance from the angle form of the Fresnel
    equations, eta = n_i / n_t: Rs = sin^2(ti - tt) / sin^2(ti + tt),
    Rp = tan^2(ti - tt) / tan^2(ti + tt), total reflection when eta sin(ti) > 1."""
    ti = np.arccos(ci)
    st = eta * np.sin(ti)
    if st >= 1:
        return 1.0
    tt = np.arcsin(st)
    rs = (np.sin(ti - tt) / np.sin(ti + tt)) ** 2
    rp = (np.tan(ti - tt) / np.tan(ti + tt)) ** 2
    return 0.5 * (rs + rp)


@pytest.mark.parametrize("eta", [1 / 1.5, 1.5, 1 / 1.33, 1.33])
def test_fresnel_matches_the_angle_form(orc, eta):
    e = float(np.float32(eta))
    assert abs(orc.lib().orc_fresnel_dielectric(1.0, e) - ((1 - e) / (1 + e)) ** 2) < 1e-6
    for ci in np.linspace(0.02, 0.98, 97):
        ci = float(np.float32(ci))
        assert abs(orc.lib().orc_fresnel_dielectric(ci, e) - fresnel64(ci, e)) < 2e-5
    if e > 1:  # from the dense side: total internal reflection below the critical cosine
        crit = np.sqrt(1 - 1 / (e * e))
        assert orc.lib().orc_fresnel_dielectric(float(crit) * 0.99, e) == 1.0
        assert orc.lib().orc_fresnel_dielectric(0.0, e) == 1.0
    else:
        assert abs(orc.lib().orc_fresnel_dielectric(0.0, e) - 1.0) < 1e-6  # grazing incidence reflects all
