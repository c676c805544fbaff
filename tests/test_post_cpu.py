"""Post-processing oracle (cr::post_processor::process, src/render/post/post_processor.cpp:110-307):
pinned against an independent numpy restatement of the same passes, and against
known answers of the blur (impulse response = the separable 15-tap kernel applied
five times in each direction) and of the reference's coverage quirks."""
import numpy as np
import pytest

from crender_gb300 import _abi

W8 = np.array([0.19744746769063704, 0.1746973469158936, 0.12099884565428047, 0.06560233156931679,
               0.027839605612666265, 0.009246250740395456, 0.002403157286908872, 0.00048872837522002], np.float32)


def settings(**kw):
    s = _abi.PostSettings(0, 0.7, 1.0, 0, 0, 0, 1.0, 2.2, 0, 0)
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def shift(a, dx, dy):
    """b[y, x] = a[y + dy, x + dx], zero outside (texelFetch with zero fill)."""
    h, w = a.shape[:2]
    b = np.zeros_like(a)
    ys, yd = (slice(dy, h), slice(0, h - dy)) if dy >= 0 else (slice(0, h + dy), slice(-dy, h))
    xs, xd = (slice(dx, w), slice(0, w - dx)) if dx >= 0 else (slice(0, w + dx), slice(-dx, w))
    b[yd, xd] = a[ys, xs]
    return b


def np_post(img, s, visited=None):
    """numpy restatement: float32 operations in the shaders' order.  `visited`
    overrides the set of pixels the brightness pass thresholds."""
    img = img.astype(np.float32)
    h, w = img.shape[:2]
    if not (s.bloom or s.gray_scale or s.tonemapping):
        return img.copy()
    faithful = s.mode == 0
    rw, rh = (w // 8 * 8, h // 8 * 8) if faithful else (w, h)
    region = np.zeros((h, w), bool)
    region[:rh, :rw] = True
    f = img[..., :3].copy()
    if s.bloom:
        if visited is None:
            i = np.arange(w * h)
            xs, ys = i % w, (i // h if faithful else i // w)
            ok = ys < h
            visited = np.zeros((h, w), bool)
            visited[ys[ok], xs[ok]] = True
        lum = (img[..., 0] * np.float32(0.2126) + img[..., 1] * np.float32(0.7152)) + img[..., 2] * np.float32(0.0722)
        zero = visited & (lum < np.float32(s.bloom_threshold))
        buf = img[..., :3].copy()
        buf[zero] = 0
        for p in range(10):
            hor = p % 2 == 0
            out = buf * W8[0]
            for k in range(1, 8):
                a = shift(buf, k, 0) if hor else shift(buf, 0, k)
                d = shift(buf, -k, 0) if hor else shift(buf, 0, -k)
                out = out + a * W8[k]
                out = out + d * W8[k]
            out[~region] = 0
            buf = out
        f = f + buf * np.float32(s.bloom_strength)
    if s.gray_scale:
        g = (np.float32(0.2126) * f[..., 0] + np.float32(0.7162) * f[..., 1]) + np.float32(0.0722) * f[..., 2]
        f = np.stack([g, g, g], -1)
    if s.tonemapping:
        e, ig = np.float32(s.exposure), np.float32(1.0) / np.float32(s.gamma)
        c = f * e
        if s.tonemap_type == 0:
            f = np.power(c, ig)
        elif s.tonemap_type == 1:
            f = np.power(c / (c + np.float32(1)), ig)
        elif s.tonemap_type == 2:
            x = np.maximum(np.float32(0), c - np.float32(0.004))
            f = (x * (np.float32(6.2) * x + np.float32(0.5))) / (x * (np.float32(6.2) * x + np.float32(1.7)) + np.float32(0.06))
        elif s.tonemap_type == 3:
            A, B, C_, D, E, F = (np.float32(v) for v in (0.15, 0.50, 0.10, 0.20, 0.02, 0.30))

            def m(x):
                return ((x * (A * x + C_ * B) + D * E) / (x * (A * x + B) + D * F)) - E / F

            f = np.power(m(np.float32(2) * c) * (np.float32(1) / m(np.float32(11.2))), ig)
    out = np.zeros_like(img)
    out[..., :3] = f
    out[..., 3] = 1
    out[~region] = 0
    return out


def hdr_image(w, h, seed):
    r = np.random.default_rng(seed)
    img = r.gamma(0.6, 0.8, (h, w, 4)).astype(np.float32)
    img[..., 3] = r.uniform(0, 1, (h, w)).astype(np.float32)
    return img


CASES = [
    dict(bloom=1),
    dict(bloom=1, bloom_threshold=0.2, bloom_strength=0.5),
    dict(gray_scale=1),
    dict(tonemapping=1, tonemap_type=0),
    dict(tonemapping=1, tonemap_type=1, exposure=1.5),
    dict(tonemapping=1, tonemap_type=2),
    dict(tonemapping=1, tonemap_type=3, gamma=2.0),
    dict(tonemapping=1, tonemap_type=7),
    dict(bloom=1, gray_scale=1, tonemapping=1, tonemap_type=1),
]


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("shape", [(32, 32), (40, 24), (37, 19), (16, 48)])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_oracle_matches_numpy_restatement(orc, mode, shape, case):
    w, h = shape
    img = hdr_image(w, h, 3 + case)
    s = settings(mode=mode, **CASES[case])
    got = orc.post_process(img, s)
    want = np_post(img, s)
    assert ulp_diff(got, want) <= (2 if uses_pow(s) else 0)


def uses_pow(s):
    """The gamma step (pow) of the linear, Reinhard and Uncharted curves is the one
    operation two libraries round differently (by at most 2 ulp)."""
    return bool(s.tonemapping) and s.tonemap_type in (0, 1, 3)


def ulp_diff(a, b):
    a = a.view(np.int32).astype(np.int64)
    b = b.view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return int(np.abs(a - b).max())


def test_no_effect_is_a_copy(orc):
    img = hdr_image(13, 7, 1)
    assert np.array_equal(orc.post_process(img, settings()), img)


def test_blur_impulse_response_is_the_separable_kernel(orc):
    """A single bright texel far from the borders blooms into k5 (x) k5, where k5 is
    the 15-tap kernel convolved with itself five times (5 horizontal + 5 vertical
    passes); the kernel sums to 1, so bloom conserves energy."""
    n = 96
    img = np.zeros((n, n, 4), np.float32)
    img[48, 48, :3] = 10.0
    s = settings(bloom=1, bloom_threshold=0.5, bloom_strength=1.0, mode=1)
    out = orc.post_process(img, s)
    k = np.concatenate([W8[:0:-1], W8]).astype(np.float64)
    assert abs(k.sum() - 1.0) < 1e-6
    k5 = k
    for _ in range(4):
        k5 = np.convolve(k5, k)
    want = 10.0 * np.outer(k5, k5)
    bloom = out[..., 0].astype(np.float64).copy()
    bloom[48, 48] -= 10.0  # the source pixel itself
    r = len(k5) // 2
    np.testing.assert_allclose(bloom[48 - r:48 + r + 1, 48 - r:48 + r + 1], want, rtol=2e-5, atol=1e-9)
    assert abs(bloom.sum() - 10.0) < 1e-4


def test_faithful_coverage_quirks(orc):
    """FAITHFUL: pixels beyond 8*floor(W/8) x 8*floor(H/8) come out as zero, and on a
    16x8 image the brightness pass only thresholds (i % 16, i / 8) for i < 64:
    columns 0-7 of even rows and 8-15 of odd rows."""
    img = np.full((12, 20, 4), 0.1, np.float32)
    out = orc.post_process(img, settings(gray_scale=1))
    assert np.all(out[8:] == 0) and np.all(out[:, 16:] == 0) and np.all(out[:8, :16, 3] == 1)
    full = orc.post_process(img, settings(gray_scale=1, mode=1))
    assert np.all(full[..., 3] == 1)

    img = hdr_image(16, 8, 5)
    s = settings(bloom=1, bloom_threshold=1.0)
    visited = np.zeros((8, 16), bool)
    visited[0::2, :8] = True
    visited[1::2, 8:] = True
    assert ulp_diff(orc.post_process(img, s), np_post(img, s, visited)) == 0
    assert ulp_diff(orc.post_process(img, s), np_post(img, s, np.ones((8, 16), bool))) > 0
    s.mode = 1
    assert ulp_diff(orc.post_process(img, s), np_post(img, s, np.ones((8, 16), bool))) == 0
