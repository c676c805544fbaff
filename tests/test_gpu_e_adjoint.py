"""Path-replay adjoint (crg_backward) of the extended estimator.

* equals the oracle's FP64 gradient (same paths, bit-identical contributions;
  only the FP64 summation order differs);
* matches central finite differences with common random numbers (h = 1e-3,
  roulette off) to 1e-3 relative at the inverse-rendering configuration
  (box scene, 256 x 256, 32 spp);
* costs at most 4x the forward pass;
* drives 200 Adam steps (lr 0.02) from albedo 0.5 / radiance 10 towards the
  4096-spp target."""
import ctypes as C
import time

import numpy as np
import pytest

from crender_gb300 import _abi, api, scenes

pytestmark = pytest.mark.gpu


class Problem:
    def __init__(self, ctx, sc, W=256, spp=32, rr=0, seed_fwd=11, seed_bwd=12):
        self.ctx, self.sc, self.W = ctx, sc, W
        self.scene = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(8, 1)
        self.nmat = len(sc["mats"])
        self.fwd = api.make_settings(W, W, spp, 8, rr, 1, seed_fwd)
        self.bwd = api.make_settings(W, W, spp, 8, rr, 1, seed_bwd)
        self.film = api.Film(ctx, W, W, f64=True)
        self.adj = api.DeviceBuffer(ctx, W * W * 12)
        self.gc = api.DeviceBuffer(ctx, self.nmat * 24)
        self.ge = api.DeviceBuffer(ctx, self.nmat * 8)
        self.cam = api.make_camera(sc["camera"])

    def set_mats(self, mats):
        api.set_materials(self.scene, mats)

    def render(self, st, f64=False):
        self.film.reset()
        self.ctx.check(self.ctx.lib.crg_render(self.scene.h, C.byref(self.cam), C.byref(st), self.film.h, None))
        d = self.film.download(f64=f64)
        return (d["sum64"] if f64 else d["sum"].astype(np.float64)) / st.spp

    def backward(self, adj):
        self.adj.upload(np.ascontiguousarray(adj, np.float32))
        zeros_c, zeros_e = np.zeros(self.nmat * 3), np.zeros(self.nmat)
        self.gc.upload(zeros_c)
        self.ge.upload(zeros_e)
        api.backward(self.scene, self.sc["camera"], self.bwd, self.adj, self.gc, self.ge)
        return self.gc.download(zeros_c).reshape(self.nmat, 3), self.ge.download(zeros_e)

    def close(self):
        for b in (self.adj, self.gc, self.ge):
            b.free()
        self.film.close()
        self.scene.close()


def _init_scene():
    return scenes.inverse_box(albedo=np.full((34, 3), 0.5), light_colour=np.full(3, 10 / 17))


def test_matches_oracle_fp64(ctx, orc):
    sc = _init_scene()
    P = Problem(ctx, sc, W=24, spp=16, rr=3)
    try:
        adj = np.random.default_rng(1).uniform(-1, 1, 24 * 24 * 3).astype(np.float32)
        gc, ge = P.backward(adj)
        oc, oe = orc.adjoint(sc, sc["camera"], P.bwd, adj)
        scale = np.abs(oc).max()
        assert scale > 0
        assert np.allclose(gc, oc, rtol=1e-9, atol=1e-12 * scale)
        assert np.allclose(ge, oe, rtol=1e-9, atol=1e-12 * np.abs(oe).max())
    finally:
        P.close()


def test_matches_finite_differences_and_cost(ctx):
    sc = _init_scene()
    P = Problem(ctx, sc)
    try:
        target = scenes.inverse_box()
        T = Problem(ctx, target, spp=256, seed_fwd=99)
        tgt = T.render(T.fwd, f64=True)
        T.close()
        img = P.render(P.fwd, f64=True)
        adj = (2.0 * (img - tgt) / img.size).astype(np.float32)
        gc, ge = P.backward(adj)
        h = 1e-3
        checked = 0
        for m, c in [(0, 0), (3, 1), (6, 0), (8, 2), (14, 1), (26, 0), (34, 0), (34, 2)]:
            mp, mm = sc["mats"].copy(), sc["mats"].copy()
            mp[m]["colour"][c] += h
            mm[m]["colour"][c] -= h
            P.set_mats(mp)
            fp = float(np.dot(adj.astype(np.float64), P.render(P.bwd, f64=True)))
            P.set_mats(mm)
            fm = float(np.dot(adj.astype(np.float64), P.render(P.bwd, f64=True)))
            P.set_mats(sc["mats"])
            fd = (fp - fm) / (2 * h)
            assert abs(gc[m, c]) > 1e-6 * np.abs(gc).max()
            assert abs(gc[m, c] - fd) <= 1e-3 * abs(gc[m, c]), (m, c, gc[m, c], fd)
            checked += 1
        assert checked == 8
        # cost: backward / forward at the same spp
        P.render(P.fwd)
        ctx.sync()
        t0 = time.perf_counter()
        for _ in range(3):
            P.render(P.fwd)
        ctx.sync()
        tf = (time.perf_counter() - t0) / 3
        t0 = time.perf_counter()
        for _ in range(3):
            P.backward(adj)
        ctx.sync()
        tb = (time.perf_counter() - t0) / 3
        assert tb <= 4.0 * tf, (tb, tf)
    finally:
        P.close()


def test_finite_differences_on_every_parameter(ctx, capsys):
    """Central FD with common random numbers on all 105 parameters of the
    inverse problem (34 x RGB albedos, the light's RGB colour) and on the
    light's emission (crg_backward's d_grad_emission), at 256 x 256, 32 spp,
    roulette off.  The forward pass sums float32 per-sample radiance, so an FD
    carries rounding noise of its own: each FD is taken at h and h/2, and a
    parameter passes when it agrees with the adjoint to 1e-3 relative, or
    within its noise floor: three times the h / h-half spread, and at least
    1e-5 of the largest gradient (parameters whose gradient is that small
    lose their digits to the rounding of the other contributions to the same
    pixels)."""
    sc = _init_scene()
    P = Problem(ctx, sc)
    try:
        target = scenes.inverse_box()
        T = Problem(ctx, target, spp=256, seed_fwd=99)
        tgt = T.render(T.fwd, f64=True)
        T.close()
        img = P.render(P.fwd, f64=True)
        adj = (2.0 * (img - tgt) / img.size).astype(np.float32)
        a64 = adj.astype(np.float64)
        gc, ge = P.backward(adj)

        def fd(field, m, c, h):
            mp, mm = sc["mats"].copy(), sc["mats"].copy()
            if field == "colour":
                mp[m]["colour"][c] += h
                mm[m]["colour"][c] -= h
            else:
                mp[m]["emission"] += h
                mm[m]["emission"] -= h
            P.set_mats(mp)
            fp = float(np.dot(a64, P.render(P.bwd, f64=True)))
            P.set_mats(mm)
            fm = float(np.dot(a64, P.render(P.bwd, f64=True)))
            return (fp - fm) / (2 * h)

        rows = []
        for m in range(35):
            for c in range(3):
                rows.append(("colour", m, c, gc[m, c], 1e-3))
        rows.append(("emission", 34, 0, ge[34], 17e-3))
        within_rel, within_floor, report = 0, 0, []
        gmax = max(np.abs(gc).max(), np.abs(ge[34]))
        for field, m, c, g, h in rows:
            f1, f2 = fd(field, m, c, h), fd(field, m, c, h / 2)
            floor = max(3.0 * abs(f1 - f2), 1e-5 * gmax)
            err = abs(g - f1)
            ok_rel = err <= 1e-3 * abs(g)
            ok_floor = err <= floor
            within_rel += ok_rel
            within_floor += (not ok_rel) and ok_floor
            report.append((field, m, c, g, f1, floor))
            assert ok_rel or ok_floor, (field, m, c, g, f1, floor)
        P.set_mats(sc["mats"])
        with capsys.disabled():
            print(f"\nFD on {len(rows)} parameters: {within_rel} within 1e-3 relative, "
                  f"{within_floor} within their FD noise floor; largest |gradient| {gmax:.3e}")
            for field, m, c, g, f1, floor in report:
                if abs(g - f1) > 1e-3 * abs(g):
                    print(f"  {field}[{m}, {c}]: adjoint {g:.6e}, FD {f1:.6e}, noise floor {floor:.2e}")
        assert within_rel >= 0.9 * len(rows)
    finally:
        P.close()


def test_matches_oracle_fp64_at_full_resolution(ctx, orc):
    """The FP64 oracle gradient at the inverse problem's 256 x 256 (2 spp)."""
    sc = _init_scene()
    P = Problem(ctx, sc, W=256, spp=2, rr=3)
    try:
        adj = np.random.default_rng(2).uniform(-1, 1, 256 * 256 * 3).astype(np.float32)
        gc, ge = P.backward(adj)
        oc, oe = orc.adjoint(sc, sc["camera"], P.bwd, adj)
        assert np.abs(oc).max() > 0
        assert np.allclose(gc, oc, rtol=1e-9, atol=1e-12 * np.abs(oc).max())
        assert np.allclose(ge, oe, rtol=1e-9, atol=1e-12 * np.abs(oe).max())
    finally:
        P.close()


def test_adam_recovers_parameters(ctx):
    true_sc = scenes.inverse_box()
    T = Problem(ctx, true_sc, spp=1024, seed_fwd=77)
    tgt = T.render(T.fwd, f64=True)
    T.fwd.spp, T.fwd.seed = 32, 5
    img = T.render(T.fwd)
    floor = float(np.mean((img - tgt) ** 2))  # 32-spp noise at the true parameters
    T.close()
    sc = _init_scene()
    P = Problem(ctx, sc, rr=3)
    theta = np.concatenate([np.full(34 * 3, 0.5), np.full(3, 10 / 17)])
    hi = np.concatenate([np.ones(102), np.full(3, 4.0)])
    m1, m2 = np.zeros_like(theta), np.zeros_like(theta)
    lr, b1, b2 = 0.02, 0.9, 0.999
    losses, seen = [], None
    try:
        for it in range(200):
            mats = scenes.inverse_box(albedo=theta[:102].reshape(34, 3), light_colour=theta[102:])["mats"]
            P.set_mats(mats)
            P.fwd.seed, P.bwd.seed = 1000 + 2 * it, 1001 + 2 * it
            img = P.render(P.fwd)
            diff = img - tgt
            losses.append(float(np.mean(diff * diff)))
            gc, _ = P.backward((2.0 * diff / img.size).astype(np.float32))
            g = np.concatenate([gc[:34].ravel(), gc[34]])
            if seen is None:
                seen = np.abs(g[:102]) > 1e-3 * np.abs(g[:102]).max()
            m1 = b1 * m1 + (1 - b1) * g
            m2 = b2 * m2 + (1 - b2) * g * g
            step = lr * (m1 / (1 - b1 ** (it + 1))) / (np.sqrt(m2 / (1 - b2 ** (it + 1))) + 1e-12)
            theta = np.clip(theta - step, 1e-3, hi)
        final = float(np.mean(losses[-10:]))
        assert final - floor < 0.1 * (losses[0] - floor), (losses[0], final, floor)
        truth = true_sc["true_albedo"].ravel()
        err0 = np.abs(0.5 - truth)[seen].mean()
        err1 = np.abs(theta[:102] - truth)[seen].mean()
        assert err1 < 0.5 * err0, (err0, err1)
        assert np.abs(theta[102:] - 1.0).max() < 0.5 * abs(10 / 17 - 1.0), theta[102:]
    finally:
        P.close()


def test_loss_l2_matches_numpy(ctx):
    sc = scenes.box_scene()
    P = Problem(ctx, dict(sc), W=64, spp=8)
    tb, ab, lb = api.DeviceBuffer(ctx, 64 * 64 * 12), api.DeviceBuffer(ctx, 64 * 64 * 12), api.DeviceBuffer(ctx, 8)
    try:
        P.film.reset()
        api.render(P.scene, sc["camera"], P.fwd, P.film)
        tgt = np.random.default_rng(4).uniform(0, 1, 64 * 64 * 3).astype(np.float32)
        tb.upload(tgt)
        api.loss_l2(P.film, tb, ab, lb)
        adj = ab.download(np.zeros(64 * 64 * 3, np.float32))
        loss = lb.download(np.zeros(1))[0]
        img = P.film.download()["sum"]
        d = img * (np.float32(1) / np.float32(8)) - tgt
        assert np.array_equal(adj, d * np.float32(2.0 / d.size))
        assert loss == pytest.approx(float(np.mean(d.astype(np.float64) ** 2)), rel=1e-12)
    finally:
        for b in (tb, ab, lb):
            b.free()
        P.close()
