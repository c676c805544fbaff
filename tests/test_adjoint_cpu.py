"""The oracle's FP64 path-replay gradient against central finite differences
with common random numbers (CPU).  With Russian roulette off and fixed random
numbers the estimator is a polynomial in the material colours and emissions,
so the derivative must match FD to 1e-3 relative."""
import numpy as np
import pytest

from crender_gb300 import api, scenes


def _phi(orc, sc, st, adj):
    f = orc.render(sc, sc["camera"], st)
    return float(np.dot(adj.astype(np.float64), f["sum64"] / st.spp))


@pytest.mark.parametrize("param", [("col", 0, 0), ("col", 7, 1), ("col", 12, 2), ("col", 34, 1), ("em", 34, 0)])
def test_oracle_gradient_matches_fd(orc, param):
    sc = scenes.inverse_box(albedo=np.full((34, 3), 0.5), light_colour=np.full(3, 10 / 17))
    st = api.make_settings(8, 8, 64, 8, 0, 1, 5)
    adj = np.random.default_rng(3).uniform(-1, 1, 8 * 8 * 3).astype(np.float32)
    gc, ge = orc.adjoint(sc, sc["camera"], st, adj)
    kind, m, c = param
    h = 1e-3
    mats_p, mats_m = sc["mats"].copy(), sc["mats"].copy()
    if kind == "col":
        mats_p[m]["colour"][c] += h
        mats_m[m]["colour"][c] -= h
        g = gc[m, c]
    else:
        mats_p[m]["emission"] += h
        mats_m[m]["emission"] -= h
        g = ge[m]
    fd = (_phi(orc, dict(sc, mats=mats_p), st, adj) - _phi(orc, dict(sc, mats=mats_m), st, adj)) / (2 * h)
    assert abs(g) > 1e-6
    assert abs(g - fd) <= 1e-3 * abs(g) + 1e-7, (g, fd)
