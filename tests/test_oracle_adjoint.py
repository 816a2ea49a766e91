"""The oracle's FP64 adjoint of the z-step against central finite differences of the
oracle's own forward (CPU).  Directional derivatives <g, v> = sum Re(conj(g) v) along
seeded random complex directions; the objective is a seeded positive weighting of
|FIELD|^2 after three propagator() calls with fixed, unequal step sizes (RK4 stages and
linear step use different dz, as propagator() does after the controller)."""
import tempfile

import numpy as np
import pytest

from gsolver_gb300 import configs
from oracle import oracle, tables


def _setup(power_cr, seed=7, **kw):
    d = tempfile.mkdtemp(prefix="gs_adj_")
    p = configs.hot_solid(d, n_r=8, n_t=512, power_cr=power_cr, tol=1e-2)
    T = tables.build(tables.Config.from_file(p), noise_seed=seed, noise_sigma=1e-4)
    T.update(kw)
    return T


@pytest.mark.parametrize("power_cr,over", [
    (20.0, {}),                       # Kerr + Raman + plasma density (below the loss threshold)
    (45.0, {}),                       # multiphoton loss active, density near rho_n
    (30.0, {"raman_fraction": 0.0}),  # instantaneous Kerr only
    (30.0, {"n2": 0.0}),              # plasma only
])
def test_adjoint_matches_central_differences(power_cr, over):
    T = _setup(power_cr, **over)
    O = oracle.Oracle(T)
    dz0 = tables.init_zstep_kerr(T, T["field"]) if T["n2"] else 2e-7
    dz_rk = [dz0, 0.9 * dz0, 1.1 * dz0]
    dz_lin = [0.9 * dz0, 1.1 * dz0, dz0]
    rng = np.random.default_rng(11)
    w = rng.random((T["n_r"], T["n_t"]))
    A0 = T["field"]
    J, g = O.gradient(A0, dz_rk, dz_lin, w)
    assert J > 0 and np.all(np.isfinite(g))

    def Jf(A):
        f, _ = O.forward_fixed(A, dz_rk, dz_lin)
        return float(np.sum(w * (f.real ** 2 + f.imag ** 2)))

    # small h: the rate table is piecewise log-linear in I, and larger steps straddle its
    # nodes, where the derivative jumps (a ~1e-6 bias at h = 1e-5)
    scale = np.linalg.norm(A0)
    h = 1e-6
    for _ in range(3):
        v = rng.standard_normal(A0.shape) + 1j * rng.standard_normal(A0.shape)
        v *= scale / np.linalg.norm(v)
        fd = (Jf(A0 + h * v) - Jf(A0 - h * v)) / (2 * h)
        ad = float(np.sum((np.conj(g) * v).real))
        assert abs(fd - ad) <= 2e-6 * abs(ad), (fd, ad)


def test_transposed_qdht_is_the_adjoint():
    T = _setup(20.0)
    O = oracle.Oracle(T)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((8, 512)) + 1j * rng.standard_normal((8, 512))
    y = rng.standard_normal((8, 512)) + 1j * rng.standard_normal((8, 512))
    lhs = np.vdot(y, O.qdht(x))
    rhs = np.vdot(O.qdht_t(y), x)
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs)
