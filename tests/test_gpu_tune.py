"""gs_autotune: the chosen launch shape of the fused RK4-stage kernels is valid, leaves the
state untouched, and the z-step it runs still meets the parity bars (FP64 against the
oracle at 1e-10, the mixed path against the FP64 path)."""
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_autotuned_steps_keep_parity():
    d = tempfile.mkdtemp(prefix="gs_tune_")
    p = configs.hot_solid(d, n_r=128, n_t=2048, power_cr=20.0, tol=1e-2)
    T = tables.build(tables.Config.from_file(p), noise_seed=5, noise_sigma=1e-4)
    O = oracle.Oracle(T)
    dz = tables.init_zstep_kerr(T, T["field"])
    out, st = O.run(T["field"], dz, steps=3)
    P64 = gs.Propagator(T, precision=gs.PREC_FP64)
    P64.set_field(T["field"])
    before = P64.get_field(want_spec=True)
    t64, ms64 = P64.autotune()
    assert t64 >= 32 and t64 % 32 == 0 and 2048 % t64 == 0 and ms64 > 0
    after = P64.get_field(want_spec=True)
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    P64.run(T["znet"], dz, steps=3)
    assert rel(P64.get_field(want_spec=False), st["field"]) < 1e-10
    Pm = gs.Propagator(T, precision=gs.PREC_MIXED)
    Pm.set_field(T["field"])
    tm, msm = Pm.autotune()
    assert tm >= 32 and 2048 % tm == 0
    assert Pm.autotune() == (tm, msm)          # cached per grid
    Pm.run(T["znet"], dz, steps=3)
    assert rel(Pm.get_field(want_spec=False), st["field"]) < 2e-5
