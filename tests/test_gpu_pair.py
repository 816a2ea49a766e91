"""Rows too long for one CTA's shared memory run each RK4 stage over a pair of CTAs (two
kernels per stage; the inverse transform's radix-2 step and the density / Raman recurrences
cross the pair through distributed shared memory): FP32 rows of N_T = 32768 on the mixed path
and FP64 rows of N_T = 16384, against the oracle.

Tolerances as elsewhere: FP64 1e-10 relative L2; one mixed NL increment 1e-5 (solid) and
2e-5 (gas build).
"""
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


def _solid(n_r, n_t, window, power_cr=20.0, seed=11, **over):
    d = tempfile.mkdtemp(prefix="gs_pair_")
    p = configs.hot_solid(d, n_r=n_r, n_t=n_t, power_cr=power_cr, tol=1e-2, window=window)
    T = tables.build(tables.Config.from_file(p), noise_seed=seed, noise_sigma=1e-4)
    T.update(over)
    return T


def _nl_step_checked(T, precision, tol):
    O = oracle.Oracle(T)
    dz = tables.init_zstep_kerr(T, T["field"]) if T["n2"] else 2e-7
    bb1, a2, n2 = O.nl_step(T["field"], dz)
    P = gs.Propagator(T, precision=precision)
    P.set_field(T["field"])
    n0 = P.launch_count()
    ga2, gn2 = P.nl_step(dz)
    assert P.launch_count() - n0 == 8   # two kernels per RK4 stage
    assert rel(P.get_nl(), bb1) < tol
    assert abs(ga2 - a2) / a2 < 1e-6
    assert abs(gn2 - n2) / n2 < tol
    return O


@pytest.mark.parametrize("over", [{}, {"n2": 0.0}])
def test_pair_mixed_32768_solid(over):
    T = _solid(128, 32768, 3.2e-12, **over)
    e = np.fft.ifft(T["field"][0])
    O = _nl_step_checked(T, gs.PREC_MIXED, 1e-5)
    pro, _ = O.plasma(e)
    assert pro.max() > 0   # the density recurrence is exercised on axis


def test_pair_fp64_16384_solid():
    T = _solid(8, 16384, 1.6e-12)
    _nl_step_checked(T, gs.PREC_FP64, 1e-10)


def test_pair_mixed_32768_gas_third_harmonic():
    d = tempfile.mkdtemp(prefix="gs_pair_gas_")
    p = configs.argon_c5(d, n_r=128, n_t=32768, build="gas_qdht", power_cr=6.0, w0=9e-4, r_max=3.6e-3)
    T = tables.build(tables.Config.from_file(p), noise_seed=2, noise_sigma=1e-4)
    assert T["th_coeff"] != 0
    _nl_step_checked(T, gs.PREC_MIXED, 2e-5)


def test_pair_mixed_32768_controller_vs_fp64():
    """propagator() steps on the pair path: the FP64 path (staged at this length) agrees."""
    T = _solid(128, 32768, 3.2e-12, power_cr=30.0)
    dz0 = tables.init_zstep_kerr(T, T["field"])
    res = {}
    for prec in (gs.PREC_FP64, gs.PREC_MIXED):
        P = gs.Propagator(T, precision=prec)
        P.set_field(T["field"])
        cz, zstep, step_n, calls = P.run(T["znet"], dz0, steps=3)
        res[prec] = (zstep, step_n, P.get_field(want_spec=False))
    assert res[gs.PREC_MIXED][1] == res[gs.PREC_FP64][1]
    assert abs(res[gs.PREC_MIXED][0] / res[gs.PREC_FP64][0] - 1) < 1e-4
    assert rel(res[gs.PREC_MIXED][2], res[gs.PREC_FP64][2]) < 5e-5
