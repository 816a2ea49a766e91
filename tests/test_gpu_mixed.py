"""Mixed-precision path (FP32 elementwise/FFT + tcgen05 QDHT with split operands) vs the FP64
oracle.

Tolerances are stated per quantity: the QDHT's split operands (FP16 pairs with power-of-two
row / column scales where 2 n_t is a multiple of 256, 3xTF32 otherwise) carry ~2^-21 relative
error per product, the FP32 FFTs ~1e-7 per pass, so one transform / step is expected near 1e-6.
"""
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables

pytestmark = pytest.mark.gpu

QDHT_TOL = 1e-5     # one transform, relative L2
STEP_TOL = 1e-5     # one NL increment / one full step, relative L2


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


def hot_setup(n_r=128, n_t=1024, power_cr=20.0, tol=1e-2, seed=11, **kw):
    d = tempfile.mkdtemp(prefix="gs_mixed_")
    p = configs.hot_solid(d, n_r=n_r, n_t=n_t, power_cr=power_cr, tol=tol, **kw)
    return tables.build(tables.Config.from_file(p), noise_seed=seed, noise_sigma=1e-4)


# (512, 4096) and (1024, 2048): 256 output tiles of 128 x 128, more than the persistent grid
# (one CTA per SM), so CTAs run several tiles through both accumulator buffers
@pytest.mark.parametrize("n_r,n_t", [(128, 64), (256, 512), (512, 256), (512, 4096), (1024, 2048)])
def test_qdht_tensor_cores(n_r, n_t):
    T = hot_setup(n_r=n_r, n_t=n_t)
    rng = np.random.default_rng(n_r + n_t)
    x = rng.standard_normal((n_r, n_t)) + 1j * rng.standard_normal((n_r, n_t))
    ref = oracle.Oracle(T).qdht(x)
    P = gs.Propagator(T, precision=gs.PREC_MIXED)
    y = P.qdht(x)
    assert rel(y, ref) < QDHT_TOL
    # every output tile is exercised: per-row errors stay small too
    assert max(rel(y[i], ref[i]) for i in range(0, n_r, max(1, n_r // 16))) < 10 * QDHT_TOL
    assert np.array_equal(P.qdht(x), y)   # the transform is deterministic


@pytest.mark.parametrize("n_r,n_t", [(256, 512), (1024, 256)])
def test_qdht_fp16_scales(n_r, n_t):
    """The FP16 operands with their scales: columns spread over 60 decades, a zero column, a
    column with one tiny entry, and a beam-like radial profile (large at small r, where the
    rows of H are small): each nonzero column within the transform tolerance of the FP64
    oracle, the zero column exactly zero."""
    T = hot_setup(n_r=n_r, n_t=n_t)
    rng = np.random.default_rng(5)
    r = np.arange(n_r)[:, None] / n_r
    x = (rng.standard_normal((n_r, n_t)) + 1j * rng.standard_normal((n_r, n_t))) * np.exp(-(r / 0.05) ** 2)
    x += 1e-6 * (rng.standard_normal((n_r, n_t)) + 1j * rng.standard_normal((n_r, n_t)))
    x *= 10.0 ** rng.uniform(-30, 30, n_t)[None, :]
    x[:, 3] = 0
    x[:, 5] = 0
    x[n_r // 2, 5] = 1e-35
    ref = oracle.Oracle(T).qdht(x)
    P = gs.Propagator(T, precision=gs.PREC_MIXED)
    y = P.qdht(x)
    assert np.all(y[:, 3] == 0)
    for c in range(n_t):
        if c != 3:
            assert rel(y[:, c], ref[:, c]) < QDHT_TOL, c


def test_nl_step_mixed():
    T = hot_setup()
    O = oracle.Oracle(T)
    dz = tables.init_zstep_kerr(T, T["field"])
    bb1, a2, n2 = O.nl_step(T["field"], dz)
    P = gs.Propagator(T, precision=gs.PREC_MIXED)
    P.set_field(T["field"])
    ga2, gn2 = P.nl_step(dz)
    assert rel(P.get_nl(), bb1) < STEP_TOL
    assert abs(ga2 - a2) / a2 < 1e-6
    assert abs(gn2 - n2) / n2 < STEP_TOL


def test_full_step_mixed_vs_fp64_gpu():
    T = hot_setup()
    dz = tables.init_zstep_kerr(T, T["field"])
    out = {}
    for prec in (gs.PREC_FP64, gs.PREC_MIXED):
        P = gs.Propagator(T, precision=prec)
        P.set_field(T["field"])
        for _ in range(3):
            P.nl_step(dz)
            P.lstep(dz)
        out[prec] = P.get_field()
    f64, s64 = out[gs.PREC_FP64]
    fm, sm = out[gs.PREC_MIXED]
    assert rel(fm, f64) < STEP_TOL
    assert rel(sm, s64) < STEP_TOL


def test_propagator_mixed_controller():
    """propagator() on the mixed path: same accepted-step count and dz as FP64."""
    T = hot_setup()
    dz0 = tables.init_zstep_kerr(T, T["field"])
    res = {}
    for prec in (gs.PREC_FP64, gs.PREC_MIXED):
        P = gs.Propagator(T, precision=prec)
        P.set_field(T["field"])
        cz, zstep, step_n, calls = P.run(T["znet"], dz0, steps=5)
        res[prec] = (zstep, step_n, P.get_field(want_spec=False))
    assert res[gs.PREC_MIXED][1] == res[gs.PREC_FP64][1]
    assert abs(res[gs.PREC_MIXED][0] / res[gs.PREC_FP64][0] - 1) < 1e-4
    assert rel(res[gs.PREC_MIXED][2], res[gs.PREC_FP64][2]) < STEP_TOL


def test_mixed_requires_multiple_of_128():
    T = hot_setup(n_r=96, n_t=64)
    with pytest.raises(gs.GsError) as ei:
        gs.Propagator(T, precision=gs.PREC_MIXED)
    assert ei.value.code == gs.GS_ERR_UNSUPPORTED
