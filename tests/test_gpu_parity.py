"""FP64 GPU path vs the CPU oracle on identical seeded inputs (bar: 1e-10 relative L2).

Every call goes through the C ABI (gsolver_gb300.Propagator -> libgsolver_gb300.so).
Inputs: the oracle's own set-up of small fused-silica grids; the "hot" grids reach
~3.4e13 W/cm^2 so that Keldysh ionization, avalanche, the loss term and plasma
defocusing are all active.
"""
import os
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables
from tests.golden_cfg import golden_config_dir, load_golden

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


def hot_setup(n_r=32, n_t=2048, power_cr=20.0, tol=1e-2, seed=7, **kw):
    d = tempfile.mkdtemp(prefix="gs_hot_")
    p = configs.hot_solid(d, n_r=n_r, n_t=n_t, power_cr=power_cr, tol=tol, **kw)
    return tables.build(tables.Config.from_file(p), noise_seed=seed, noise_sigma=1e-4)


@pytest.fixture(scope="module")
def hot():
    T = hot_setup()
    return T, oracle.Oracle(T)


def test_qdht_matches_run_many():
    T = hot_setup(n_r=96, n_t=256)
    O = oracle.Oracle(T)
    rng = np.random.default_rng(3)
    x = rng.standard_normal((96, 256)) + 1j * rng.standard_normal((96, 256))
    P = gs.Propagator(T)
    y = P.qdht(x)
    assert rel(y, O.qdht(x)) < 1e-13
    # C is (up to rounding) an involution: ht_run twice returns the input
    assert rel(P.qdht(y), x) < 1e-6


def test_set_get_field_roundtrip(hot):
    T, O = hot
    P = gs.Propagator(T)
    P.set_field(T["field"])
    f, s = P.get_field()
    assert np.array_equal(f, T["field"])
    assert rel(s, O.qdht(T["field"])) < 1e-13


def test_nl_step_hot(hot):
    T, O = hot
    dz = tables.init_zstep_kerr(T, T["field"])
    bb1, a2, n2 = O.nl_step(T["field"], dz)
    P = gs.Propagator(T)
    P.set_field(T["field"])
    ga2, gn2 = P.nl_step(dz)
    g = P.get_nl()
    assert rel(g, bb1) < TOL
    assert abs(ga2 - a2) / a2 < 1e-14
    assert abs(gn2 - n2) / n2 < TOL
    # the plasma terms are active on this grid
    e = np.fft.ifft(T["field"][0])
    pro, loss = O.plasma(e)
    assert pro.max() > 1e26 and np.abs(loss).max() > 0


def test_nl_step_no_raman_no_kerr():
    T = hot_setup(n_r=8, n_t=1024)
    for fr, n2 in ((0.0, None), (0.18, 0.0)):
        T2 = dict(T)
        T2["raman_fraction"] = fr
        if n2 is not None:
            T2["n2"] = n2
        O = oracle.Oracle(T2)
        bb1, a2, nl2 = O.nl_step(T2["field"], 1e-7)
        P = gs.Propagator(T2)
        P.set_field(T2["field"])
        P.nl_step(1e-7)
        assert rel(P.get_nl(), bb1) < TOL


def test_nl_step_two_level_fft():
    """N_T = 16384 exceeds one CTA's FP64 shared-memory row: each RK4 stage over two CTAs per row."""
    T = hot_setup(n_r=4, n_t=16384, window=1.6e-12)
    O = oracle.Oracle(T)
    dz = tables.init_zstep_kerr(T, T["field"])
    bb1, a2, n2 = O.nl_step(T["field"], dz)
    P = gs.Propagator(T)
    P.set_field(T["field"])
    P.nl_step(dz)
    assert rel(P.get_nl(), bb1) < TOL


def test_lstep_hot(hot):
    T, O = hot
    dz = tables.init_zstep_kerr(T, T["field"])
    bb1, _, _ = O.nl_step(T["field"], dz)
    bb2 = O.qdht(T["field"])
    fk, bb2n = O.lstep(O.qdht(bb1), bb2, dz)
    ref_field = O.qdht(fk)
    P = gs.Propagator(T)
    P.set_field(T["field"])
    P.nl_step(dz)
    P.lstep(dz)
    f, s = P.get_field()
    assert rel(f, ref_field) < TOL
    assert rel(s, bb2n) < TOL


def test_propagator_steps_hot(hot):
    """Ten propagator() calls: final field, fluence and on-axis plasma density."""
    T, O = hot
    dz0 = tables.init_zstep_kerr(T, T["field"])
    znet = T["znet"]
    out, st = O.run(T["field"], dz0, steps=10)
    P = gs.Propagator(T)
    P.set_field(T["field"])
    cz, zstep, step_n, calls = P.run(znet, dz0, steps=10)
    assert calls == 10
    assert step_n == st["step_n"]
    assert abs(zstep - st["zstep"]) <= 1e-10 * st["zstep"]
    f, s = P.get_field()
    assert rel(f, st["field"]) < TOL
    assert rel(s, st["bb2"]) < TOL
    dg, dr = O.dumps(f), O.dumps(st["field"])
    assert rel(dg["f"], dr["f"]) < TOL           # fluence
    assert dr["pm"][0] > 0
    e_g = np.fft.ifft(f[0]); e_r = np.fft.ifft(st["field"][0])
    assert rel(O.plasma(e_g)[0], O.plasma(e_r)[0]) < TOL   # on-axis plasma density


def test_golden_run_on_gpu():
    """The reference's golden linear run, stepped on the GPU, dumped by the oracle."""
    g = load_golden()
    d = golden_config_dir()
    T = tables.build(tables.Config.from_file(os.path.join(d, "fil_SiO2_1d.txt")))
    O = oracle.Oracle(T, nonlinear=False)
    dz0 = tables.init_zstep_kerr(T, T["field"])
    P = gs.Propagator(T, nonlinear=False)
    P.set_field(T["field"])
    dumps = {}

    def on_dump(n_z, prop):
        if n_z in set(g["slabs"].tolist()):
            dumps[n_z] = O.dumps(prop.get_field(want_spec=False))

    P.run(T["znet"], dz0, on_dump=on_dump)
    for key, tol in (("mI", 5e-8), ("f", 5e-8), ("s", 1e-8), ("fa", 1e-7)):
        mine = np.array([dumps[z][key] for z in g["slabs"]])
        assert rel(mine, g["udf_" + key]) < tol, key


def test_blast_error():
    T = hot_setup(n_r=4, n_t=512)
    P = gs.Propagator(T)
    P.set_field(T["field"] * 1e6)
    with pytest.raises(gs.GsError) as ei:
        P.nl_step(1e-9)
    assert ei.value.code == gs.GS_ERR_BLAST
    assert "blast is possible" in str(ei.value)


def test_nan_error():
    T = hot_setup(n_r=4, n_t=512)
    P = gs.Propagator(T)
    f = T["field"].copy()
    f[1, 3] = np.nan
    P.set_field(f)
    with pytest.raises(gs.GsError) as ei:
        P.nl_step(1e-9)
    assert ei.value.code == gs.GS_ERR_NAN


def test_collapse_error():
    T = hot_setup(n_r=4, n_t=512, tol=1e-16)
    P = gs.Propagator(T)
    P.set_field(T["field"])
    with pytest.raises(gs.GsError) as ei:
        P.step(0.0, T["znet"][1], T["znet"][0], 1e-9)
    assert ei.value.code == gs.GS_ERR_COLLAPSE
    assert "collapse" in str(ei.value)


def test_argon_parity_no_raman():
    """3.9 um argon (Raman off, Ip 15.76 eV, ~6e13 W/cm^2): NL step and three propagator() calls."""
    d = tempfile.mkdtemp(prefix="gs_ar_")
    p = configs.argon_c5(d, n_r=64, n_t=4096)
    T = tables.build(tables.Config.from_file(p), noise_seed=3, noise_sigma=1e-4)
    O = oracle.Oracle(T)
    dz0 = tables.init_zstep_kerr(T, T["field"])
    bb1, a2, n2 = O.nl_step(T["field"], dz0)
    P = gs.Propagator(T)
    P.set_field(T["field"])
    P.nl_step(dz0)
    assert rel(P.get_nl(), bb1) < TOL
    out, st = O.run(T["field"], dz0, steps=3)
    P.set_field(T["field"])
    cz, zstep, step_n, calls = P.run(T["znet"], dz0, steps=3)
    assert rel(P.get_field(want_spec=False), st["field"]) < TOL


def test_fused_silica_256x2048_steps():
    """The CPU-runnable fused-silica workload (256 x 2048) at full size, five propagator() calls,
    set up by the product's own C++ and by the oracle (they agree to 1e-12)."""
    d = tempfile.mkdtemp(prefix="gs_c1_")
    p = configs.fused_silica_c1(d)
    S = gs.Setup(p, noise_seed=1234, noise_sigma=1e-4).as_dict()
    T = tables.build(tables.Config.from_file(p), noise_seed=1234, noise_sigma=1e-4)
    O = oracle.Oracle(T)
    out, st = O.run(T["field"], S["init_zstep"], steps=5)
    P = gs.Propagator(S)
    P.set_field(S["field"])
    P.run(S["znet"], S["init_zstep"], steps=5)
    f = P.get_field(want_spec=False)
    assert rel(f, st["field"]) < TOL
    dg, dr = O.dumps(f), O.dumps(st["field"])
    assert rel(dg["f"], dr["f"]) < TOL
    assert rel(dg["mI"], dr["mI"]) < TOL
