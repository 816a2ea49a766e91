"""The gas build on the GPU against the oracle: single-level PPT ionization with neutral
depletion and the third harmonic (FP64 1e-10; mixed 2e-5), on the fused path (rows in one
CTA) and the pair path (FP64 N_T = 16384: each row over two CTAs, 8192 points each); several
ionization levels (MULTI_LEVEL_IONIZATION, ionization.cpp:45-84) on the staged kernels."""
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


POTENTIALS_EV = (15.76, 27.63, 40.74)   # argon's first three ionization potentials


def _argon(n_r=16, n_t=4096, power_cr=6.0, w0=9e-4, seed=2, levels=1):
    d = tempfile.mkdtemp(prefix="gs_ggas_")
    p = configs.argon_c5(d, n_r=n_r, n_t=n_t, build="gas_qdht", power_cr=power_cr, w0=w0, r_max=4 * w0)
    if levels > 1:
        with open(p, "a") as fh:
            fh.write(f"IONIZATION_LEVEL_N {levels}\n")
            for n in range(levels):
                fh.write(f"IONIZATION_POTENTIAL{n + 1} {POTENTIALS_EV[n]}\n")
    return tables.build(tables.Config.from_file(p), noise_seed=seed, noise_sigma=1e-4)


@pytest.mark.parametrize("n_t", [4096, 16384])
def test_gas_nl_step_fp64(n_t):
    T = _argon(n_t=n_t, n_r=8 if n_t > 8192 else 16)
    O = oracle.Oracle(T)
    dz = tables.init_zstep_kerr(T, T["field"])
    bb1, a2, n2 = O.nl_step(T["field"], dz)
    e = np.fft.ifft(T["field"][0])
    pro, loss = O.plasma(e)
    assert pro.max() > 1e-4 * T["neutral_density"] and np.abs(loss).max() > 0   # ionization is on
    P = gs.Propagator(T, precision=gs.PREC_FP64)
    P.set_field(T["field"])
    ga2, gn2 = P.nl_step(dz)
    assert rel(P.get_nl(), bb1) < 1e-10
    assert abs(gn2 - n2) <= 1e-10 * n2


def test_gas_propagator_steps_fp64_and_mixed():
    T = _argon(n_r=128, n_t=4096)
    O = oracle.Oracle(T)
    dz0 = tables.init_zstep_kerr(T, T["field"])
    out, st = O.run(T["field"], dz0, steps=3)
    P = gs.Propagator(T, precision=gs.PREC_FP64)
    P.set_field(T["field"])
    cz, zstep, step_n, calls = P.run(T["znet"], dz0, steps=3)
    assert step_n == st["step_n"] and abs(zstep - st["zstep"]) <= 1e-10 * st["zstep"]
    f = P.get_field(want_spec=False)
    assert rel(f, st["field"]) < 1e-10
    d_g, d_r = O.dumps(f), O.dumps(st["field"])
    assert rel(d_g["pm"], d_r["pm"]) < 1e-10          # plasma_max through the gas recurrence
    g = P.dumps(T["qdht_x"], T["r_max"])
    assert rel(g["pm"], d_r["pm"]) < 1e-10            # the device reduction
    Pm = gs.Propagator(T, precision=gs.PREC_MIXED)
    Pm.set_field(T["field"])
    Pm.run(T["znet"], dz0, steps=3)
    assert rel(Pm.get_field(want_spec=False), st["field"]) < 2e-5


@pytest.mark.parametrize("levels", [2, 3])
def test_gas_levels_nl_step_and_steps(levels):
    """Several ionization levels, solved level by level (each a scalar multiple shooting).
    FP64: the NL step at the Kerr estimate of the first step, three propagator() calls and the
    plasma dump's density (the levels' sum), each at 1e-10.  Mixed: the NL step at the size the
    controller settles on, 1e-5 (the Kerr estimate is ~10^3 times larger on this strongly
    ionizing pulse: RK4's stage inputs then carry the plasma term's huge low-frequency
    increments and FP32 rounding grows to ~1e-3 on any path, single level included), and the
    field after three calls within 1e-5 of the FP64 path's."""
    T = _argon(n_r=128, n_t=4096, power_cr=8.0, levels=levels)   # the tensor-core QDHT: n_r % 128 == 0
    O = oracle.Oracle(T)
    dz = tables.init_zstep_kerr(T, T["field"])
    bb1, a2, n2 = O.nl_step(T["field"], dz)
    e = np.fft.ifft(T["field"][0])
    pro, loss = O.plasma(e)
    assert pro.max() > 1e-4 * T["neutral_density"] and np.abs(loss).max() > 0
    P = gs.Propagator(T, precision=gs.PREC_FP64)
    P.set_field(T["field"])
    ga2, gn2 = P.nl_step(dz)
    assert rel(P.get_nl(), bb1) < 1e-10
    assert abs(gn2 - n2) <= 1e-10 * n2
    out, st = O.run(T["field"], dz, steps=3)
    P.set_field(T["field"])
    cz, zstep, step_n, calls = P.run(T["znet"], dz, steps=3)
    assert step_n == st["step_n"] and abs(zstep / st["zstep"] - 1) < 1e-10
    f64 = P.get_field(want_spec=False)
    assert rel(f64, st["field"]) < 1e-10
    dg, dr = P.dumps(T["qdht_x"], T["r_max"]), O.dumps(f64)
    assert rel(dg["pm"], dr["pm"]) < 1e-10
    P.close()
    dzc = st["zstep"]   # the controller's proposal
    bbc, _, nc = O.nl_step(T["field"], dzc)
    M = gs.Propagator(T, precision=gs.PREC_MIXED)
    M.set_field(T["field"])
    _, mn2 = M.nl_step(dzc)
    assert rel(M.get_nl(), bbc) < 1e-5
    assert abs(mn2 - nc) <= 1e-5 * nc
    M.set_field(T["field"])
    M.run(T["znet"], dz, steps=3)
    assert rel(M.get_field(want_spec=False), f64) < 1e-5
    M.close()
