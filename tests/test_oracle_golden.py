"""Pin the CPU oracle against the reference's own committed outputs.

bin/fil_SiO2_1d.txt -> bin/fil_SiO2__{f,fa,mI,pm,s}.udf (N_R=512, N_T=512, 127 z-steps)
and bin/omega.bin / bin/wavenum.bin, extracted into tests/golden/ by make_golden.py.
The golden run is linear (E = 1 fJ), so it pins the QDHT, the linear propagator, the
step controller, the Gaussian start field, the dispersion tables and the dumps.
"""
import os

import numpy as np
import pytest

from oracle import oracle, tables
from tests.golden_cfg import golden_config_dir, load_golden


@pytest.fixture(scope="module")
def golden_run():
    g = load_golden()
    d = golden_config_dir()
    cfg = tables.Config.from_file(os.path.join(d, "fil_SiO2_1d.txt"))
    T = tables.build(cfg)
    dz0 = tables.init_zstep_kerr(T, T["field"])
    O = oracle.Oracle(T, nonlinear=False)
    out, st = O.run(T["field"], dz0)
    return g, T, out, st


def test_omega_and_wavenumber_tables_match_reference_bins():
    g = load_golden()
    d = golden_config_dir()
    T = tables.build(tables.Config.from_file(os.path.join(d, "fil_SiO2_1d.txt")))
    assert np.array_equal(T["omega"], g["omega_bin"])
    k = g["wavenum_bin"]
    assert np.max(np.abs(T["wavenum"] - k)) / np.max(np.abs(k)) < 1e-15


def test_golden_run_step_count(golden_run):
    g, T, out, st = golden_run
    assert st["n_z"] == 127 and len(out["z"]) == 128
    assert st["step_n"] == 127          # one accepted step per ZNET interval


@pytest.mark.parametrize("key,tol", [("mI", 5e-8), ("f", 5e-8), ("s", 1e-8), ("fa", 1e-7)])
def test_golden_dumps(golden_run, key, tol):
    g, T, out, st = golden_run
    sl = g["slabs"]
    mine = np.array(out[key])[sl]
    ref = g["udf_" + key]
    # z = Z_MIN slab: only the start field and the dump arithmetic are involved
    assert np.linalg.norm(mine[0] - ref[0]) / np.linalg.norm(ref[0]) < (1e-10 if key == "s" else 1e-14)
    err = np.linalg.norm(mine - ref) / np.linalg.norm(ref)
    assert err < tol, (key, err)


def test_golden_plasma_max_is_zero(golden_run):
    g, T, out, st = golden_run
    assert np.all(g["udf_pm"] == 0)
    assert np.all(np.array(out["pm"]) == 0)
