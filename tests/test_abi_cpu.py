"""CPU-side checks: the C-ABI library loads and exports every declared entry point, and the
product's own C++ set-up matches the oracle's numpy restatement of the reference start-up."""
import glob
import os
import re
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import tables
from tests.golden_cfg import golden_config_dir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(gs_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    L = gs.load_library()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(gs.ABI_FUNCTIONS) == names


def test_the_default_build_is_not_the_checked_one():
    # GS_CHECK index tests live in their own library (_build_check/), loaded only under GS_CHECK=1
    assert gs.load_library().gs_check_build() == 0
    assert gs.LIB_PATH.endswith(os.path.join("_build", "libgsolver_gb300.so"))


def test_status_strings_are_the_reference_messages():
    L = gs.load_library()
    assert L.gs_status_string(gs.GS_ERR_BLAST).decode() == \
        "Attention!!!! Intensity is too big! Keep away, blast is possible."
    assert L.gs_status_string(gs.GS_ERR_COLLAPSE).decode() == "Minimum Z step size reached, collapse is possible!"


def _compare(S, T, tol_rate=1e-11):
    for k in ("plasma_func", "raman_func", "kerr", "omega", "wavenum", "ho_disp", "kt2", "qdht_c", "qdht_m1", "field"):
        a, b = np.asarray(S[k]), np.asarray(T[k])
        assert np.linalg.norm(a - b) <= 1e-13 * np.linalg.norm(b), k
    assert np.linalg.norm(S["rate_ln"] - T["rate_ln"]) <= tol_rate * np.linalg.norm(T["rate_ln"])
    for k in gs.PARAM_KEYS:
        assert abs(S[k] - T[k]) <= 1e-13 * abs(T[k]), k
    dz = tables.init_zstep_kerr(T, T["field"])
    assert abs(S["init_zstep"] - dz) <= 1e-13 * dz


def test_setup_matches_oracle_on_golden_config():
    p = os.path.join(golden_config_dir(), "fil_SiO2_1d.txt")
    _compare(gs.Setup(p).as_dict(), tables.build(tables.Config.from_file(p)))


def test_setup_matches_oracle_with_seeded_noise():
    d = tempfile.mkdtemp()
    p = configs.hot_solid(d, n_r=16, n_t=512, power_cr=20.0)
    S = gs.Setup(p, noise_seed=5, noise_sigma=1e-4).as_dict()
    T = tables.build(tables.Config.from_file(p), noise_seed=5, noise_sigma=1e-4)
    _compare(S, T)


def test_setup_overrides_take_precedence():
    d = tempfile.mkdtemp()
    p = configs.hot_solid(d, n_r=16, n_t=512)
    S = gs.Setup(p, overrides={"N_T": 256, "NONLIN_REFRINDEX": "5e-20"}).as_dict()
    T = tables.build(tables.Config.from_file(p, overrides={"N_T": 256, "NONLIN_REFRINDEX": "5e-20"}))
    assert S["n_t"] == 256
    _compare(S, T)


def test_setup_errors():
    with pytest.raises(gs.GsError):
        gs.Setup("/nonexistent/config.txt")
    d = tempfile.mkdtemp()
    p = configs.hot_solid(d, n_r=16, n_t=512)
    with pytest.raises(gs.GsError) as ei:
        gs.Setup(p, overrides={"N_T": 500})
    assert "power of two" in str(ei.value)
