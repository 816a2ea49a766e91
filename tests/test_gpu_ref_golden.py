"""The FP64 GPU path against golden vectors produced by the reference solver itself.

tests/golden/make_ref_golden.py ran the reference's own sources (built by oracle/Makefile.ref,
NONLINEARITY_ON) on seeded start fields and stored its outputs: calculate_NLstep at the first
step size, the on-axis carrier density, and several propagator() calls through its z-loop.
Here the product sets the grid up from the same config with its own C++ (gs_setup_from_config,
no oracle involved), takes the stored start field and runs the same calls through the C ABI.

Bar: 1e-10 relative L2 on the NL increment, the field and BIGBUFFER2 (the FP64 parity target);
identical controller decisions (STEP_N, the last ZSTEP to 1e-10).
"""
import os
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-10


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


def _config(text, medium):
    """Write the stored config and regenerate its RAW dispersion table."""
    d = tempfile.mkdtemp(prefix="gs_refgold_")
    p = os.path.join(d, "case.txt")
    with open(p, "w") as f:
        f.write(bytes(text).decode())
    if medium == "fused_silica":
        configs.tabulate_medium(os.path.join(d, "fused_silica.rawdisp"))
    else:
        configs.tabulate_medium(os.path.join(d, "argon.rawdisp"), medium="argon", lam_min_um=0.15, lam_max_um=20.0)
    return p


def _check_run(P, S, g, prefix, steps):
    P.set_field(g["field0"])
    cz, zstep, step_n, calls = P.run(S["znet"], float(g[prefix + "dz0"]), steps=steps)
    assert calls == steps
    assert step_n == int(g[prefix + "step_n"])
    assert abs(zstep / float(g[prefix + "zstep"]) - 1) < TOL
    f, s = P.get_field(want_spec=True)
    assert rel(f, g[prefix + "field"]) < TOL
    assert rel(s, g[prefix + "bb2"]) < TOL


def test_solid_matches_reference_golden():
    g = np.load(os.path.join(HERE, "golden", "ref_hot_solid.npz"))
    S = gs.Setup(_config(g["config"], "fused_silica")).as_dict()
    assert abs(S["rate_ln"][:8191] - g["rate_ln"][:8191]).max() < 1e-11 * abs(g["rate_ln"][:8191]).max()
    P = gs.Propagator(S, precision=gs.PREC_FP64)
    P.set_field(g["field0"])
    a2, n2 = P.nl_step(float(g["dz0"]))
    assert rel(P.get_nl(), g["bb1"]) < TOL
    assert abs(a2 / float(g["max_a2"]) - 1) < 1e-14
    assert abs(n2 / float(g["max_nl2"]) - 1) < TOL
    # the on-axis carrier density the reference computed for the start field (max over t)
    d = P.dumps(S["qdht_x"], S["r_max"])
    assert g["rho_axis"].max() > 1e26
    assert abs(d["pm"][0] / g["rho_axis"].max() - 1) < TOL
    _check_run(P, S, g, "", int(g["steps"]))
    P.close()


def test_gas_single_level_matches_reference_golden():
    g = np.load(os.path.join(HERE, "golden", "ref_argon_gas.npz"))
    S = gs.Setup(_config(g["l1_config"], "argon")).as_dict()
    assert S["gas"] == 1
    P = gs.Propagator(S, precision=gs.PREC_FP64)
    P.set_field(g["field0"])
    P.nl_step(float(g["l1_dz0"]))
    assert rel(P.get_nl(), g["l1_bb1"]) < TOL
    _check_run(P, S, g, "l1_", 3)
    P.close()


def test_gas_two_levels_matches_reference_golden():
    """IONIZATION_LEVEL_N 2 (MULTI_LEVEL_IONIZATION, ionization.cpp:45-84): the reference's own
    NL step and three propagator() calls, on the staged kernels' level-by-level recurrence."""
    g = np.load(os.path.join(HERE, "golden", "ref_argon_gas.npz"))
    S = gs.Setup(_config(g["l2_config"], "argon")).as_dict()
    assert S["gas"] == 1 and S["ion_levels"] == 2
    P = gs.Propagator(S, precision=gs.PREC_FP64)
    P.set_field(g["field0"])
    a2, n2 = P.nl_step(float(g["l2_dz0"]))
    assert rel(P.get_nl(), g["l2_bb1"]) < TOL
    assert abs(n2 / float(g["l2_max_nl2"]) - 1) < TOL
    _check_run(P, S, g, "l2_", 3)
    P.close()
