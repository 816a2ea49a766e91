"""Accuracy at the end of a whole run and at full size, not only after a few steps.

* The CPU-runnable fused-silica workload (256 x 2048, 1 mm in 500 propagator() calls) run to
  its last ZNET point on the FP64 GPU path and by the oracle (propagator.cu:125-266 restated
  in FP64): final field, fluence and on-axis plasma density within 1e-10 relative L2, the same
  controller decisions; the mixed path's final field within 1e-5 of the FP64 path's.
* One propagator() call of the 1024 x 16384 workload on the FP64 GPU path against the oracle
  within 1e-10 (the full-size grid: window-compacted FP64 transforms, the FP64 row kernels of
  16384 points over two CTAs).
* The mixed path's error against the FP64 path on the 1024 x 16384 workload does not grow with
  the number of steps (200 fixed steps): the QDHT's chunked accumulation, the double-float
  propagator factors and BIGBUFFER2's double-float window columns leave no error that builds up.
"""
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-5


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


def on_axis_plasma(O, field):
    """Carrier density of the on-axis row over time (calculate_plasmadensity_losses_small of
    E = BW-FFT(FIELD[0]) / N_T)."""
    return O.plasma(np.fft.ifft(field[0]))[0]


def test_fused_silica_256x2048_whole_run():
    d = tempfile.mkdtemp(prefix="gs_c1_run_")
    p = configs.fused_silica_c1(d)
    T = tables.build(tables.Config.from_file(p), noise_seed=1234, noise_sigma=1e-4)
    O = oracle.Oracle(T)
    dz0 = tables.init_zstep_kerr(T, T["field"])
    _, st = O.run(T["field"], dz0, dump_every=10 ** 9)
    assert st["n_z"] == len(T["znet"]) - 1
    res = {}
    for prec in (gs.PREC_FP64, gs.PREC_MIXED):
        P = gs.Propagator(T, precision=prec)
        P.set_field(T["field"])
        cz, zstep, step_n, calls = P.run(T["znet"], dz0)
        res[prec] = (P.get_field(want_spec=True), cz, zstep, step_n, calls)
        P.close()
    (f64, s64), cz, zstep, step_n, calls = res[gs.PREC_FP64]
    assert calls == 500 and step_n == st["step_n"]
    assert abs(cz - st["z"]) <= 1e-12 * st["z"]
    assert rel(f64, st["field"]) < FP64_TOL
    assert rel(s64, st["bb2"]) < FP64_TOL
    dg, dr = O.dumps(f64), O.dumps(st["field"])
    assert rel(dg["f"], dr["f"]) < FP64_TOL          # fluence
    assert rel(dg["mI"], dr["mI"]) < FP64_TOL        # peak intensity per row
    pg, pr = on_axis_plasma(O, f64), on_axis_plasma(O, st["field"])
    assert pr.max() > 0
    assert rel(pg, pr) < FP64_TOL                    # on-axis plasma density
    # the mixed path at the end of the same run
    (fm, sm), czm, _, step_nm, callsm = res[gs.PREC_MIXED]
    assert callsm == 500 and step_nm == step_n
    err = rel(fm, f64)
    assert err < MIXED_TOL, err
    assert rel(O.dumps(fm)["f"], dg["f"]) < MIXED_TOL


def test_fused_silica_1024x16384_one_step_fp64():
    d = tempfile.mkdtemp(prefix="gs_c2_step_")
    p = configs.fused_silica_c2(d)
    T = tables.build(tables.Config.from_file(p), noise_seed=1234, noise_sigma=1e-4)
    O = oracle.Oracle(T)
    dz0 = tables.init_zstep_kerr(T, T["field"])
    _, st = O.run(T["field"], dz0, steps=1, dump_every=10 ** 9)
    P = gs.Propagator(T, precision=gs.PREC_FP64)
    P.set_field(T["field"])
    cz, zstep, step_n, calls = P.run(T["znet"], dz0, steps=1)
    assert calls == 1 and step_n == st["step_n"]
    assert abs(zstep / st["zstep"] - 1) < 1e-10
    f, s = P.get_field(want_spec=True)
    assert rel(f, st["field"]) < FP64_TOL
    assert rel(s, st["bb2"]) < FP64_TOL
    dg, dr = O.dumps(f), O.dumps(st["field"])
    assert rel(dg["f"], dr["f"]) < FP64_TOL
    assert rel(on_axis_plasma(O, f), on_axis_plasma(O, st["field"])) < FP64_TOL
    P.close()


def test_fused_silica_1024x16384_mixed_error_does_not_grow():
    d = tempfile.mkdtemp(prefix="gs_c2_err_")
    S = gs.Setup(configs.fused_silica_c2(d), noise_seed=1234, noise_sigma=1e-4).as_dict()
    dz = float(S["init_zstep"])
    P64 = gs.Propagator(S, precision=gs.PREC_FP64)
    Pm = gs.Propagator(S, precision=gs.PREC_MIXED)
    errs = []
    done = 0
    for P in (P64, Pm):
        P.set_field(S["field"])
    for n in (20, 200):
        for P in (P64, Pm):
            for _ in range(n - done):
                P.nl_step(dz)
                P.lstep(dz)
        done = n
        errs.append(rel(Pm.get_field(want_spec=False), P64.get_field(want_spec=False)))
    assert errs[1] < 1e-6, errs
    assert errs[1] < 1.5 * errs[0], errs
    P64.close()
    Pm.close()
