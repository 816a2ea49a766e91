"""gs_advance: the z-loop (solver_main.cpp:202-225) with propagator()'s step controller
(propagator.cu:139-164) on the device, no host round trip per call.

The same loop through gs_step (the host controller, call by call) and through gs_advance must
agree bit for bit: CURRENT_Z, ZSTEP, STEP_N (rejected attempts counted), the number of calls,
the fields at every ZNET point (the dumps) and at the end.  Covered: the 1024 x 16384 workload
(16384-point FP32 rows with the compact tensor-core plan), a strongly ionizing 640-row grid whose
first proposal is rejected and whose calls are clamped to close ZNET points (dumps in between),
mixed grids of shorter rows on the fused stage kernels (per-stage launches and the four-stage
launch), which take their step sizes from the device too, and FP64, whose calls take the host
(gs_step per call).
"""
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import tables

pytestmark = pytest.mark.gpu


def both(T, dz0, steps, prec=gs.PREC_MIXED):
    res = []
    for device in (False, True):
        P = gs.Propagator(T, precision=prec)
        P.set_field(T["field"])
        dumps = []
        out = P.run(T["znet"], dz0, steps=steps, device=device,
                    on_dump=lambda n, p: dumps.append((n, p.get_field(want_spec=False))))
        res.append((out, dumps, P.get_field(want_spec=True), P.launch_count()))
        P.close()
    return res


def same(a, b):
    (oa, da, (fa, sa), _), (ob, db, (fb, sb), _) = a, b
    assert oa == ob, (oa, ob)   # CURRENT_Z, ZSTEP, STEP_N, calls
    assert [n for n, _ in da] == [n for n, _ in db]
    for (_, x), (_, y) in zip(da, db):
        assert np.array_equal(x, y)
    assert np.array_equal(fa, fb) and np.array_equal(sa, sb)


def test_advance_matches_host_loop_on_the_1024x16384_workload():
    d = tempfile.mkdtemp(prefix="gs_adv_c2_")
    S = gs.Setup(configs.fused_silica_c2(d), noise_seed=1234, noise_sigma=1e-4).as_dict()
    host, dev = both(S, float(S["init_zstep"]), 8)
    same(host, dev)
    assert host[0][3] == 8


def test_advance_with_rejections_and_znet_points():
    d = tempfile.mkdtemp(prefix="gs_adv_hot_")
    p = configs.hot_solid(d, n_r=640, n_t=16384, power_cr=20.0, tol=1e-2, window=1.6e-12)
    T = tables.build(tables.Config.from_file(p), noise_seed=21, noise_sigma=1e-4)
    # the Kerr estimate of the first step is ~4x what the controller accepts on this grid: the
    # first attempt is rejected; ZNET points every 2 um, calls of ~2e-8 m: the whole run (all
    # ZNET points, a dump at each) within the call budget
    dz0 = tables.init_zstep_kerr(T, T["field"])
    host, dev = both(T, dz0, 400)
    same(host, dev)
    (cz, zstep, step_n, calls), dumps = host[0], host[1]
    assert 0 < calls < 400
    assert step_n > calls          # rejected attempts counted in STEP_N
    assert [n for n, _ in dumps] == list(range(len(T["znet"])))   # every ZNET point dumped


def test_advance_on_short_rows():
    # FP64 (host-driven) and mixed on the per-stage fused kernels (device-driven)
    d = tempfile.mkdtemp(prefix="gs_adv_small_")
    p = configs.hot_solid(d, n_r=128, n_t=1024, power_cr=20.0, tol=1e-2)
    T = tables.build(tables.Config.from_file(p), noise_seed=5, noise_sigma=1e-4)
    dz0 = tables.init_zstep_kerr(T, T["field"])
    for prec in (gs.PREC_FP64, gs.PREC_MIXED):
        host, dev = both(T, dz0, 6, prec)
        same(host, dev)
        assert host[0][2] > host[0][3]   # rejected attempts on the way


def test_advance_on_the_four_stage_fused_kernel():
    # 8192-point rows, enough of them for the four-stage launch; ZNET points every 2 um with dumps
    d = tempfile.mkdtemp(prefix="gs_adv_f4_")
    p = configs.hot_solid(d, n_r=1920, n_t=8192, power_cr=20.0, tol=1e-2, window=1.6e-12)
    T = tables.build(tables.Config.from_file(p), noise_seed=9, noise_sigma=1e-4)
    dz0 = tables.init_zstep_kerr(T, T["field"])
    host, dev = both(T, dz0, 12)
    same(host, dev)
    assert host[0][3] == 12 and host[0][2] > 12   # rejected attempts on the way
    P = gs.Propagator(T)   # the grid takes the four-stage kernel: one NL launch per attempt
    P.set_field(T["field"])
    n0 = P.launch_count()
    P.nl_step(dz0)
    assert P.launch_count() - n0 == 1
    P.close()


def test_advance_on_paired_rows():
    # 32768-point FP32 rows over a pair of CTAs (solid and the gas build's argon); the paired
    # kernels take their step sizes from the device as well
    d = tempfile.mkdtemp(prefix="gs_adv_pair_")
    p = configs.hot_solid(d, n_r=128, n_t=32768, power_cr=20.0, tol=1e-2, window=1.6e-12)
    T = tables.build(tables.Config.from_file(p), noise_seed=13, noise_sigma=1e-4)
    host, dev = both(T, tables.init_zstep_kerr(T, T["field"]), 5)
    same(host, dev)
    assert host[0][3] == 5
    d = tempfile.mkdtemp(prefix="gs_adv_ar_")
    pa = configs.argon_c5(d, cep=0.0, name="argon_adv", build="gas_qdht")
    S = gs.Setup(pa, overrides={"N_R": "128"}, noise_seed=200, noise_sigma=1e-4).as_dict()
    host, dev = both(S, float(S["init_zstep"]), 4)
    same(host, dev)
    assert host[0][3] == 4
