"""Batches of independent pulses (gs_batch_*): a batch z-step, captured in a CUDA graph or
issued directly, gives each pulse exactly (bitwise) what stepping it alone gives."""
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs

pytestmark = pytest.mark.gpu


def _pulses(precision):
    d = tempfile.mkdtemp(prefix="gs_batch_")
    cfgs = configs.c3_batch(d, seed=3, n=4)
    S = [gs.Setup(p, noise_seed=10 + i, noise_sigma=1e-4).as_dict() for i, (p, _) in enumerate(cfgs)]
    return S, [gs.Propagator(s, precision=precision) for s in S]


@pytest.mark.parametrize("precision", [gs.PREC_MIXED, gs.PREC_FP64])
def test_batch_matches_single_pulse_steps(precision):
    S, P = _pulses(precision)
    dz = np.array([s["init_zstep"] for s in S])
    # reference: each pulse alone, nl_step + lstep with the same fixed dz
    ref = []
    for s, p in zip(S, P):
        p.set_field(s["field"])
        for _ in range(3):
            p.nl_step(float(s["init_zstep"]))
            p.lstep(float(s["init_zstep"]))
        ref.append(p.get_field(want_spec=True))
    for graph in (True, False):
        for s, p in zip(S, P):
            p.set_field(s["field"])
        B = gs.Batch(P)
        B.step(dz, 2, graph=graph)
        B.step(dz, 1, graph=graph)   # a graph is reused for the same step sizes
        for i, p in enumerate(P):
            f, sp = p.get_field(want_spec=True)
            assert np.array_equal(f, ref[i][0]) and np.array_equal(sp, ref[i][1]), (graph, i)
        assert B.launch_count() > 0
        B.close()


def test_batch_rejects_bad_arguments():
    S, P = _pulses(gs.PREC_MIXED)
    B = gs.Batch(P)
    with pytest.raises(gs.GsError):     # field not set
        B.step(np.full(len(P), 1e-6), 1)
    for s, p in zip(S, P):
        p.set_field(s["field"])
    with pytest.raises(gs.GsError):
        B.step(np.array([1e-6, -1.0, 1e-6, 1e-6]), 1)
    with pytest.raises(gs.GsError):
        gs.Batch([P[0], P[0]])


def test_batch_autotune_restores_state_and_keeps_results():
    S, P = _pulses(gs.PREC_MIXED)
    dz = np.array([s["init_zstep"] for s in S])
    for s, p in zip(S, P):
        p.set_field(s["field"])
    B = gs.Batch(P)
    before = [p.get_field(want_spec=True) for p in P]
    ms_def, ms_tun, chose = B.autotune(dz)
    assert ms_def > 0 and ms_tun > 0
    for b, p in zip(before, P):
        f, sp = p.get_field(want_spec=True)
        assert np.array_equal(f, b[0]) and np.array_equal(sp, b[1])
    B.step(dz, 2)
    # each pulse alone with the same launch shape gives the same result
    for s, p in zip(S, P):
        got = p.get_field(want_spec=False)
        p.set_field(s["field"])
        for _ in range(2):
            p.nl_step(float(s["init_zstep"]))
            p.lstep(float(s["init_zstep"]))
        assert np.array_equal(p.get_field(want_spec=False), got)
