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


def test_batch_advance_matches_each_pulse_advanced_alone():
    """gs_batch_advance: every pulse's adaptive controller on the device, one graph launch per
    attempt of all pulses; each pulse's CURRENT_Z, ZSTEP, STEP_N, calls and FIELD / BIGBUFFER2
    equal gs_advance on it alone, bit for bit.  Strongly ionizing pulses (rejected attempts) on
    the per-stage fused kernels and on the 16384-point row kernel."""
    from oracle import tables
    grids = [(128, 1024, 5, None), (256, 2048, 6, None), (128, 4096, 7, None), (640, 16384, 8, 1.6e-12)]
    Ts = []
    for nr, nt, seed, win in grids:
        d = tempfile.mkdtemp(prefix="gs_badv_")
        kw = dict(n_r=nr, n_t=nt, power_cr=20.0, tol=1e-2)
        if win:
            kw["window"] = win
        p = configs.hot_solid(d, **kw)
        Ts.append(tables.build(tables.Config.from_file(p), noise_seed=seed, noise_sigma=1e-4))
    dz0 = [tables.init_zstep_kerr(T, T["field"]) for T in Ts]
    K = 7
    alone = []
    for T, d0 in zip(Ts, dz0):
        P = gs.Propagator(T, precision=gs.PREC_MIXED)
        P.set_field(T["field"])
        out = P.advance(T["znet"], 1, float(T["znet"][0]), d0, 0, K)
        alone.append((out, P.get_field(want_spec=True)))
        P.close()
    Ps = [gs.Propagator(T, precision=gs.PREC_MIXED) for T in Ts]
    for P, T in zip(Ps, Ts):
        P.set_field(T["field"])
    B = gs.Batch(Ps)
    cz, dz, sn, calls, reached = B.advance([T["znet"] for T in Ts], [1] * len(Ts), [float(T["znet"][0]) for T in Ts],
                                           dz0, [0] * len(Ts), K)
    for i, P in enumerate(Ps):
        (a_cz, a_dz, a_sn, a_calls, a_reached), (fa, sa) = alone[i]
        assert (cz[i], dz[i], int(sn[i]), int(calls[i]), bool(reached[i])) == (a_cz, a_dz, a_sn, a_calls, a_reached), i
        f, s = P.get_field(want_spec=True)
        assert np.array_equal(f, fa) and np.array_equal(s, sa), i
    assert all(int(calls[i]) == K for i in range(len(Ts)))
    assert all(int(sn[i]) > K for i in range(len(Ts)))   # rejected attempts counted in STEP_N
    # a second call continues from there
    cz2, dz2, sn2, calls2, _ = B.advance([T["znet"] for T in Ts], [1] * len(Ts), cz, dz, sn, 3)
    assert all(int(c) == 3 for c in calls2) and all(cz2 > cz) and all(sn2 >= sn + 3)
    B.close()
    for P in Ps:
        P.close()
