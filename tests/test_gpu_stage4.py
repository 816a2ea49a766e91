"""The four-stage NL kernel of 16384-point FP32 rows against the FP64 oracle.

nl_row16k_kernel (gs_nl_row16k.cu) runs all four RK4 stages of a row in one CTA, keeps the RK4
sum and the row's spectrum in tensor memory, and on steps after the first reads FIELD from the
masked inverse's compact window columns.  It is chosen for mixed handles with n_t = 16384,
1024 threads per row and at least four waves of rows (n_r >= 4 x resident CTAs: 608 rows on
152 SMs), which is the 1024 x 16384 fused-silica workload's kernel.  These tests run it on 640
rows of a strongly ionizing pulse (rows near the axis ionize, the outer rows take the
no-ionization branch) and compare with calculate_NLstep / propagator() restated in FP64
(propagator.cu:125-266, 375-425).

Bar: 1e-5 relative L2 (the mixed path's accuracy target), as for the other mixed tests.
"""
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5    # relative L2 against the FP64 oracle
MODES_TOL = 2e-6    # four-stage vs per-stage launches: the same arithmetic, FP32 rounding apart
ROWS = 640          # >= 4 waves of one 1024-thread CTA per SM on 152 SMs


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


@pytest.fixture(scope="module")
def hot16k():
    d = tempfile.mkdtemp(prefix="gs_stage4_")
    p = configs.hot_solid(d, n_r=ROWS, n_t=16384, power_cr=20.0, tol=1e-2, window=1.6e-12)
    T = tables.build(tables.Config.from_file(p), noise_seed=21, noise_sigma=1e-4)
    return T, oracle.Oracle(T)


def _rows(T, n):
    """The set-up restricted to the first n radial rows: the NL step treats rows independently
    and reads only per-omega tables, so its rows agree with the full grid's."""
    S = dict(T)
    S["n_r"] = n
    S["kt2"] = T["kt2"][:n]
    S["qdht_m1"] = T["qdht_m1"][:n]
    S["qdht_c"] = np.ascontiguousarray(T["qdht_c"][:n, :n])
    S["field"] = np.ascontiguousarray(T["field"][:n])
    return S


def test_stage4_nl_step_vs_oracle(hot16k):
    T, O = hot16k
    dz = tables.init_zstep_kerr(T, T["field"])
    bb1, a2, n2 = O.nl_step(T["field"], dz)
    P = gs.Propagator(T, precision=gs.PREC_MIXED)
    assert P.nl_threads() == 1024
    P.set_field(T["field"])
    P.nl_timing(enable=True)
    ga2, gn2 = P.nl_step(dz)
    _, stages, launches = P.nl_timing(enable=False)
    assert (stages, launches) == (4, 1)   # the four stages in one launch: nl_row16k_kernel
    g = P.get_nl()
    assert rel(g, bb1) < MIXED_TOL
    assert abs(ga2 - a2) / a2 < 1e-6
    assert abs(gn2 - n2) / n2 < MIXED_TOL
    # both branches ran: ionizing rows near the axis, rows without ionization further out
    e = np.fft.ifft(T["field"][0])
    assert O.plasma(e)[0].max() > 1e26
    e_out = np.fft.ifft(T["field"][ROWS - 1])
    assert O.plasma(e_out)[0].max() == 0
    # rows across the ionizing core and its edge, each to 10x the bar; and every element of the
    # grid within the bar of the largest increment (the outer rows' increments, ~1e-39, lie below
    # FP32's normal range and are compared in this absolute sense only)
    for r in (0, 1, 20, 50, 100):
        assert rel(g[r], bb1[r]) < 10 * MIXED_TOL, r
    assert np.abs(g - bb1).max() <= MIXED_TOL * np.abs(bb1).max()
    P.close()


def test_stage4_propagator_steps_vs_oracle(hot16k):
    """Three propagator() calls: steps 2 and 3 read FIELD from the compact window columns that
    the previous step's masked inverse left; final field, spectrum, fluence and on-axis plasma
    density against the oracle."""
    T, O = hot16k
    dz0 = tables.init_zstep_kerr(T, T["field"])
    out, st = O.run(T["field"], dz0, steps=3)
    P = gs.Propagator(T, precision=gs.PREC_MIXED)
    P.set_field(T["field"])
    P.nl_timing(enable=True)
    cz, zstep, step_n, calls = P.run(T["znet"], dz0, steps=3)
    _, stages, launches = P.nl_timing(enable=False)
    assert calls == 3 and step_n == st["step_n"]
    assert launches * 4 == stages   # one launch per NL attempt
    assert abs(zstep / st["zstep"] - 1) < 1e-4
    f, s = P.get_field()
    assert rel(f, st["field"]) < MIXED_TOL
    assert rel(s, st["bb2"]) < MIXED_TOL
    dg, dr = O.dumps(f), O.dumps(st["field"])
    assert rel(dg["f"], dr["f"]) < MIXED_TOL
    assert rel(O.plasma(np.fft.ifft(f[0]))[0], O.plasma(np.fft.ifft(st["field"][0]))[0]) < 10 * MIXED_TOL
    P.close()


def test_stage4_agrees_with_per_stage_launches(hot16k):
    """The same rows stepped by one launch per RK4 stage (a grid of 256 rows, under four waves)
    and by the four-stage kernel (640 rows): the NL increments of the shared rows agree to FP32
    rounding."""
    T, _ = hot16k
    n = 256
    S = _rows(T, n)
    dz = tables.init_zstep_kerr(T, T["field"])
    big = gs.Propagator(T, precision=gs.PREC_MIXED)
    small = gs.Propagator(S, precision=gs.PREC_MIXED)
    big.set_field(T["field"])
    small.set_field(S["field"])
    counts = []
    for P in (big, small):
        P.nl_timing(enable=True)
        P.nl_step(dz)
        counts.append(P.nl_timing(enable=False)[2])
    assert counts == [1, 4]   # four-stage launch vs four per-stage launches
    assert rel(big.get_nl()[:n], small.get_nl()) < MODES_TOL
    big.close()
    small.close()


def test_table_reupload_expands_compact_field(hot16k):
    """Re-uploading the tables on a handle whose FIELD is held compactly (after a step of the
    four-stage grid) first expands FIELD through the old column lists: the field read after the
    re-upload is the one read before it, and stepping on agrees with a handle that was never
    re-uploaded: the field bit for bit, BIGBUFFER2 (kept as double-float pairs across the
    rebuild) to below FP32 resolution."""
    T, _ = hot16k
    dz = 2e-8
    a = gs.Propagator(T, precision=gs.PREC_MIXED)
    b = gs.Propagator(T, precision=gs.PREC_MIXED)
    for P in (a, b):
        P.set_field(T["field"])
        P.nl_step(dz)
        P.lstep(dz)
        P.nl_step(dz)   # reads FIELD compactly
        P.lstep(dz)     # leaves it compact again
    fb, sb = b.get_field(want_spec=True)
    a.upload_tables(T)
    fa, sa = a.get_field(want_spec=True)
    assert np.array_equal(fa, fb) and np.array_equal(sa, sb)
    assert np.abs(fa).max() > 0
    for P in (a, b):
        P.nl_step(dz)
        P.lstep(dz)
    fa, sa = a.get_field(want_spec=True)
    fb, sb = b.get_field(want_spec=True)
    assert np.array_equal(fa, fb)
    assert np.all(np.abs(sa - sb) <= 2.0 ** -30 * np.abs(sb))
    a.close()
    b.close()
