"""The GS_CHECK build (``python -m gsolver_gb300.build --check``, loaded when GS_CHECK=1 is set
at import): the hot kernels test the indices they take from index tables -- the compact
window-column maps of the NL kernel's FIELD gather and BIGBUFFER1 stores and of the QDHT
epilogue, the rate-table rows -- before each access; a failed test sets a bit in the error word,
skips the access (no trap) and the call returns GS_ERR_CUDA "index out of bounds".

* gs_selftest_bounds makes the test fail on purpose on an index that still lies inside its
  buffer (so nothing could fault either way) and must report it, the handle usable afterwards;
* on the 1024 x 16384 workload (mixed, gs_advance), on an ionizing 640 x 16384 grid (mixed,
  gs_step) and on an ionizing 256 x 2048 grid (the fused stage kernels, gs_advance) the checked
  build reports nothing and gives the main build's results bit for bit."""
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import gsolver_gb300 as gs  # noqa: E402
from gsolver_gb300 import configs  # noqa: E402


def workloads(out):
    """Run the two cases with whichever library this process loaded; save the results."""
    from oracle import tables
    res = {}
    d = tempfile.mkdtemp(prefix="gs_chk_c2_")
    S = gs.Setup(configs.fused_silica_c2(d), noise_seed=1234, noise_sigma=1e-4).as_dict()
    P = gs.Propagator(S, precision=gs.PREC_MIXED)
    P.set_field(S["field"])
    cz, dz, sn, calls, _ = P.advance(S["znet"], 1, float(S["znet"][0]), float(S["init_zstep"]), 0, 3)
    f, s = P.get_field(want_spec=True)
    res.update(c2_f=f, c2_s=s, c2_scalars=np.array([cz, dz, sn, calls]))
    P.close()
    d = tempfile.mkdtemp(prefix="gs_chk_hot_")
    p = configs.hot_solid(d, n_r=640, n_t=16384, power_cr=20.0, tol=1e-2, window=1.6e-12)
    T = tables.build(tables.Config.from_file(p), noise_seed=21, noise_sigma=1e-4)
    P = gs.Propagator(T, precision=gs.PREC_MIXED)
    P.set_field(T["field"])
    dz = tables.init_zstep_kerr(T, T["field"])
    znet = T["znet"]
    cz, sn = float(znet[0]), 0
    for _ in range(2):
        dz, sn, _, _ = P.step(cz, znet[1], znet[0], dz, sn)
        cz += dz
        sn += 1
    f, s = P.get_field(want_spec=True)
    res.update(hot_f=f, hot_s=s, hot_scalars=np.array([cz, dz, sn]))
    P.close()
    # shorter rows on the fused stage kernels (their compact BIGBUFFER1 columns and rate rows)
    d = tempfile.mkdtemp(prefix="gs_chk_fused_")
    p = configs.hot_solid(d, n_r=256, n_t=2048, power_cr=20.0, tol=1e-2)
    T = tables.build(tables.Config.from_file(p), noise_seed=23, noise_sigma=1e-4)
    P = gs.Propagator(T, precision=gs.PREC_MIXED)
    P.set_field(T["field"])
    out_adv = P.advance(T["znet"], 1, float(T["znet"][0]), tables.init_zstep_kerr(T, T["field"]), 0, 4)
    f, s = P.get_field(want_spec=True)
    res.update(fused_f=f, fused_s=s, fused_scalars=np.array(out_adv[:4], dtype=np.float64))
    P.close()
    np.savez(out, **res)


def child(out):
    """In the GS_CHECK process: the build flag, the self-test, then the workloads."""
    assert gs.LIB_PATH.endswith(os.path.join("_build_check", "libgsolver_gb300.so")), gs.LIB_PATH
    L = gs.load_library()
    assert L.gs_check_build() == 1
    from oracle import tables
    d = tempfile.mkdtemp(prefix="gs_chk_st_")
    p = configs.hot_solid(d, n_r=128, n_t=2048, power_cr=20.0, tol=1e-2)
    T = tables.build(tables.Config.from_file(p), noise_seed=5, noise_sigma=1e-4)
    P = gs.Propagator(T, precision=gs.PREC_MIXED)
    P.set_field(T["field"])
    try:
        P.selftest_bounds()
        raise AssertionError("gs_selftest_bounds did not report")
    except gs.GsError as e:
        assert e.code == gs.GS_ERR_CUDA and "index out of bounds" in str(e), e
    znet = T["znet"]
    P.step(float(znet[0]), znet[1], znet[0], tables.init_zstep_kerr(T, T["field"]), 0)   # still usable
    P.close()
    workloads(out)


pytestmark = pytest.mark.gpu


def test_check_build_reports_and_matches_the_main_build():
    from gsolver_gb300 import build as B
    B.build(check=True)
    assert gs.load_library().gs_check_build() == 0
    d = tempfile.mkdtemp(prefix="gs_chk_")
    out_c, out_m = os.path.join(d, "check.npz"), os.path.join(d, "main.npz")
    env = dict(os.environ, GS_CHECK="1")
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--child", out_c], env=env, cwd=ROOT,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    workloads(out_m)
    c, m = np.load(out_c), np.load(out_m)
    for k in m.files:
        assert np.array_equal(c[k], m[k]), k


if __name__ == "__main__" and len(sys.argv) == 3 and sys.argv[1] == "--child":
    child(sys.argv[2])
