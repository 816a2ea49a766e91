"""Device dump reductions and the whole-run driver (.udf files) against the oracle and the
reference's own golden dumps."""
import os
import struct
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables
from tests.golden_cfg import golden_config_dir, load_golden

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


def read_udf(path):
    with open(path, "rb") as f:
        b = f.read()
    assert b[:7] == b"UDF1.0\x00"
    hdr = struct.unpack("6i", b[7:31])
    a = np.frombuffer(b, dtype=np.complex128 if hdr[1] else np.float64, offset=31)
    return hdr, a.reshape(hdr[5], -1)


@pytest.mark.parametrize("prec,tol", [(gs.PREC_FP64, 1e-12), (gs.PREC_MIXED, 2e-6)])
def test_dump_reductions_match_oracle(prec, tol):
    d = tempfile.mkdtemp()
    p = configs.hot_solid(d, n_r=128, n_t=1024, power_cr=20.0, tol=1e-2)
    T = tables.build(tables.Config.from_file(p), noise_seed=2, noise_sigma=1e-4)
    O = oracle.Oracle(T)
    P = gs.Propagator(T, precision=prec)
    P.set_field(T["field"])
    g = P.dumps(T["qdht_x"], T["r_max"])
    r = O.dumps(T["field"])
    for k in ("mI", "f", "pm", "fa", "s"):
        assert rel(g[k], r[k]) < tol, k
    assert r["pm"].max() > 1e25
    e = P.time_field()
    assert rel(e, np.fft.ifft(T["field"], axis=1)) < tol


def test_run_config_writes_the_golden_udf_files():
    """bin/fil_SiO2_1d.txt through the driver: same .udf headers as the reference's files
    and the same values as its golden dumps (bounds of the oracle's own pinning)."""
    g = load_golden()
    d = golden_config_dir()
    out = tempfile.mkdtemp(prefix="gs_udf_")
    st = gs.run_config(os.path.join(d, "fil_SiO2_1d.txt"), out, overrides={"NZ_DENOM4": "64"})
    assert st["n_z"] == 127 and st["calls"] == 127
    sl = g["slabs"]
    for key, tol in (("f", 5e-8), ("fa", 1e-7), ("mI", 5e-8), ("pm", 0.0), ("s", 1e-8)):
        hdr, a = read_udf(os.path.join(out, f"fil_SiO2__{key}.udf"))
        assert hdr[0] == 8 and list(hdr[1:]) == list(g["hdr_" + key]), key   # fixture: (iscomplex, tN, xN, yN, zN)
        ref = g["udf_" + key]
        if key == "pm":
            assert np.all(a[sl] == 0)
        else:
            assert rel(a[sl], ref) < tol, key
    hdr, full = read_udf(os.path.join(out, "fil_SiO2__full.udf"))
    assert hdr == (8, 1, 512, 512, 1, 2)
    T = tables.build(tables.Config.from_file(os.path.join(d, "fil_SiO2_1d.txt")))
    e0 = np.fft.ifft(T["field"], axis=1).reshape(-1)
    assert rel(full[0], e0) < 1e-12
