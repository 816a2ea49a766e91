"""Apertures (propagator.cu:232-261) applied by gs_step, against the oracle (FP64 1e-10),
with the product's own set-up parsing APERTURE_N / APERTURE_Zi / APERTURE_Ri."""
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables

pytestmark = pytest.mark.gpu


def test_apertures_match_oracle():
    d = tempfile.mkdtemp(prefix="gs_gap_")
    p = configs.fused_silica_c1(d)
    over = {"N_R": "64", "N_T": "512", "N_Z": "11", "APERTURE_N": "2", "APERTURE_Z0": "0", "APERTURE_R0": "1.5e-4",
            "APERTURE_Z1": "2.5e-4", "APERTURE_R1": "1e-4"}
    S = gs.Setup(p, overrides=over, noise_seed=1, noise_sigma=1e-4).as_dict()
    T = tables.build(tables.Config.from_file(p, overrides=over), noise_seed=1, noise_sigma=1e-4)
    assert np.array_equal(S["aperture_z"], T["aperture_z"]) and np.array_equal(S["aperture_r"], T["aperture_r"])
    O = oracle.Oracle(T)
    dz0 = tables.init_zstep_kerr(T, T["field"])
    R = np.asarray(T["qdht_x"]) * T["r_max"]
    for steps in (1, 4):
        out, st = O.run(T["field"], dz0, steps=steps)
        P = gs.Propagator(S, precision=gs.PREC_FP64)   # registers the config's apertures
        P.set_field(S["field"])
        P.run(S["znet"], S["init_zstep"], steps=steps)
        f, sp = P.get_field(want_spec=True)
        assert np.linalg.norm(f - st["field"]) <= 1e-10 * np.linalg.norm(st["field"])
        assert np.linalg.norm(sp - st["bb2"]) <= 1e-10 * np.linalg.norm(st["bb2"])
        assert np.all(f[R > (1.5e-4 if steps == 1 else 1e-4)] == 0)
        P.close()
