"""gs_step_host: propagator() on host-resident FIELD / BIGBUFFER2 (the reference's globals,
solver.h:169) -- both copied in, one call's attempts, both copied out, with BIGBUFFER2's copy
in overlapping the first NL attempt on a copy stream.  It must equal gs_set_field + gs_step +
gs_get_field bit for bit (ZSTEP, STEP_N, FIELD and BIGBUFFER2 after every call), for pinned
and for pageable host buffers, on the mixed 1024 x 16384 workload and on FP64 / mixed grids
whose steps reject attempts."""
import tempfile

import numpy as np
import pytest
import torch

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import tables

pytestmark = pytest.mark.gpu


def host_bufs(T, pinned):
    nr, nt = T["field"].shape
    if pinned:
        f = torch.empty((nr, nt), dtype=torch.complex128, pin_memory=True)
        s = torch.empty((nr, nt), dtype=torch.complex128, pin_memory=True)
        return f, s, f.data_ptr(), s.data_ptr(), f.numpy(), s.numpy()
    f = np.empty((nr, nt), np.complex128)
    s = np.empty((nr, nt), np.complex128)
    return f, s, f.ctypes.data, s.ctypes.data, f, s


def compare(T, prec, dz0, calls, pinned, prep=None):
    znet = T["znet"]
    P1 = gs.Propagator(T, precision=prec)
    P2 = gs.Propagator(T, precision=prec)
    if prep:
        prep(P1)
        prep(P2)
    P1.set_field(T["field"])
    P2.set_field(T["field"])
    _, _, fp, sp, fa, sa = host_bufs(T, pinned)
    P1.get_field_ptr(fp, sp)
    ref_f, ref_s = fa.copy(), sa.copy()
    st1 = st2 = (float(znet[0]), 0, float(dz0), 0)
    for _ in range(calls):
        cz, n_z, zstep, step_n = st1
        if cz >= znet[n_z]:
            n_z += 1
        # the reference sequence: set both, one gs_step, read both
        P2.set_field(ref_f, ref_s)
        z2, s2, _, _ = P2.step(cz, znet[n_z], znet[n_z - 1], zstep, step_n)
        ref_f, ref_s = P2.get_field(want_spec=True)
        z1, s1 = P1.step_host(fp, sp, cz, znet[n_z], znet[n_z - 1], zstep, step_n)
        assert (z1, s1) == (z2, s2)
        assert np.array_equal(fa, ref_f) and np.array_equal(sa, ref_s)
        st1 = (cz + z1, n_z, z1, s1 + 1)
    P1.close()
    P2.close()
    return st1


@pytest.mark.parametrize("pinned", [True, False])
def test_step_host_matches_set_step_get_on_the_1024x16384_workload(pinned):
    d = tempfile.mkdtemp(prefix="gs_sh_c2_")
    S = gs.Setup(configs.fused_silica_c2(d), noise_seed=1234, noise_sigma=1e-4).as_dict()
    compare(S, gs.PREC_MIXED, float(S["init_zstep"]), 3, pinned)


@pytest.mark.parametrize("prec", [gs.PREC_FP64, gs.PREC_MIXED])
def test_step_host_with_rejected_attempts(prec):
    d = tempfile.mkdtemp(prefix="gs_sh_hot_")
    p = configs.hot_solid(d, n_r=128, n_t=2048, power_cr=20.0, tol=1e-2)
    T = tables.build(tables.Config.from_file(p), noise_seed=5, noise_sigma=1e-4)
    dz0 = tables.init_zstep_kerr(T, T["field"])   # ~8x what the controller accepts: rejected
    _, _, _, step_n = compare(T, prec, dz0, 4, True)
    assert step_n > 4   # rejected attempts counted


@pytest.mark.parametrize("prec", [gs.PREC_FP64, gs.PREC_MIXED])
def test_step_host_with_apertures(prec):
    # apertures zero FIELD's outer rows after an accepted step and take BIGBUFFER2 anew from it:
    # after gs_step_host has installed BIGBUFFER2 for the linear step
    d = tempfile.mkdtemp(prefix="gs_sh_ap_")
    over = {"N_R": "128", "N_T": "512", "N_Z": "11", "APERTURE_N": "2", "APERTURE_Z0": "0", "APERTURE_R0": "1.5e-4",
            "APERTURE_Z1": "2.5e-4", "APERTURE_R1": "1e-4"}
    S = gs.Setup(configs.fused_silica_c1(d), overrides=over, noise_seed=1, noise_sigma=1e-4).as_dict()
    compare(S, prec, float(S["init_zstep"]), 3, True)


def test_step_host_with_the_photon_number_check():
    # the check repeats the linear step from the saved BIGBUFFER2 until the photon number moves by
    # at most tol: it reads BIGBUFFER2 before the first linear step
    d = tempfile.mkdtemp(prefix="gs_sh_en_")
    p = configs.hot_solid(d, n_r=128, n_t=2048, power_cr=20.0, tol=1e-2)
    T = tables.build(tables.Config.from_file(p), noise_seed=5, noise_sigma=1e-4)
    compare(T, gs.PREC_MIXED, tables.init_zstep_kerr(T, T["field"]), 3, True,
            prep=lambda P: P.set_energy_tolerance(2e-4, T["qdht_x"], T["r_max"]))
