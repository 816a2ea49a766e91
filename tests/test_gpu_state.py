"""Energy / photon number (gs_energy), the optional photon-number check of gs_step, and
checkpoints (gs_checkpoint_save / gs_checkpoint_load), through the C ABI.

* gs_energy is the sum over omega of the reference's average spectrum (dump_types.cpp:427-457),
  the oracle's restatement of that dump summed here: 1e-12 in FP64.
* The check, on a strongly ionizing grid (photons absorbed by the plasma): with a tolerance
  it rejects and halves steps until the photon number changes by at most the tolerance per step;
  with it off, steps are those of the reference's controller, bit for bit.
* A checkpoint written mid-run and loaded into a fresh handle continues exactly as the
  original does (both precisions), z-loop state included.
"""
import os
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables

pytestmark = pytest.mark.gpu


def hot(n_r=128, n_t=1024, seed=5):
    d = tempfile.mkdtemp(prefix="gs_state_")
    p = configs.hot_solid(d, n_r=n_r, n_t=n_t, power_cr=20.0, tol=1e-2)
    return tables.build(tables.Config.from_file(p), noise_seed=seed, noise_sigma=1e-4)


@pytest.mark.parametrize("prec,tol", [(gs.PREC_FP64, 1e-12), (gs.PREC_MIXED, 1e-6)])
def test_energy_is_the_sum_of_the_average_spectrum(prec, tol):
    T = hot()
    O = oracle.Oracle(T)
    P = gs.Propagator(T, precision=prec)
    P.set_field(T["field"])
    dz = tables.init_zstep_kerr(T, T["field"])
    for _ in range(2):   # a mixed handle's FIELD is then the masked inverse's result
        P.nl_step(dz)
        P.lstep(dz)
    f = P.get_field(want_spec=False)
    E, N = P.energy(T["qdht_x"], T["r_max"])
    s = O.dumps(f)["s"]
    om = np.asarray(T["omega"])
    assert abs(E / s.sum() - 1) < tol
    assert abs(N / s[om > 0].dot(1.0 / om[om > 0]) - 1) < tol
    P.close()


def test_photon_number_check_bounds_the_loss_per_step():
    T = hot(n_r=64, n_t=2048)
    znet = T["znet"]
    dz0 = tables.init_zstep_kerr(T, T["field"])
    # off: identical to the reference's controller alone
    a = gs.Propagator(T)
    b = gs.Propagator(T)
    b.set_energy_tolerance(0.0)
    for P in (a, b):
        P.set_field(T["field"])
        P.run(znet, dz0, steps=4)
    assert np.array_equal(a.get_field(want_spec=False), b.get_field(want_spec=False))
    # on, tight: steps are halved until the photon number moves by at most tol per step
    c = gs.Propagator(T)
    c.set_field(T["field"])
    n0 = c.energy(T["qdht_x"], T["r_max"])[1]
    tol = 2e-4
    c.set_energy_tolerance(tol, T["qdht_x"], T["r_max"])
    cz, zstep, step_n = float(znet[0]), dz0, 0
    rel = []
    for _ in range(4):
        nb = c.energy(T["qdht_x"], T["r_max"])[1]
        zstep, step_n, _, _ = c.step(cz, znet[1], znet[0], zstep, step_n)
        step_n += 1
        cz += zstep
        na = c.energy(T["qdht_x"], T["r_max"])[1]
        rel.append(abs(na / nb - 1))
        assert c.energy_stats()[0] == pytest.approx(rel[-1], rel=1e-12, abs=1e-18)
    last, rejections = c.energy_stats()
    assert rejections > 0                   # the plasma absorbs more than tol per full step
    assert max(rel) <= tol
    assert c.energy(T["qdht_x"], T["r_max"])[1] < n0   # photons are lost, not gained
    for P in (a, b, c):
        P.close()


@pytest.mark.parametrize("prec", [gs.PREC_FP64, gs.PREC_MIXED])
def test_checkpoint_continues_exactly(prec):
    T = hot(seed=9)
    znet = T["znet"]
    dz0 = tables.init_zstep_kerr(T, T["field"])
    a = gs.Propagator(T, precision=prec)
    a.set_field(T["field"])
    cz, zstep, step_n, n_z = float(znet[0]), dz0, 0, 1
    for _ in range(3):
        zstep, step_n, _, _ = a.step(cz, znet[n_z], znet[n_z - 1], zstep, step_n)
        step_n += 1
        cz += zstep
    path = os.path.join(tempfile.mkdtemp(prefix="gs_ckpt_"), "state.gsckpt")
    a.checkpoint_save(path, cz, zstep, n_z, step_n)
    b = gs.Propagator(T, precision=prec)
    st = b.checkpoint_load(path)
    assert st == {"z": cz, "zstep": zstep, "n_z": n_z, "step_n": step_n}
    fa0, sa0 = a.get_field()
    fb0, sb0 = b.get_field()
    assert np.array_equal(fa0, fb0) and np.array_equal(sa0, sb0)
    za, zb = (cz, zstep, step_n), (st["z"], st["zstep"], st["step_n"])
    for P, (z, dz, sn) in ((a, za), (b, zb)):
        for _ in range(3):
            dz, sn, _, _ = P.step(z, znet[n_z], znet[n_z - 1], dz, sn)
            sn += 1
            z += dz
    fa, sa = a.get_field()
    fb, sb = b.get_field()
    assert np.array_equal(fa, fb) and np.array_equal(sa, sb)
    # a checkpoint of another grid is refused
    other = gs.Propagator(hot(n_r=256, n_t=1024), precision=prec)
    with pytest.raises(gs.GsError) as ei:
        other.checkpoint_load(path)
    assert "grid or precision" in str(ei.value)
    for P in (a, b, other):
        P.close()
