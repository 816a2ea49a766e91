"""Known-answer tests of the oracle's physics pieces (no GPU)."""
import math
import tempfile

import numpy as np

from gsolver_gb300 import configs
from oracle import oracle, tables


def small(**kw):
    d = tempfile.mkdtemp()
    p = configs.hot_solid(d, **kw)
    return tables.build(tables.Config.from_file(p))


def test_qdht_is_an_involution_and_preserves_energy():
    T = small(n_r=64, n_t=64)
    O = oracle.Oracle(T)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
    y = O.qdht(x)
    assert np.linalg.norm(O.qdht(y) - x) / np.linalg.norm(x) < 1e-6
    # Parseval for the QDHT: sum |f|^2 / m1^2 is conserved (Guizar-Sicairos & Gutierrez-Vega)
    m1 = T["qdht_m1"][:, None]
    e0 = np.sum(np.abs(x) ** 2 / m1 ** 2)
    e1 = np.sum(np.abs(y) ** 2 / m1 ** 2)
    assert abs(e1 / e0 - 1) < 1e-6


def test_raman_response_integrates_to_one_at_dc():
    T = small(n_r=8, n_t=4096, window=2e-12)
    R0 = T["raman_func"][0]
    # R(0) = f_R * (Riemann sum of the normalised oscillator) + (1 - f_R) ~ 1
    assert abs(R0.real - 1.0) < 2e-3
    assert abs(R0.imag) < 1e-12


def test_plasma_flat_top_matches_heun_closed_form():
    """Constant intensity, no avalanche/recombination: rho(t) = rho0 + W t exactly."""
    T = small(n_r=4, n_t=512)
    T = dict(T)
    T["avalanche_cs"] = 0.0
    T["recombination_tau"] = 1e300
    O = oracle.Oracle(T)
    E = np.full(512, math.sqrt(40.0) + 0j)            # I = 40 in scaled units (4e13 W/cm^2)
    pro, loss = O.plasma(E)
    # the first step sees E_0 = 0 (reference quirk): k1 = 0, k2 = dt W
    lnI = math.log(40.0) + 36.841361487904734
    n = int(math.floor((lnI - tables.IONIZATION_MIN_I_LN) / tables.IONIZATION_I_LN_TOLERANCE))
    lnIn = tables.IONIZATION_MIN_I_LN + n * tables.IONIZATION_I_LN_TOLERANCE
    r = T["rate_ln"]
    W = math.exp(r[n] + (lnI - lnIn) * (r[n + 1] - r[n]) / tables.IONIZATION_I_LN_TOLERANCE)
    dt = T["tstep"] * T["ionrate_denom"]
    expect = np.concatenate([[0.0], 0.5 * dt * W + dt * W * np.arange(511)])
    assert np.allclose(pro, expect, rtol=1e-12, atol=0)
    assert np.all(loss[1:-1] != 0) and loss[0] == 0 and loss[-1] == 0


def test_keldysh_multiphoton_slope():
    """At low intensity the Keldysh rate scales as I^K, K = ceil(U / hbar omega) (6 for 9 eV at 800 nm)."""
    T = small(n_r=4, n_t=64)
    r = T["rate_ln"]
    i0, i1 = 100, 400       # ~1.4e13 .. 2.7e13 W/m^2 region of the table
    slope = (r[i1] - r[i0]) / ((i1 - i0) * tables.IONIZATION_I_LN_TOLERANCE)
    assert 5.5 < slope < 6.5
    assert r[-1] == 0.0          # top entry left unset, as the reference leaves it


def test_linear_diffraction_of_collimated_gaussian():
    """Linear run (no NL): the beam radius follows w(z) = w0 sqrt(1 + (z/zR)^2)."""
    w0 = 20e-6
    T = small(n_r=128, n_t=64, w0=w0, power_cr=1e-6, r_max=10 * w0, z_max=4e-3, n_z=3, tol=1e3)
    O = oracle.Oracle(T, nonlinear=False)
    dz0 = tables.init_zstep_kerr(T, T["field"])
    out, st = O.run(T["field"], dz0)
    r = T["qdht_x"] * T["r_max"]
    k0 = T["wavenum0"].real
    zR = k0 * w0 * w0 / 2
    for fl, z in zip(out["f"], (0.0, 2e-3, 4e-3)):
        w2 = 2 * np.sum(fl * r ** 3) / np.sum(fl * r)   # second moment of the fluence (QDHT grid)
        wz = w0 * math.sqrt(1 + (z / zR) ** 2)
        assert abs(math.sqrt(w2) / wz - 1) < 2e-2


def test_aperture_zeroes_rows_once_in_config_order():
    """propagator.cu:232-261: after the step whose start z reaches an aperture's z, FIELD
    rows outside its radius are zero and BIGBUFFER2 = QDHT(FIELD); each aperture once, number
    0 first (process_input.cpp:176-179 reverses the order)."""
    import tempfile
    from gsolver_gb300 import configs
    d = tempfile.mkdtemp(prefix="gs_ap_")
    p = configs.fused_silica_c1(d)
    over = {"N_R": "32", "N_T": "256", "N_Z": "11", "APERTURE_N": "2", "APERTURE_Z0": "0", "APERTURE_R0": "1.5e-4",
            "APERTURE_Z1": "2.5e-4", "APERTURE_R1": "1e-4"}
    T = tables.build(tables.Config.from_file(p, overrides=over), noise_seed=1, noise_sigma=1e-4)
    assert list(T["aperture_z"]) == [2.5e-4, 0.0] and list(T["aperture_r"]) == [1e-4, 1.5e-4]
    O = oracle.Oracle(T, nonlinear=False)
    R = np.asarray(T["qdht_x"]) * T["r_max"]
    dz0 = tables.init_zstep_kerr(T, T["field"])
    out, st = O.run(T["field"], dz0, steps=1)              # the step from z = 0: aperture 0
    assert np.all(st["field"][R > 1.5e-4] == 0) and np.abs(st["field"][R <= 1.5e-4]).max() > 0
    assert np.array_equal(st["bb2"], O.qdht(st["field"]))
    out, st = O.run(T["field"], dz0, steps=2)               # z = 1e-4 < 2.5e-4: no second one yet
    assert np.abs(st["field"][R > 1.5e-4]).max() > 0
    out, st = O.run(T["field"], dz0, steps=4)               # the step from z = 3e-4: aperture 1
    assert np.all(st["field"][R > 1e-4] == 0)


def test_fft_is_the_dft_with_fftws_conventions():
    # the oracle's FFT (FFTW3's unnormalised transform, sign -1 forward / +1 backward, as the
    # reference calls it): radix-4 Stockham passes and a radix-2 pass for odd powers of two,
    # the plain DFT for other lengths; in place and out of place
    T = small(n_r=64, n_t=64)
    O = oracle.Oracle(T)
    rng = np.random.default_rng(3)
    for n in (1, 2, 4, 8, 32, 128, 2048, 16384, 32768, 12):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        for sign in (-1, 1):
            ref = np.fft.fft(x) if sign < 0 else np.fft.ifft(x) * n
            got = O.fft(x, sign)
            assert np.linalg.norm(got - ref) <= 1e-14 * max(1.0, np.linalg.norm(ref)), (n, sign)
    x = rng.standard_normal(1024) + 1j * rng.standard_normal(1024)
    assert np.allclose(O.fft(O.fft(x, -1), 1) / 1024, x, rtol=0, atol=1e-14)
