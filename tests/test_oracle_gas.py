"""The gas build (gsolver_gas_qdht: PPT rates, single-level ionization with neutral
depletion, third harmonic) in the oracle and in the product's C++ set-up (CPU)."""
import tempfile

import numpy as np

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables


def _argon(power_cr=6.0, w0=9e-4, n_r=16, n_t=4096):
    d = tempfile.mkdtemp(prefix="gs_gas_")
    p = configs.argon_c5(d, n_r=n_r, n_t=n_t, build="gas_qdht", power_cr=power_cr, w0=w0, r_max=4 * w0)
    return p, tables.build(tables.Config.from_file(p), noise_seed=1, noise_sigma=1e-4)


def test_gas_density_closed_form_at_constant_intensity():
    """ionization.cpp:45-60 with one level and a constant intensity I above threshold:
    rho_t = rho_n (1 - q^(t-1)), q = 1 - dt W + (dt W)^2 / 2 (the first step starts from
    E_0 = 0 and does nothing); loss_t = -W (rho_n - rho_t)(U + P I)/(2 I) E_t."""
    p, T = _argon()
    O = oracle.Oracle(T)
    N = T["n_t"]
    I = 1e14 * 1e4 / 1e16          # 1e14 W/cm^2 in the scaled units
    e = np.full(N, np.sqrt(I), dtype=np.complex128)
    pro, loss = O.plasma(e)
    lnI = np.log(I) + 36.841361487904734
    n = int(np.floor((lnI - 29.933606208922594) / 0.003304003148325))
    lnIn = 29.933606208922594 + n * 0.003304003148325
    r = T["rate_ln"][0]
    W = np.exp(r[n] + (lnI - lnIn) * (r[n + 1] - r[n]) / 0.003304003148325)
    dt = T["tstep"] * T["ionrate_denom"]
    q = 1 - dt * W + 0.5 * (dt * W) ** 2
    ND = T["neutral_density"]
    t = np.arange(N)
    ref = np.where(t >= 1, ND * (1 - q ** np.maximum(t - 1, 0)), 0.0)
    assert pro.max() > 1e-6 * ND
    assert np.allclose(pro, ref, rtol=1e-12, atol=1e-12 * ND)
    U, P = T["ionization_potential"], T["ponderomotive"]
    lref = -0.5 * W * (ND - pro) * (U + P * I) / I * e
    lref[0] = 0
    lref[-1] = 0
    assert np.allclose(loss, lref, rtol=1e-12, atol=1e-12 * np.abs(lref).max())


def test_product_setup_matches_oracle_gas_build():
    p, T = _argon()
    S = gs.Setup(p, noise_seed=1, noise_sigma=1e-4).as_dict()
    assert S["gas"] == 1 and T["gas"] == 1
    assert abs(S["th_coeff"] - T["th_coeff"]) < 1e-15
    rel = lambda a, b: float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))
    # PPT tables: the product's dawson series vs scipy's dawsn
    assert rel(S["rate_ln"], T["rate_ln"][0]) < 1e-10
    for k in ("plasma_func", "kerr", "wavenum", "ho_disp", "field"):
        assert rel(S[k], T[k]) < 1e-13, k
    for k in ("ionization_potential", "ponderomotive", "ionrate_denom", "neutral_density"):
        assert abs(S[k] - T[k]) <= 1e-15 * abs(T[k]), k
    assert T["ionrate_denom"] == 1e10


def test_product_setup_matches_oracle_with_three_levels():
    """IONIZATION_LEVEL_N 3: the product's set-up builds one PPT row per level (level 0 with
    PPT_Z, level n with Z = n + 1) and the levels' potentials as the oracle does."""
    p, _ = _argon()
    with open(p, "a") as fh:
        fh.write("IONIZATION_LEVEL_N 3\nIONIZATION_POTENTIAL1 15.76\nIONIZATION_POTENTIAL2 27.63\n"
                 "IONIZATION_POTENTIAL3 40.74\n")
    T = tables.build(tables.Config.from_file(p), noise_seed=1, noise_sigma=1e-4)
    S = gs.Setup(p, noise_seed=1, noise_sigma=1e-4).as_dict()
    assert S["ion_levels"] == T["ion_levels"] == 3
    rel = lambda a, b: float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))
    assert np.asarray(S["rate_ln"]).shape == (3, 8192)
    for n in range(3):
        assert rel(S["rate_ln"][n], T["rate_ln"][n]) < 1e-10, n
    assert rel(S["ion_potentials"], T["ion_potentials"]) < 1e-15


def test_third_harmonic_generates_the_third_harmonic():
    """A Kerr-only gas pulse: with the third-harmonic term the NL response has power near
    3 omega0 (inside the grid), without it none beyond the rounding floor."""
    p, T = _argon(power_cr=1.0, n_t=8192)
    om = np.asarray(T["omega"])
    near3 = np.abs(om - 3 * T["omega0"]) < 0.05 * T["omega0"]
    assert near3.any()
    O = oracle.Oracle(T)
    n_th = O.nl_response(T["field"][0])
    T2 = dict(T)
    T2["th_coeff"] = 0.0
    n_no = oracle.Oracle(T2).nl_response(T["field"][0])
    assert np.abs(n_th[near3]).max() > 1e3 * np.abs(n_no[near3]).max()
