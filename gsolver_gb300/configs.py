"""Reference-format configs and dispersion tables for the benchmark workloads.

The reference reads whitespace ``KEY value`` configs (process_input.cpp:297-482) and RAW
dispersion files (type 3: int type, int N, double omega[N], double n[2N];
process_input.cpp:677-721).  Its HO dispersion only accepts RAW files
(process_input.cpp:864), so Sellmeier media are tabulated here onto an omega grid that
covers the whole spectral window.

Workloads (synthetic: no dataset, the pulse is generated):
  fused_silica_c1   N_R=256,  N_T=2048,  R=600 um, 400 fs window, 1 mm in 500 fixed steps
  fused_silica_c2   N_R=1024, N_T=16384, R=1.2 mm, 1.6 ps window, 3 mm, adaptive (tol 1e-6)
  fused_silica_c4   N_R=256,  N_T=4096,  R=600 um, 800 fs window, 2 mm in 1000 fixed steps;
                    the adjoint workload: a seeded degree-6 spectral phase on the input
                    (spectral_phase) and the output energy in the 500-600 nm band
                    (band_weights) as the objective
  fused_silica_c3   64 pulses (c3_batch): N_R in {128, 256, 512}, N_T in {1024 .. 8192},
                    P ~ U[1, 8] P_cr, CEP ~ U[0, 2 pi), 30-100 fs, w0 50-150 um drawn from a
                    seed; window 400 fs * N_T / 2048 and R = 6 w0 (unstated by the workload);
                    1 mm in 500 fixed 2 um steps
  argon_c5          N_R=512, N_T=32768, 3.9 um 80 fs w0 = 1 mm 4 P_cr pulse in 1 atm argon,
                    2 ps window, R = 4 mm (R unstated by the workload; 4 w0 chosen), z = 20 cm,
                    solid-path Keldysh rate with Ip = 15.76 eV (the gas PPT build is not on
                    this path)
  hot_solid         small high-intensity grids where Keldysh, avalanche, loss and plasma
                    defocusing all act (peak ~5e13 W/cm^2)
"""
from __future__ import annotations

import math
import os

import numpy as np

LIGHT_VELOCITY = 299792458.0

# Malitson fused silica: n^2 - 1 = sum B_i lam^2 / (lam^2 - C_i^2), lam in um
MALITSON_B = (0.6961663, 0.4079426, 0.8974794)
MALITSON_C = (0.0684043, 0.1162414, 9.896161)


def sellmeier_n(lam_um, B=MALITSON_B, Cum=MALITSON_C):
    lam2 = np.asarray(lam_um, dtype=np.float64) ** 2
    n2 = 1.0 + sum(b * lam2 / (lam2 - c * c) for b, c in zip(B, Cum))
    return np.sqrt(n2)


def argon_n(lam_um, pressure=1.0):
    lam2 = np.asarray(lam_um, dtype=np.float64) ** 2
    return 1.0 + pressure * 5.547e-4 * (1 + 5.15e-3 / lam2 + 4.19e-5 / lam2 ** 2)


def write_rawdisp(path, omega, n):
    omega = np.ascontiguousarray(omega, dtype=np.float64)
    n = np.asarray(n)
    inter = np.empty(2 * len(omega))
    inter[0::2] = np.real(n)
    inter[1::2] = np.imag(n) if np.iscomplexobj(n) else 0.0
    with open(path, "wb") as f:
        f.write(np.array([3, len(omega)], dtype=np.int32).tobytes())
        f.write(omega.tobytes())
        f.write(inter.tobytes())


def tabulate_medium(path, medium="fused_silica", lam_min_um=0.2, lam_max_um=5.0, npts=20001):
    """RAW table uniform in omega between 2 pi c / lam_max and 2 pi c / lam_min."""
    wmin = 2 * math.pi * LIGHT_VELOCITY / (lam_max_um * 1e-6)
    wmax = 2 * math.pi * LIGHT_VELOCITY / (lam_min_um * 1e-6)
    omega = np.linspace(wmin, wmax, npts)
    lam_um = 2 * math.pi * LIGHT_VELOCITY / omega * 1e6
    n = sellmeier_n(lam_um) if medium == "fused_silica" else argon_n(lam_um)
    write_rawdisp(path, omega, n)
    return path


def _fmt(d):
    return "\n".join(f"{k} {v}" for k, v in d.items()) + "\n"


SILICA_NL = {
    "NONLIN_REFRINDEX": "2.5e-20", "RAMAN_FRACTION": "0.18", "TAU_RAMAN": "32e-15",
    "OMEGA_RAMAN": repr(1 / 12.2e-15), "IONIZATION_POTENTIAL": "9", "NEUTRAL_DENSITY": "2.1e28",
    "COLLISION_TAU": "1.7e-15", "RECOMBINATION_TAU": "150e-15", "AMBIENT_CARRIERS": "0",
}


def fused_silica_c1(dirpath):
    """256 x 2048, collimated 800 nm 50 fs w0 = 100 um 3 P_cr pulse, 1 mm in 500 steps."""
    tabulate_medium(os.path.join(dirpath, "fused_silica.rawdisp"))
    d = {"LAMBDA_V": "8e-7", "N_T": "2048", "T_MIN": "-200e-15", "T_MAX": "200e-15",
         "DISPERSION_FILE": "fused_silica.rawdisp", "N_R": "256", "R_MAX": "6e-4",
         "N_Z": "501", "Z_MIN": "0", "Z_MAX": "1e-3", "ZNET_TYPE": "e", "MAX_TOLERANCE": "1e3",
         "PULSE_SHAPE": "gg", "DURATION_FWHM": "50e-15", "DIAMETER_FWHM": repr(100e-6 * math.sqrt(2 * math.log(2))),
         "POWER_CR": "3", "WAVEFRONT_RADIUS": "1e100", "CE_PHASE": "0"}
    d.update(SILICA_NL)
    p = os.path.join(dirpath, "fused_silica_c1.txt")
    with open(p, "w") as f:
        f.write(_fmt(d))
    return p


def fused_silica_c2_rows(dirpath, n_r):
    """The 1024 x 16384 workload's pulse, window and physics on n_r radial points with R
    scaled by n_r / 1024 (same radial spacing): a smaller case of the same kernels for
    profiling captures."""
    p = fused_silica_c2(dirpath)
    with open(p) as f:
        txt = f.read()
    txt = txt.replace("N_R 1024", f"N_R {n_r}").replace("R_MAX 1.2e-3", f"R_MAX {1.2e-3 * n_r / 1024!r}")
    q = os.path.join(dirpath, f"fused_silica_c2_{n_r}.txt")
    with open(q, "w") as f:
        f.write(txt)
    return q


def fused_silica_c2(dirpath):
    """1024 x 16384, same pulse, R = 1.2 mm, 1.6 ps window, 3 mm, adaptive dz (tol 1e-6)."""
    tabulate_medium(os.path.join(dirpath, "fused_silica.rawdisp"))
    d = {"LAMBDA_V": "8e-7", "N_T": "16384", "T_MIN": "-0.8e-12", "T_MAX": "0.8e-12",
         "DISPERSION_FILE": "fused_silica.rawdisp", "N_R": "1024", "R_MAX": "1.2e-3",
         "N_Z": "31", "Z_MIN": "0", "Z_MAX": "3e-3", "ZNET_TYPE": "e", "MAX_TOLERANCE": "1e-6",
         "PULSE_SHAPE": "gg", "DURATION_FWHM": "50e-15", "DIAMETER_FWHM": repr(100e-6 * math.sqrt(2 * math.log(2))),
         "POWER_CR": "3", "WAVEFRONT_RADIUS": "1e100", "CE_PHASE": "0"}
    d.update(SILICA_NL)
    p = os.path.join(dirpath, "fused_silica_c2.txt")
    with open(p, "w") as f:
        f.write(_fmt(d))
    return p


def fused_silica_c4(dirpath):
    """256 x 4096, the C1 pulse (800 nm, 50 fs, w0 = 100 um, 3 P_cr) over 2 mm in 1000 fixed
    2 um steps (the C1 step size; MAX_TOLERANCE large so the ZNET clamp sets dz).  The window
    (800 fs) and R (600 um) are not stated by the workload: C1's time step and radius."""
    tabulate_medium(os.path.join(dirpath, "fused_silica.rawdisp"))
    d = {"LAMBDA_V": "8e-7", "N_T": "4096", "T_MIN": "-400e-15", "T_MAX": "400e-15",
         "DISPERSION_FILE": "fused_silica.rawdisp", "N_R": "256", "R_MAX": "6e-4",
         "N_Z": "1001", "Z_MIN": "0", "Z_MAX": "2e-3", "ZNET_TYPE": "e", "MAX_TOLERANCE": "1e3",
         "PULSE_SHAPE": "gg", "DURATION_FWHM": "50e-15", "DIAMETER_FWHM": repr(100e-6 * math.sqrt(2 * math.log(2))),
         "POWER_CR": "3", "WAVEFRONT_RADIUS": "1e100", "CE_PHASE": "0"}
    d.update(SILICA_NL)
    p = os.path.join(dirpath, "fused_silica_c4.txt")
    with open(p, "w") as f:
        f.write(_fmt(d))
    return p


def c3_batch(dirpath, seed=0, n=64):
    """The batched-scan workload: n fused-silica pulses with uneven grids and parameters
    drawn from numpy PCG64(seed).  Returns [(config path, draw dict)]."""
    tabulate_medium(os.path.join(dirpath, "fused_silica.rawdisp"))
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nr = int(rng.choice([128, 256, 512]))
        nt = int(rng.choice([1024, 2048, 4096, 8192]))
        pcr = float(rng.uniform(1, 8))
        cep = float(rng.uniform(0, 2 * math.pi))
        tau = float(rng.uniform(30e-15, 100e-15))
        w0 = float(rng.uniform(50e-6, 150e-6))
        win = 400e-15 * nt / 2048
        d = {"LAMBDA_V": "8e-7", "N_T": str(nt), "T_MIN": repr(-win / 2), "T_MAX": repr(win / 2),
             "DISPERSION_FILE": "fused_silica.rawdisp", "N_R": str(nr), "R_MAX": repr(6 * w0),
             "N_Z": "501", "Z_MIN": "0", "Z_MAX": "1e-3", "ZNET_TYPE": "e", "MAX_TOLERANCE": "1e3",
             "PULSE_SHAPE": "gg", "DURATION_FWHM": repr(tau), "DIAMETER_FWHM": repr(w0 * math.sqrt(2 * math.log(2))),
             "POWER_CR": repr(pcr), "WAVEFRONT_RADIUS": "1e100", "CE_PHASE": repr(cep)}
        d.update(SILICA_NL)
        p = os.path.join(dirpath, f"fused_silica_c3_{i:02d}.txt")
        with open(p, "w") as f:
            f.write(_fmt(d))
        out.append((p, {"n_r": nr, "n_t": nt, "power_cr": pcr, "cep": cep, "duration_fwhm": tau, "w0": w0}))
    return out


def spectral_phase(omega, omega0, duration_fwhm, seed, degree=6):
    """phi(omega) = sum_{k=2..degree} c_k x^k, x = (omega - omega0)/d_omega, c_k ~ N(0,1) rad
    (numpy PCG64, the seed given); d_omega = 4 ln2 / duration_fwhm, the intensity FWHM
    bandwidth of the transform-limited pulse."""
    c = np.random.default_rng(seed).standard_normal(degree - 1)
    x = (np.asarray(omega) - omega0) * duration_fwhm / (4 * math.log(2))
    return sum(ck * x ** (k + 2) for k, ck in enumerate(c))


def band_weights(omega, qdht_x, r_max, lo_m, hi_m):
    """Objective weights [n_r][n_t]: the average_spectrum radial weights
    (dump_types.cpp:427-457: x_0 (x_1 - x_0), x_i (x_i - x_{i-1}), times R^2/2) on the
    spectral band lo_m..hi_m (wavelengths), zero outside it."""
    om = np.asarray(omega)
    band = (om >= 2 * math.pi * LIGHT_VELOCITY / hi_m) & (om <= 2 * math.pi * LIGHT_VELOCITY / lo_m)
    x = np.asarray(qdht_x)
    wr = np.empty_like(x)
    wr[0] = x[0] * (x[1] - x[0])
    wr[1:] = x[1:] * (x[1:] - x[:-1])
    return np.outer(wr * r_max * r_max / 2, band.astype(float))


def clamp_schedule(znet, dz0, steps):
    """(dz_rk, dz_lin) of `steps` propagator() calls when the controller's proposal always
    exceeds the distance to the next ZNET point (MAX_TOLERANCE large): the z-loop of
    solver_main.cpp:202-225 with the clamp of propagator.cu:164; RK4 stages use the previous
    ZSTEP, the linear step the clamped one."""
    cz, n_z, zstep = float(znet[0]), 0, float(dz0)
    rk, lin = [], []
    for _ in range(steps):
        if cz >= znet[n_z]:
            n_z += 1
        new = float(znet[n_z]) - cz
        rk.append(zstep)
        lin.append(new)
        zstep = new
        cz += new
    return np.array(rk), np.array(lin)


ARGON_NL = {
    "NONLIN_REFRINDEX": "1e-23", "RAMAN_FRACTION": "0", "TAU_RAMAN": "32e-15", "OMEGA_RAMAN": "1e13",
    "IONIZATION_POTENTIAL": "15.76", "NEUTRAL_DENSITY": "2.5e25", "COLLISION_TAU": "190e-15",
    "RECOMBINATION_TAU": "1e30", "AMBIENT_CARRIERS": "0",
}


def argon_c5(dirpath, n_r=512, n_t=32768, cep=0.0, name="argon_c5", build="solid_qdht", power_cr=4.0, w0=1e-3,
             r_max=4e-3, window=2e-12):
    """Argon filament at 3.9 um (Sellmeier n-1 = 5.547e-4 (1 + 5.15e-3/lam^2 + 4.19e-5/lam^4)).
    build "gas_qdht" selects the reference's gas binary (gsolver_gas_qdht: PPT multi-level
    ionization, third harmonic, IONRATE_DENOM 1e10) through the GSOLVER_BUILD key."""
    tabulate_medium(os.path.join(dirpath, "argon.rawdisp"), medium="argon", lam_min_um=0.15, lam_max_um=20.0)
    d = {"LAMBDA_V": "3.9e-6", "N_T": str(n_t), "T_MIN": repr(-window / 2), "T_MAX": repr(window / 2),
         "DISPERSION_FILE": "argon.rawdisp", "N_R": str(n_r), "R_MAX": repr(r_max),
         "N_Z": "201", "Z_MIN": "0", "Z_MAX": "0.2", "ZNET_TYPE": "e", "MAX_TOLERANCE": "1e-3",
         "PULSE_SHAPE": "gg", "DURATION_FWHM": "80e-15", "DIAMETER_FWHM": repr(w0 * math.sqrt(2 * math.log(2))),
         "POWER_CR": repr(power_cr), "WAVEFRONT_RADIUS": "1e100", "CE_PHASE": repr(cep)}
    d.update(ARGON_NL)
    if build != "solid_qdht":
        d["GSOLVER_BUILD"] = build
    p = os.path.join(dirpath, name + ".txt")
    with open(p, "w") as f:
        f.write(_fmt(d))
    return p


def hot_solid(dirpath, n_r=32, n_t=2048, power_cr=30.0, w0=10e-6, window=400e-15, r_max=None,
              tol=1e3, z_max=2e-5, n_z=11, name="hot_solid"):
    """Small fused-silica grid with a tightly focused, strongly ionizing pulse."""
    tabulate_medium(os.path.join(dirpath, "fused_silica.rawdisp"))
    r_max = r_max or 6 * w0
    d = {"LAMBDA_V": "8e-7", "N_T": str(n_t), "T_MIN": repr(-window / 2), "T_MAX": repr(window / 2),
         "DISPERSION_FILE": "fused_silica.rawdisp", "N_R": str(n_r), "R_MAX": repr(r_max),
         "N_Z": str(n_z), "Z_MIN": "0", "Z_MAX": repr(z_max), "ZNET_TYPE": "e", "MAX_TOLERANCE": repr(tol),
         "PULSE_SHAPE": "gg", "DURATION_FWHM": "50e-15", "DIAMETER_FWHM": repr(w0 * math.sqrt(2 * math.log(2))),
         "POWER_CR": repr(power_cr), "WAVEFRONT_RADIUS": "1e100", "CE_PHASE": "0"}
    d.update(SILICA_NL)
    p = os.path.join(dirpath, name + ".txt")
    with open(p, "w") as f:
        f.write(_fmt(d))
    return p
