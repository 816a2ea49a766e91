"""Set-up restatement for the oracle (TEST INFRASTRUCTURE, FP64 numpy).

Builds every per-omega table, scalar, the Keldysh rate table, the QDHT matrix and the
Gaussian start field the reference computes before its z-loop, from a reference-format
``KEY value`` config.  Used only by tests/, smoke() and bench.py's CPU legs as the
checker for the product's own C++ set-up and as input to the C oracle.

Reference functions restated (file:line):
  load_named* config lookups          process_input.cpp:297-482
  load_info (incl. apertures)         process_input.cpp:98-182
  calculate_omega                     process_input.cpp:569-582
  calculate_wavenumber                process_input.cpp:585-623
  load_refrindex_raw                  process_input.cpp:677-721
  calculate_HOdispersion              process_input.cpp:806-871
  load_nonlindata                     process_input.cpp:211-250
  initialize_variables (plasma part)  solver_main.cpp:346-393
  calc_raman_function                 solver_main.cpp:401-413
  calc_ionization_rate/keldysh_rate   ionization.cpp:203-232, 313-355
  PPT_rate_ln (gas build)             ionization.cpp:235-294
  ellipke, dawson                     extmath.cpp:154-294 (restated by scipy.special)
  qdht_plan::qdht_plan                fhatha.cpp:177-198 (GSL Bessel restated by scipy)
  load_kerr_th_profiles               process_input.cpp:966-975
  create_gg                           pulse_gg.cpp:6-124
  init_zstep_kerr                     process_input.cpp:734-753
  create_net                          process_input.cpp:550-566
"""
from __future__ import annotations

import math
import os
import struct

import numpy as np
import scipy.special as sps

# SIconstants.h:4-38
LIGHT_VELOCITY = 299792458.0
VACUUM_PERMEABILITY = 1.2566370615e-6
ELECTRON_CHARGE = 1.60217733e-19
ELECTRON_MASS = 9.1093897e-31
PLANCK_CONSTANT_REDUCED = 1.0545727e-34

# solver.h:55-107
IONIZATION_I_LN_TOLERANCE = 0.003304003148325
IONIZATION_MIN_I_LN = 29.933606208922594
IONIZATION_N = 8192
INTENSITY_DENOM = 1e16
FIELD_DENOM = 1e8
IONRATE_DENOM = 1e20            # solid build (no IONIZATION_GAS)
IONRATE_DENOM_LN = 46.0517018
ABSORBTION_LAYER_WIDTH = 0.1
ABSORBTION_LAYER_BETA = 10.0
MAX_TOLERANCE_DEFAULT = 1e-4


class Config:
    """Token-pair config reader with command-line overrides (process_input.cpp:297-482).

    The reference reads the file as consecutive whitespace-separated token pairs and
    returns the first pair whose key matches; ``overrides`` plays the role of the
    ``argv[2:]`` ``KEY value`` pairs, which are consulted first.
    """

    def __init__(self, text: str, overrides: dict | None = None, base_dir: str = "."):
        toks = text.split()
        self.pairs = list(zip(toks[0::2], toks[1::2]))
        self.over = {k: str(v) for k, v in (overrides or {}).items()}
        self.base_dir = base_dir

    @classmethod
    def from_file(cls, path, overrides=None):
        with open(path) as f:
            return cls(f.read(), overrides, os.path.dirname(os.path.abspath(path)))

    def raw(self, name):
        if name in self.over:
            return self.over[name]
        for k, v in self.pairs:
            if k == name:
                return v
        return None

    def float(self, name, default=None):
        v = self.raw(name)
        if v is None:
            if default is None:
                raise KeyError(f"load_namedparameter: parameter {name} not found")
            return float(default)
        return _atof(v)

    def int(self, name, default=None):
        v = self.raw(name)
        if v is None:
            if default is None:
                raise KeyError(f"load_namedint: parameter {name} not found")
            return int(default)
        return int(_atof(v))

    def num(self, name, i, default=None):
        """load_namednumfloat (process_input.cpp:321-343): NAMEi, then NAME."""
        v = self.raw(f"{name}{i}")
        if v is None:
            v = self.raw(name)
        if v is None:
            if default is None:
                raise KeyError(f"load_namednumfloat: parameter {name}{i} not found")
            return float(default)
        return _atof(v)

    def str(self, name, default=None):
        v = self.raw(name)
        if v is None:
            if default is None:
                raise KeyError(f"parameter {name} not found")
            return default
        return v


def _atof(s: str) -> float:
    s = s.strip()
    for end in range(len(s), 0, -1):
        try:
            return float(s[:end])
        except ValueError:
            continue
    return 0.0


def read_rawdisp(path):
    """Type-3 RAW dispersion file: int type, int N, double omega[N], double n[2N]."""
    with open(path, "rb") as f:
        b = f.read()
    typ, n = struct.unpack("ii", b[:8])
    if typ != 3:
        raise ValueError("only RAW (type 3) dispersion files are supported")
    pw = np.frombuffer(b, dtype=np.float64, count=n, offset=8).copy()
    pn = np.frombuffer(b, dtype=np.float64, count=2 * n, offset=8 + 8 * n).copy()
    return pw, pn


def refrindex_raw(pw, pn, cfreq, P=1.0):
    """load_refrindex_raw interpolation; returns (n complex, omega_max, omega_min)."""
    cfreq = np.asarray(cfreq, dtype=np.float64)
    out = np.ones(cfreq.shape, dtype=np.complex128)
    npts = len(pw)
    for i, w in enumerate(cfreq):
        for j in _bracket_candidates(pw, w):
            if (pw[j - 1] - w) * (pw[j] - w) <= 0:
                ren_ = P * (pn[2 * j - 2] - 1) + 1
                imn_ = P * pn[2 * j - 1]
                ren = P * (pn[2 * j] - 1) + 1
                imn = P * pn[2 * j + 1]
                renc = ren_ + (ren - ren_) * (abs(w) - pw[j - 1]) / (pw[j] - pw[j - 1])
                imnc = imn_ + (imn - imn_) * (abs(w) - pw[j - 1]) / (pw[j] - pw[j - 1])
                out[i] = complex(renc, imnc)
                break
        else:
            out[i] = 1.0
    del npts
    return out, float(np.max(pw)), float(np.min(pw))


def _bracket_candidates(pw, w):
    """Indices j (ascending) that can satisfy the bracket test first; the table is
    ascending so the first bracketing interval is at searchsorted(left) (or 1)."""
    j = int(np.searchsorted(pw, w, side="left"))
    if j <= 0:
        j = 1
    if j >= len(pw):
        return []
    return [j]


def calculate_omega(nt, tmin, tmax, omega0):
    wstep = 2 * math.pi / (tmax - tmin)
    om = np.empty(nt)
    for i in range(nt // 2):
        om[i] = omega0 + wstep * i
    for i in range(nt // 2, nt):
        om[i] = omega0 - wstep * (nt - i)
    return om


def calculate_wavenumber(refr, omega):
    omega = np.asarray(omega, dtype=np.float64)
    wmax = float(np.max(omega))
    k = np.conj(refr) * omega / LIGHT_VELOCITY
    d = (omega / wmax - 1 - ABSORBTION_LAYER_WIDTH) / ABSORBTION_LAYER_WIDTH
    m = d > 0
    k = k.copy()
    k.imag[m] = k.imag[m] + (-k.real[m]) * (math.exp(ABSORBTION_LAYER_BETA) * d[m] * d[m])
    return k


def hfgaussfilter(w, omega_max):
    d = (w / omega_max - 1) / ABSORBTION_LAYER_WIDTH
    return np.where(d < 0, 1.0, np.exp(-ABSORBTION_LAYER_BETA * d * d))


def lfgaussfilter(w, omega_min):
    d = w * (1 - ABSORBTION_LAYER_WIDTH) / omega_min - 1
    return np.where(d > 0, 1.0, np.exp(-ABSORBTION_LAYER_BETA * d * d))


def create_net(xmin, xmax, n, nettype):
    if nettype.startswith("e") or not nettype:
        step = (xmax - xmin) / (n - 1)
        return np.array([xmin + i * step for i in range(n)])
    raise ValueError("only equidistant z nets are restated")


def bessel_j0_zeros(n):
    """First n positive zeros of J0, refined by Newton on scipy's j0/j1."""
    z = sps.jn_zeros(0, n).astype(np.float64)
    for _ in range(3):
        z = z + sps.j0(z) / sps.j1(z)
    return z


def qdht_matrix(n):
    """qdht_plan ctor: S=j_{0,N+1}; x_i = j_{0,i}; m1_i=|J1(x_i)|;
    C_ij = 2/S J0(x_i x_j/S)/|J1(x_i)|/|J1(x_j)|; x/=S; V=S/2pi."""
    zz = bessel_j0_zeros(n + 1)
    S = zz[n]
    x = zz[:n]
    m1 = np.abs(sps.j1(x))
    C = (2.0 / S) * sps.j0(np.outer(x, x) / S) / m1[:, None] / m1[None, :]
    return {"x": x / S, "m1": m1, "C": C, "V": S / 2.0 / math.pi, "S": S}


def ellipke(z):
    return float(sps.ellipk(z)), float(sps.ellipe(z))


def keldysh_rate_ln(lnI, k0, U, omega0, vg, reduced_mass):
    phase_v = omega0 / k0
    E = math.exp(lnI / 2) * math.sqrt(2 * phase_v / vg * phase_v * VACUUM_PERMEABILITY)
    m = ELECTRON_MASS * reduced_mass
    kgamma = omega0 * math.sqrt(m / ELECTRON_CHARGE / ELECTRON_CHARGE * U) / E
    Gamma = kgamma * kgamma / (1 + kgamma * kgamma)
    Xi = 1 / (1 + kgamma * kgamma)
    Kg, Eg = ellipke(Gamma)
    Kx, Ex = ellipke(Xi)
    alpha = math.pi * (Kg - Eg) / Ex
    beta = math.pi * math.pi / 4.0 / Kx / Ex
    x = 2 / math.pi * U / PLANCK_CONSTANT_REDUCED / omega0 * Ex / math.sqrt(Gamma)
    nu = math.floor(x + 1) - x
    sumN = min(int(math.ceil(10 / alpha)), 1000)
    i = np.arange(sumN, dtype=np.float64)
    Q = float(np.sum(np.exp(-i * alpha) * sps.dawsn(np.sqrt(beta * (i + 2 * nu)))))
    Q = Q * math.sqrt(math.pi / 2 / Kx)
    return (math.log(2 * omega0 / 9 / math.pi) + 1.5 * math.log(omega0 * m / PLANCK_CONSTANT_REDUCED)
            - 0.75 * math.log(Gamma) + math.log(Q) - alpha * math.floor(x + 1))


def keldysh_table(k0, U, omega0, vg, reduced_mass):
    t = np.zeros(IONIZATION_N)
    for i in range(IONIZATION_N - 1):
        lnI = IONIZATION_MIN_I_LN + IONIZATION_I_LN_TOLERANCE * i
        t[i] = keldysh_rate_ln(lnI, k0, U, omega0, vg, reduced_mass) - IONRATE_DENOM_LN
    return t   # top entry left at 0 (ionization.cpp:324)


# the gas build (IONIZATION_GAS, solver.h:32-33, 86-92)
IONRATE_DENOM_GAS = 1e10
IONRATE_DENOM_GAS_LN = 23.025850929940457
HARTREE_ENERGY = 4.359748124303985e-018   # SIconstants.h:35


def ppt_rate_ln(lnI, Ui, Z, l, k0, omega0, vg):
    """PPT_rate_ln (ionization.cpp:235-294) without the Yudin-Ivanov correction; n_eff is
    held in single precision as in the reference (`float neff`)."""
    phase_v = omega0 / k0
    E = math.exp(lnI / 2) * math.sqrt(2 * VACUUM_PERMEABILITY * phase_v * phase_v / vg)
    m = ELECTRON_MASS
    g = omega0 * math.sqrt(2 * m / ELECTRON_CHARGE / ELECTRON_CHARGE * Ui) / E
    Ueff = Ui * (1 + 1.0 / 2.0 / g / g)
    nu = Ueff / PLANCK_CONSTANT_REDUCED / omega0
    nu0 = int(math.floor(1 + nu))
    alpha = 2 * (math.asinh(g) - g / math.sqrt(1 + g * g))
    beta = 2 * g / math.sqrt(1 + g * g)
    E0 = math.sqrt(2 * Ui / ELECTRON_CHARGE * Ui / ELECTRON_CHARGE * Ui / PLANCK_CONSTANT_REDUCED * m
                   / PLANCK_CONSTANT_REDUCED)
    neff = float(np.float32(Z / math.sqrt(2 * Ui / HARTREE_ENERGY)))
    if g > 0.1:
        sumN = int(math.ceil(10 / alpha))
        k = np.arange(sumN, dtype=np.float64)
        x = k + nu0 - nu
        Q = float(np.sum(np.exp(-alpha * x) * sps.dawsn(np.sqrt(beta * x))))
    else:
        Q = math.sqrt(3 * math.pi) / 4 / g / g
    Cnl2 = 2.0 ** (2.0 * neff) / (neff * math.gamma(2 * neff))
    lnW = math.log(4 * math.sqrt(2.0) / math.pi * Cnl2) + math.log(2 * E0 / E / math.sqrt(1 + g * g)) * (2 * neff - 1.5)
    lnW += -2 * nu * (math.asinh(g) - g * math.sqrt(1 + g * g) / (1 + 2 * g * g))
    lnW += math.log((2 * l + 1) * Ui / PLANCK_CONSTANT_REDUCED * g * g / (1 + g * g) * Q)
    return lnW


def ppt_tables(potentials, ppt_z, ppt_l, k0, omega0, vg):
    """calc_ionization_rate, MULTI_LEVEL_IONIZATION + PPT (ionization.cpp:313-331,
    ionization.h:26-49): level 0 with PPT_Z, level n >= 1 with Z = n + 1; rows of 8192,
    the top entry of each left at 0."""
    L = len(potentials)
    t = np.zeros((L, IONIZATION_N))
    for n in range(L):
        Z = ppt_z if n == 0 else n + 1
        for i in range(IONIZATION_N - 1):
            lnI = IONIZATION_MIN_I_LN + IONIZATION_I_LN_TOLERANCE * i
            t[n, i] = ppt_rate_ln(lnI, potentials[n], Z, ppt_l, k0, omega0, vg) - IONRATE_DENOM_GAS_LN
    return t


def sqrt_ho_coeffs():
    k, b = [], 1.0
    for n in range(1, 21):
        b *= (0.5 - (n - 1)) / n
        k.append(b)
    return np.array(k)


def splitmix_normals(seed: int, count: int) -> np.ndarray:
    """Seeded standard normals shared with the product's C++ set-up:
    u_j = ((splitmix64(seed, j) >> 11) + 0.5) * 2^-53,
    n_k = sqrt(-2 ln u_{2k}) cos(2 pi u_{2k+1})."""
    M = np.uint64(0xFFFFFFFFFFFFFFFF)
    j = np.arange(2 * count, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) + (j + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)) & M
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & M
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & M
        z = z ^ (z >> np.uint64(31))
    u = ((z >> np.uint64(11)).astype(np.float64) + 0.5) * (2.0 ** -53)
    return np.sqrt(-2.0 * np.log(u[0::2])) * np.cos(2.0 * math.pi * u[1::2])


def build(cfg: Config, noise_seed: int | None = None, noise_sigma: float | None = None):
    """All set-up state for one pulse; returns a dict (arrays FP64 / complex128)."""
    T = {}
    lam = cfg.float("LAMBDA_V")
    omega0 = 2 * math.pi * LIGHT_VELOCITY / lam
    tmin = cfg.float("T_MIN", float("nan"))
    tmin = cfg.float("T_MIN_OMEGA", tmin * omega0) / omega0
    tmax = cfg.float("T_MAX", float("nan"))
    tmax = cfg.float("T_MAX_OMEGA", tmax * omega0) / omega0
    nt = cfg.int("N_T")
    tstep = (tmax - tmin) / nt
    omega = calculate_omega(nt, tmin, tmax, omega0)

    P = cfg.float("PRESSURE", 1)
    dispfile = cfg.str("DISPERSION_FILE", "NO")
    if dispfile == "NO":
        raise ValueError("a RAW dispersion file is required")
    dpath = dispfile if os.path.isabs(dispfile) else os.path.join(cfg.base_dir, dispfile)
    pw, pn = read_rawdisp(dpath)
    refr, omax_f, omin_f = refrindex_raw(pw, pn, omega, P)
    wavenum = calculate_wavenumber(refr, omega)
    refr0, _, _ = refrindex_raw(pw, pn, np.array([omega0]), P)
    k0c = calculate_wavenumber(refr0, np.array([omega0]))[0]
    omega_max, omega_min = omax_f, omin_f

    # calculate_HOdispersion (OMEGA0 == OMEGA[0] branch)
    n0 = refr[0].real
    dndw = (refr[1] - refr[nt - 1]).real / (omega[1] - omega[nt - 1])
    ngr = n0 + omega0 * dndw
    ho = (omega / LIGHT_VELOCITY) * (refr.real - ngr)
    vg = LIGHT_VELOCITY / ngr
    ho = ho * (lfgaussfilter(omega, omega_min) * hfgaussfilter(omega, omega_max))
    omega_max = min(omega_max, (1 - ABSORBTION_LAYER_WIDTH) * omega[nt // 2 - 1])

    tol = cfg.float("MAX_TOLERANCE", MAX_TOLERANCE_DEFAULT)
    nr = cfg.int("N_R")
    rmax = cfg.float("R_MAX")
    nz = cfg.int("N_Z")
    zmin = cfg.float("Z_MIN", 0)
    zmax = cfg.float("Z_MAX", 0)
    znettype = cfg.str("ZNET_TYPE")
    znet = create_net(zmin, zmax, nz, znettype)
    ambient = cfg.float("AMBIENT_CARRIERS", 0) * cfg.float("NEUTRAL_DENSITY", 0)
    # apertures (process_input.cpp:176-179): entry i holds APERTURE_Z/R number N-1-i, so the
    # last entry (number 0) is the first one applied
    n_ap = int(cfg.float("APERTURE_N", 0))
    ap_z = np.array([cfg.num("APERTURE_Z", n_ap - i - 1) for i in range(n_ap)])
    ap_r = np.array([cfg.num("APERTURE_R", n_ap - i - 1) for i in range(n_ap)])

    # load_nonlindata
    n2 = cfg.float("NONLIN_REFRINDEX", 0) * P
    fR = cfg.float("RAMAN_FRACTION")
    tauR = cfg.float("TAU_RAMAN")
    omR = cfg.float("OMEGA_RAMAN")
    rho_n = cfg.float("NEUTRAL_DENSITY") * P
    tau_rec = cfg.float("RECOMBINATION_TAU")
    tau_c = cfg.float("COLLISION_TAU") / P
    Ui = cfg.float("IONIZATION_POTENTIAL") * ELECTRON_CHARGE

    # qdht plan
    Q = qdht_matrix(nr)

    # initialize_variables: plasma constants
    red_mass = cfg.float("REDUCED_MASS", 1)
    m = ELECTRON_MASS * red_mass
    k0r = k0c.real
    IBS = ELECTRON_CHARGE / m * ELECTRON_CHARGE * VACUUM_PERMEABILITY / k0r
    aval = IBS * omega0 * tau_c / (1 + omega0 * tau_c * omega0 * tau_c)
    pond = IBS / 2.0 / k0r / vg / (1.0 + 1.0 / (omega0 * tau_c))
    alpha = tau_c * omega
    kw = wavenum.real
    pf = -(alpha / (1.0 + 1j * alpha) / 2.0 / kw * ELECTRON_CHARGE * ELECTRON_CHARGE / m * VACUUM_PERMEABILITY)

    build_kind = cfg.str("GSOLVER_BUILD", "solid_qdht")
    gas = build_kind == "gas_qdht"
    if build_kind not in ("solid_qdht", "gas_qdht"):
        raise ValueError(f"GSOLVER_BUILD {build_kind}: solid_qdht or gas_qdht")
    ion_denom = IONRATE_DENOM_GAS if gas else IONRATE_DENOM
    if gas:
        if cfg.float("NONLIN_REFRINDEX4", 0) != 0:
            raise ValueError("NONLIN_REFRINDEX4 != 0 is not supported")
        if cfg.str("TH_PROFILE", "NO") != "NO" or cfg.str("KERR_PROFILE", "NO") != "NO":
            raise ValueError("KERR_PROFILE / TH_PROFILE files are not supported")
        levels = int(cfg.float("IONIZATION_LEVEL_N", 1))
        pots = [cfg.num("IONIZATION_POTENTIAL", i + 1) * ELECTRON_CHARGE for i in range(levels)]
        Ui = pots[0]
        rate = ppt_tables(pots, cfg.float("PPT_Z", 1), cfg.int("PPT_L", 0), k0r, omega0, vg)
        th_coeff = (1 - fR) / 3.0 * cfg.float("TH_FACTOR", 1)
    else:
        levels, pots, th_coeff = 1, [Ui], 0.0
        rate = keldysh_table(k0r, Ui, omega0, vg, red_mass)

    # calc_raman_function
    M = tstep * (1 + omR * omR * tauR * tauR) / tauR / (omR * tauR)
    t = tstep * np.arange(nt)
    h = fR * M * np.exp(-t / tauR) * np.sin(omR * t)
    raman = np.fft.fft(h.astype(np.complex128)) + (1 - fR)

    # scalings (solver_main.cpp:385-393)
    Ui_s = Ui * (ion_denom / INTENSITY_DENOM)
    pots_s = np.array(pots) * (ion_denom / INTENSITY_DENOM)
    n2_s = n2 * INTENSITY_DENOM
    tau_rec_s = tau_rec * ion_denom
    pond_s = pond * ion_denom

    kerr = n2_s * omega / LIGHT_VELOCITY / kw * omega / LIGHT_VELOCITY

    kt = 2 * math.pi * Q["x"] * Q["V"] / rmax
    kt2 = kt * kt

    T.update(dict(
        n_r=nr, n_t=nt, omega0=omega0, tmin=tmin, tmax=tmax, tstep=tstep, omega=omega,
        wavenum=wavenum, wavenum0=k0c, ho_disp=ho, group_velocity=vg, omega_min=omega_min,
        omega_max=omega_max, max_tolerance=tol, r_max=rmax, znet=znet, n_z=nz,
        ambient=ambient, n2=n2_s, raman_fraction=fR, neutral_density=rho_n,
        recombination_tau=tau_rec_s, ionization_potential=Ui_s, ponderomotive=pond_s,
        avalanche_cs=aval, plasma_func=pf, rate_ln=rate, raman_func=raman, kerr=kerr,
        qdht_c=Q["C"], qdht_m1=Q["m1"], qdht_x=Q["x"], qdht_V=Q["V"], kt2=kt2,
        ionrate_denom=ion_denom, raman_tau=tauR, raman_omega=omR,
        gas=1 if gas else 0, ion_levels=levels, ion_potentials=pots_s, th_coeff=th_coeff,
        aperture_z=ap_z, aperture_r=ap_r,
    ))
    T["field"] = create_gg(cfg, T, noise_seed, noise_sigma)
    return T


def create_gg(cfg: Config, T, noise_seed=None, noise_sigma=None):
    """create_gg (pulse_gg.cpp:6-124) followed by FIELD /= FIELD_DENOM.

    The reference's uniform ``NOISE_LEVEL`` draws from an unseeded drand48; here the
    start field is noiseless unless ``noise_sigma`` is given, in which case complex
    Gaussian noise sigma*(n1 + j n2) from ``splitmix_normals(noise_seed)`` multiplies
    the envelope exactly where the reference puts its uniform noise term."""
    omega0 = T["omega0"]
    nt, nr = T["n_t"], T["n_r"]
    tau_fwhm = cfg.float("DURATION_FWHM", -1)
    tau_fwhm = cfg.float("DURATION_FWHM_OMEGA", tau_fwhm * omega0) / omega0
    d_fwhm = cfg.float("DIAMETER_FWHM")
    ce_phase = cfg.float("CE_PHASE", 0)
    sg_T = cfg.float("PULSE_SG_ORDER", 1)
    sg_r = cfg.float("BEAM_SG_ORDER", 1)
    k0 = T["wavenum0"].real
    E = cfg.float("ENERGY", -1)
    E_P_factor = 2 * math.pow(math.log(2), 1.0 / 2.0 / sg_T) / math.gamma(1.0 / 2.0 / sg_T)
    Pcr = 2 * math.pi * LIGHT_VELOCITY / k0 / omega0 / T["n2"] * INTENSITY_DENOM
    P0 = cfg.float("POWER_CR", E / tau_fwhm * E_P_factor / Pcr) * Pcr
    P0 = cfg.float("POWER", P0)
    A0 = math.sqrt(P0 / d_fwhm / d_fwhm * 4 * math.pow(math.log(2), 1.0 / sg_r) / math.pi / math.gamma(1.0 / sg_r))
    tau = tau_fwhm / 2.0 / math.pow(math.log(math.sqrt(2.0)), 1.0 / 2.0 / sg_T)
    ro = d_fwhm / 2.0 / math.pow(math.log(math.sqrt(2.0)), 1.0 / 2.0 / sg_r)
    zR = k0 * ro * ro / 2
    C = cfg.float("CHIRP_SI", 0)
    C = cfg.float("CHIRP", C * tau * tau)
    Cw = cfg.float("CHIRP_SPECTRAL", 0)
    f = np.float64(cfg.float("FOCUSING_DISTANCE", 0))
    zR64 = np.float64(zR)
    with np.errstate(all="ignore"):
        f = np.float64(cfg.float("FOCUSING_DISTANCE_DIFFRACTION", f / zR64))
        if zR64 > 2 * f:
            f = zR64 * zR64 / 2 / f * (1 - np.sqrt(1 - 4 * f * f / zR64 / zR64))
    f = cfg.float("WAVEFRONT_RADIUS", float(f))
    f = cfg.float("WAVEFRONT_RADIUS_DIFFRACTION", f / zR) * zR

    R = T["qdht_x"] * T["r_max"]
    tgrid = T["tmin"] + T["tstep"] * np.arange(nt)
    Tn = tgrid / tau
    cph = ce_phase - Tn * Tn * C
    env_t = np.exp(-(np.power(Tn, 2.0 * sg_T)))
    amax = A0 * np.exp(-np.power(R / ro, 2.0 * sg_r))
    car = np.exp(1j * cph)
    field = np.empty((nr, nt), dtype=np.complex128)
    if noise_sigma:
        nz = splitmix_normals(int(noise_seed or 0), 2 * nr * nt).reshape(nr, nt, 2)
    for r in range(nr):
        row_c = car
        if noise_sigma:
            row_c = car + noise_sigma * (nz[r, :, 0] + 1j * nz[r, :, 1])
        row = (amax[r] * env_t) * row_c
        spec = np.fft.fft(row)
        kk = T["wavenum"].real
        phase = (R[r] * R[r] * kk / 2.0 / f) - Cw * (T["omega"] - omega0) * (T["omega"] - omega0) / 2
        field[r] = spec * np.exp(1j * phase)
    field /= FIELD_DENOM
    return field


def init_zstep_kerr(T, field):
    """Initial dz (process_input.cpp:734-753)."""
    e = np.fft.ifft(field, axis=1)
    maxI = float(np.max(e.real ** 2 + e.imag ** 2))
    dz = T["znet"][1] - T["znet"][0]
    kNL = T["omega0"] / LIGHT_VELOCITY * T["n2"] * maxI
    if dz * kNL > T["max_tolerance"]:
        dz = T["max_tolerance"] / kNL
    return dz
