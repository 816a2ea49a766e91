"""ctypes front end of the C oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this module, and only
as the checker / CPU baseline.  ``Oracle`` wraps one pulse's set-up (a dict from
``oracle.tables.build``) and exposes the reference's hot-path functions:
``nl_step`` (calculate_NLstep), ``lstep`` (calculate_Lstep), ``qdht`` (ht_run),
``propagator`` (propagator) and ``run`` (the z-loop of solver_main.cpp:202-225 with the
flux / field_axis / plasma_max / average_spectrum / maxI dumps of dump_types.cpp).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libgs_oracle.so")

ERRORS = {
    1: "Attention!!!! Intensity is too big! Keep away, blast is possible.",
    2: "float_type photoionization_function(...): Intensity is nan!",
    3: "Minimum Z step size reached, collapse is possible!",
    4: "bad argument",
}


class OracleError(RuntimeError):
    pass


class _Ctx(C.Structure):
    _fields_ = [
        ("n_r", C.c_int), ("n_t", C.c_int), ("nonlinear", C.c_int), ("nthreads", C.c_int),
        ("tstep", C.c_double), ("tmin", C.c_double), ("tmax", C.c_double), ("omega0", C.c_double),
        ("ionrate_denom", C.c_double), ("neutral_density", C.c_double), ("rho0", C.c_double),
        ("ionization_potential", C.c_double), ("ponderomotive", C.c_double),
        ("avalanche_cs", C.c_double), ("recombination_tau", C.c_double),
        ("raman_fraction", C.c_double), ("n2", C.c_double),
        ("rate_ln", C.c_void_p), ("plasma_func", C.c_void_p), ("raman_func", C.c_void_p),
        ("kerr", C.c_void_p), ("omega", C.c_void_p), ("wavenum", C.c_void_p),
        ("ho_disp", C.c_void_p), ("omega_min", C.c_double), ("omega_max", C.c_double),
        ("kt2", C.c_void_p), ("qdht_c", C.c_void_p), ("qdht_m1", C.c_void_p),
        ("max_tolerance", C.c_double),
        ("gas", C.c_int), ("levels", C.c_int), ("potentials", C.c_void_p), ("th_coeff", C.c_double),
    ]


_lib = None


def build():
    """Compile the oracle library (make, gcc) if it is missing or stale."""
    src = [os.path.join(HERE, f) for f in ("gs_oracle.c", "gs_oracle_adj.c", "gs_oracle.h", "Makefile")]
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in src):
        return LIB
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        L.gso_fft.argtypes = [C.c_int, P, P, C.c_int]
        L.gso_qdht_run_many.argtypes = [P, P, C.c_long, C.c_long, C.c_long]
        L.gso_plasma_losses.argtypes = [P, P, P, C.c_int, P]
        L.gso_nl_response.argtypes = [P, P, P]
        L.gso_nl_step.argtypes = [P, P, P, C.c_double, P, P]
        L.gso_lstep.argtypes = [P, P, P, P, C.c_double]
        L.gso_propagator.argtypes = [P, P, P, P, P, C.c_double, C.c_double, C.c_double, P, P, P]
        L.gso_row_reductions.argtypes = [P, P, P, P, P]
        L.gso_nl_response_vjp.argtypes = [P, P, P, P]
        L.gso_nl_step_vjp.argtypes = [P, P, C.c_double, P, P]
        L.gso_lstep_vjp.argtypes = [P, P, P, P, C.c_double]
        L.gso_qdht_transposed.argtypes = [P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _check(rc):
    if rc:
        raise OracleError(ERRORS.get(rc, f"oracle error {rc}"))


class Oracle:
    def __init__(self, T: dict, nonlinear: bool = True, nthreads: int = 0):
        self.T = T
        self.keep = {}
        c = _Ctx()
        c.n_r, c.n_t = int(T["n_r"]), int(T["n_t"])
        c.nonlinear = 1 if nonlinear else 0
        c.nthreads = int(nthreads)
        for k in ("tstep", "tmin", "tmax", "omega0", "ionrate_denom", "neutral_density",
                  "ionization_potential", "ponderomotive", "avalanche_cs", "recombination_tau",
                  "raman_fraction", "n2", "omega_min", "omega_max", "max_tolerance"):
            setattr(c, k, float(T[k]))
        c.rho0 = float(T.get("rho0", 0.0))
        for k, dt in (("rate_ln", np.float64), ("plasma_func", np.complex128),
                      ("raman_func", np.complex128), ("kerr", np.float64), ("omega", np.float64),
                      ("wavenum", np.complex128), ("ho_disp", np.float64), ("kt2", np.float64),
                      ("qdht_m1", np.float64)):
            a = np.ascontiguousarray(T[k], dtype=dt)
            self.keep[k] = a
            setattr(c, k, a.ctypes.data)
        c.gas = int(T.get("gas", 0))
        c.levels = int(T.get("ion_levels", 1))
        pot = np.ascontiguousarray(T.get("ion_potentials", [T["ionization_potential"]]), dtype=np.float64)
        self.keep["ion_potentials"] = pot
        c.potentials = pot.ctypes.data
        c.th_coeff = float(T.get("th_coeff", 0.0))
        cm = np.asfortranarray(np.asarray(T["qdht_c"], dtype=np.float64))  # C[i + N*j]
        self.keep["qdht_c"] = cm
        c.qdht_c = cm.ctypes.data
        self.ctx = c
        self.cp = C.byref(c)
        self.L = lib()

    # -- hot-path functions ------------------------------------------------
    def nl_response(self, row):
        row = np.ascontiguousarray(row, dtype=np.complex128)
        out = np.empty_like(row)
        _check(self.L.gso_nl_response(self.cp, _p(row), _p(out)))
        return out

    def plasma(self, e_row):
        e_row = np.ascontiguousarray(e_row, dtype=np.complex128)
        pro = np.empty(len(e_row))
        loss = np.empty_like(e_row)
        _check(self.L.gso_plasma_losses(self.cp, _p(e_row), _p(pro), 1, _p(loss)))
        return pro, loss

    def nl_step(self, field, dz):
        field = np.ascontiguousarray(field, dtype=np.complex128)
        bb1 = np.empty_like(field)
        a2, n2 = C.c_double(), C.c_double()
        _check(self.L.gso_nl_step(self.cp, _p(field), _p(bb1), float(dz), C.byref(a2), C.byref(n2)))
        return bb1, a2.value, n2.value

    def qdht(self, data):
        """ht_run on a [n_r][n_t] array, returning a new array."""
        d = np.array(data, dtype=np.complex128, order="C", copy=True)
        _check(self.L.gso_qdht_run_many(self.cp, _p(d), self.ctx.n_t, self.ctx.n_t, 1))
        return d

    def lstep(self, bb1_k, bb2, dz):
        """calculate_Lstep: returns (FIELD in (k,omega), updated BIGBUFFER2)."""
        bb1_k = np.ascontiguousarray(bb1_k, dtype=np.complex128)
        b2 = np.array(bb2, dtype=np.complex128, order="C", copy=True)
        f = np.empty_like(b2)
        _check(self.L.gso_lstep(self.cp, _p(f), _p(bb1_k), _p(b2), float(dz)))
        return f, b2

    def apply_apertures(self, field, bb2, current_z, state):
        """The aperture block at the end of an accepted propagator() call (propagator.cu:
        232-261): with CURRENT_Z still the z before the step, when it has reached the next
        aperture's z, FIELD rows whose QDHT radius x_n R_MAX exceeds its radius are zeroed,
        BIGBUFFER2 = QDHT(FIELD), and the aperture is used up.  `state` holds the count left."""
        zs, rs = self.T.get("aperture_z", []), self.T.get("aperture_r", [])
        n = state.setdefault("aperture_n", len(zs))
        if n > 0 and current_z >= zs[n - 1]:
            R = np.asarray(self.T["qdht_x"]) * self.T["r_max"]
            field = np.array(field, copy=True)
            field[R > rs[n - 1]] = 0.0
            bb2 = self.qdht(field)
            state["aperture_n"] = n - 1
        return field, bb2

    def propagator(self, field, bb2, zstep, current_z, znet_cur, znet_prev, step_n=0):
        """One propagator() call; returns (field, bb2, zstep, step_n, max_a2, max_nl2)."""
        f = np.array(field, dtype=np.complex128, order="C", copy=True)
        b2 = np.array(bb2, dtype=np.complex128, order="C", copy=True)
        b1 = np.empty_like(f)
        dz = C.c_double(zstep)
        sn = C.c_uint(step_n)
        a2, n2 = C.c_double(), C.c_double()
        _check(self.L.gso_propagator(self.cp, _p(f), _p(b1), _p(b2), C.byref(dz), float(current_z),
                                     float(znet_cur), float(znet_prev), C.byref(sn),
                                     C.byref(a2), C.byref(n2)))
        return f, b2, dz.value, sn.value, a2.value, n2.value

    # -- dumps (dump_types.cpp) --------------------------------------------
    def dumps(self, field):
        nr, nt = self.ctx.n_r, self.ctx.n_t
        field = np.ascontiguousarray(field, dtype=np.complex128)
        mI = np.empty(nr); fl = np.empty(nr); pm = np.empty(nr)
        _check(self.L.gso_row_reductions(self.cp, _p(field), _p(mI), _p(fl), _p(pm)))
        fa = self.fft(field[0], +1) / nt
        x = self.T["qdht_x"]
        a2 = field.real ** 2 + field.imag ** 2
        # average_spectrum, uniaxial branch (dump_types.cpp:427-457)
        s = a2[0] * x[0] * (x[1] - x[0])
        x1 = x[0]
        for cx in range(1, nr):
            x2 = x[cx]
            s = s + a2[cx] * x2 * (x2 - x1)
            x1 = x2
        s = s * (self.T["r_max"] * self.T["r_max"] / 2.0)
        return {"mI": mI, "f": fl, "pm": pm, "fa": fa, "s": s}

    def fft(self, row, sign):
        row = np.ascontiguousarray(row, dtype=np.complex128)
        out = np.empty_like(row)
        _check(self.L.gso_fft(len(row), _p(row), _p(out), int(sign)))
        return out

    def run(self, field, dz0, steps=None, dump_every=1):
        """The z-loop (solver_main.cpp:202-225).  Returns (dict of dump lists, final state).
        ``steps`` bounds the number of propagator() calls (None = until the last ZNET)."""
        T = self.T
        znet = T["znet"]
        nz = len(znet)
        f = np.array(field, dtype=np.complex128, copy=True)
        bb2 = self.qdht(f)
        cz = float(znet[0]); n_z = 0; step_n = 0; zstep = float(dz0)
        out = {k: [] for k in ("mI", "f", "pm", "fa", "s", "z")}
        calls = 0
        ap_state = {}
        while True:
            if cz >= znet[n_z]:
                if n_z % dump_every == 0 or n_z == nz - 1:
                    d = self.dumps(f)
                    for k in d:
                        out[k].append(d[k])
                    out["z"].append(n_z)
                if n_z == nz - 1:
                    break
                n_z += 1
            if steps is not None and calls >= steps:
                break
            f, bb2, zstep, step_n, _, _ = self.propagator(f, bb2, zstep, cz, znet[n_z], znet[n_z - 1], step_n)
            f, bb2 = self.apply_apertures(f, bb2, cz, ap_state)
            step_n += 1
            calls += 1
            cz += zstep
        return out, {"field": f, "bb2": bb2, "z": cz, "zstep": zstep, "step_n": step_n, "n_z": n_z}

    # -- adjoint (gs_oracle_adj.c) ------------------------------------------
    def nl_response_vjp(self, y_row, kbar_row):
        y = np.ascontiguousarray(y_row, dtype=np.complex128)
        kb = np.ascontiguousarray(kbar_row, dtype=np.complex128)
        out = np.empty_like(y)
        _check(self.L.gso_nl_response_vjp(self.cp, _p(y), _p(kb), _p(out)))
        return out

    def nl_step_vjp(self, field, dz, rbar):
        f = np.ascontiguousarray(field, dtype=np.complex128)
        rb = np.ascontiguousarray(rbar, dtype=np.complex128)
        out = np.empty_like(f)
        _check(self.L.gso_nl_step_vjp(self.cp, _p(f), float(dz), _p(rb), _p(out)))
        return out

    def lstep_vjp(self, fbar_k, sbar, dz):
        """Returns (cotangent of BIGBUFFER2 before the step, of BIGBUFFER1 in (k,omega))."""
        fb = np.ascontiguousarray(fbar_k, dtype=np.complex128)
        sb = np.array(sbar, dtype=np.complex128, order="C", copy=True)
        b1 = np.empty_like(sb)
        _check(self.L.gso_lstep_vjp(self.cp, _p(fb), _p(sb), _p(b1), float(dz)))
        return sb, b1

    def qdht_t(self, data):
        d = np.array(data, dtype=np.complex128, order="C", copy=True)
        _check(self.L.gso_qdht_transposed(self.cp, _p(d)))
        return d

    def forward_fixed(self, field, dz_rk, dz_lin):
        """propagator() calls with the step sizes given (RK4 stages use dz_rk[n], the linear
        step dz_lin[n]; the controller is bypassed).  Returns (FIELD, BIGBUFFER2) after."""
        f = np.array(field, dtype=np.complex128, copy=True)
        s = self.qdht(f)
        for a, b in zip(dz_rk, dz_lin):
            bb1, _, _ = self.nl_step(f, a)
            fk, s = self.lstep(self.qdht(bb1), s, b)
            f = self.qdht(fk)
        return f, s

    def gradient(self, field, dz_rk, dz_lin, weights):
        """J = sum w |FIELD_final|^2 after forward_fixed and dJ/dFIELD_0 (g = dJ/dRe + i dJ/dIm)
        by the adjoint, storing every step's FIELD."""
        f = np.array(field, dtype=np.complex128, copy=True)
        s = self.qdht(f)
        hist = []
        for a, b in zip(dz_rk, dz_lin):
            hist.append(f)
            bb1, _, _ = self.nl_step(f, a)
            fk, s = self.lstep(self.qdht(bb1), s, b)
            f = self.qdht(fk)
        J = float(np.sum(weights * (f.real ** 2 + f.imag ** 2)))
        ab = 2 * weights * f
        sb = np.zeros_like(f)
        for n in range(len(hist) - 1, -1, -1):
            sb, b1 = self.lstep_vjp(self.qdht_t(ab), sb, dz_lin[n])
            ab = self.nl_step_vjp(hist[n], dz_rk[n], self.qdht_t(b1))
        ab = ab + self.qdht_t(sb)
        return J, ab
