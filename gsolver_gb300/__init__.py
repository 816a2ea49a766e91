"""gsolver_gb300 -- GB300-native (sm_103a) z-step core of the gsolver_solid_qdht path.

Python mirror of the C ABI in include/gs_abi.h (ctypes, no torch types).  The compute
path is libgsolver_gb300.so built in-tree by gsolver_gb300.build; importing a handle
fails loudly if that library is missing: there is no CPU fallback.

``Propagator`` mirrors the reference's hot-path functions on one pulse:
  set_field / get_field  <- FIELD, BIGBUFFER2 host globals (solver.h:169)
  nl_step                <- calculate_NLstep (propagator.cu:268-426)
  lstep                  <- ht_run + calculate_Lstep + ht_run (propagator.cu:179-213)
  qdht                   <- ht_run -> qdht_plan::run_many (fhatha.cpp:218-230)
  step                   <- propagator() (propagator.cu:125-266)
Physics errors raise ``GsError`` with the reference's exception text.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# GS_CHECK=1 in the environment at import: the GS_CHECK build (python -m gsolver_gb300.build --check)
LIB_PATH = os.path.join(HERE, "_build_check" if os.environ.get("GS_CHECK") == "1" else "_build", "libgsolver_gb300.so")

GS_OK, GS_ERR_ARG, GS_ERR_CUDA, GS_ERR_BLAST, GS_ERR_NAN, GS_ERR_COLLAPSE = 0, 1, 2, 3, 4, 5
GS_ERR_STATE, GS_ERR_UNSUPPORTED, GS_ERR_NOMEM = 6, 7, 8
PREC_FP64, PREC_MIXED = 0, 1

# every function declared in include/gs_abi.h
ABI_FUNCTIONS = (
    "gs_create", "gs_upload_tables", "gs_set_field", "gs_get_field", "gs_nl_step", "gs_get_nl",
    "gs_lstep", "gs_qdht", "gs_step", "gs_step_host", "gs_advance", "gs_stream", "gs_launch_count", "gs_qdht_timing", "gs_nl_timing",
    "gs_destroy",
    "gs_last_error", "gs_status_string",
    # include/gs_setup.h
    "gs_setup_from_config", "gs_setup_last_error", "gs_setup_grid", "gs_setup_params",
    "gs_setup_tables", "gs_setup_field", "gs_setup_znet", "gs_setup_destroy",
    "gs_run_config", "gs_run_last_error", "gs_dump_reductions", "gs_get_time_field",
    "gs_plasma_max_noalloc", "gs_noalloc_max_samples", "gs_noalloc_last_error",
    "gs_forward_fixed", "gs_gradient", "gs_adjoint_step", "gs_adjoint_stride",
    "gs_batch_create", "gs_batch_step", "gs_batch_stream", "gs_batch_launch_count", "gs_batch_last_error",
    "gs_batch_destroy", "gs_batch_advance", "gs_autotune", "gs_set_nl_threads", "gs_get_nl_threads", "gs_batch_autotune",
    "gs_set_apertures", "gs_setup_apertures", "gs_setup_from_config_dev",
    "gs_energy", "gs_set_energy_tolerance", "gs_energy_stats", "gs_checkpoint_save", "gs_checkpoint_load",
    "gs_selftest_bounded_wait", "gs_check_build", "gs_selftest_bounds",
)


class GsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("n_r", C.c_int), ("n_t", C.c_int), ("precision", C.c_int), ("nonlinear", C.c_int),
        ("device", C.c_int), ("gas", C.c_int),
        ("tstep", C.c_double), ("tmin", C.c_double), ("tmax", C.c_double), ("omega0", C.c_double),
        ("ionrate_denom", C.c_double), ("neutral_density", C.c_double), ("rho0", C.c_double),
        ("ionization_potential", C.c_double), ("ponderomotive", C.c_double),
        ("avalanche_cs", C.c_double), ("recombination_tau", C.c_double),
        ("raman_fraction", C.c_double), ("n2", C.c_double),
        ("omega_min", C.c_double), ("omega_max", C.c_double), ("max_tolerance", C.c_double),
        ("raman_tau", C.c_double), ("raman_omega", C.c_double), ("th_coeff", C.c_double),
        ("ion_levels", C.c_int), ("ion_potentials", C.c_double * 8),
    ]


class Tables(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in (
        "rate_ln", "plasma_func", "raman_func", "kerr", "omega", "wavenum", "ho_disp", "kt2",
        "qdht_c", "qdht_m1")]


class RunStats(C.Structure):
    _fields_ = [("calls", C.c_longlong), ("step_n", C.c_uint), ("n_z", C.c_int), ("z", C.c_double),
                ("zstep", C.c_double), ("seconds", C.c_double)]


_lib = None


def load_library(path: str | None = None):
    """Load libgsolver_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with `python -m gsolver_gb300.build` "
                           "(the GPU path has no fallback)")
    L = C.CDLL(p)
    V, D, I = C.c_void_p, C.c_double, C.c_int
    PD = C.POINTER(C.c_double)
    L.gs_create.argtypes = [C.POINTER(Params), C.POINTER(V)]
    L.gs_upload_tables.argtypes = [V, C.POINTER(Tables)]
    L.gs_set_field.argtypes = [V, V, V]
    L.gs_get_field.argtypes = [V, V, V]
    L.gs_nl_step.argtypes = [V, D, PD, PD]
    L.gs_get_nl.argtypes = [V, V]
    L.gs_lstep.argtypes = [V, D]
    L.gs_qdht.argtypes = [V, V]
    L.gs_step.argtypes = [V, D, D, D, PD, C.POINTER(C.c_uint), PD, PD]
    L.gs_step_host.argtypes = [V, V, V, D, D, D, PD, C.POINTER(C.c_uint), PD, PD]
    L.gs_advance.argtypes = [V, V, C.c_int, C.c_int, PD, PD, C.POINTER(C.c_uint), C.c_int, C.POINTER(C.c_int),
                             C.POINTER(C.c_int)]
    L.gs_stream.argtypes = [V]
    L.gs_stream.restype = V
    L.gs_launch_count.argtypes = [V]
    L.gs_launch_count.restype = C.c_longlong
    L.gs_qdht_timing.argtypes = [V, I, PD, C.POINTER(C.c_int)]
    L.gs_nl_timing.argtypes = [V, I, PD, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.gs_destroy.argtypes = [V]
    L.gs_last_error.argtypes = [V]
    L.gs_last_error.restype = C.c_char_p
    L.gs_status_string.argtypes = [I]
    L.gs_status_string.restype = C.c_char_p
    L.gs_dump_reductions.argtypes = [V, V, D, V, V, V, V, V]
    L.gs_get_time_field.argtypes = [V, V]
    L.gs_run_config.argtypes = [C.c_char_p, C.c_char_p, I, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), I, I,
                                C.c_ulonglong, D, C.c_longlong, C.POINTER(RunStats)]
    L.gs_run_last_error.restype = C.c_char_p
    L.gs_forward_fixed.argtypes = [V, V, I, V, V, V, PD, V]
    L.gs_gradient.argtypes = [V, V, I, V, V, V, I, PD, V]
    L.gs_adjoint_step.argtypes = [V, D, D, V, V]
    L.gs_adjoint_stride.argtypes = [V, C.POINTER(C.c_int)]
    L.gs_batch_create.argtypes = [I, C.POINTER(V), C.POINTER(V)]
    L.gs_batch_step.argtypes = [V, I, V, I]
    L.gs_batch_stream.argtypes = [V]
    L.gs_batch_stream.restype = V
    L.gs_batch_launch_count.argtypes = [V]
    L.gs_batch_launch_count.restype = C.c_longlong
    L.gs_batch_last_error.argtypes = [V]
    L.gs_batch_last_error.restype = C.c_char_p
    L.gs_batch_destroy.argtypes = [V]
    L.gs_autotune.argtypes = [V, C.POINTER(C.c_int), PD]
    L.gs_set_nl_threads.argtypes = [V, I]
    L.gs_get_nl_threads.argtypes = [V]
    L.gs_batch_autotune.argtypes = [V, V, PD, PD, C.POINTER(C.c_int)]
    L.gs_batch_advance.argtypes = [V, V, V, V, V, V, V, I, V, V]
    L.gs_set_apertures.argtypes = [V, I, V, V, V, D]
    L.gs_setup_apertures.argtypes = [V, C.POINTER(C.c_int), V, V]
    L.gs_energy.argtypes = [V, V, D, PD, PD]
    L.gs_selftest_bounded_wait.argtypes = [V, D]
    L.gs_check_build.argtypes = []
    L.gs_selftest_bounds.argtypes = [V]
    L.gs_set_energy_tolerance.argtypes = [V, D, V, D]
    L.gs_energy_stats.argtypes = [V, PD, C.POINTER(C.c_longlong)]
    L.gs_checkpoint_save.argtypes = [V, C.c_char_p, D, D, I, C.c_uint]
    L.gs_checkpoint_load.argtypes = [V, C.c_char_p, PD, PD, C.POINTER(C.c_int), C.POINTER(C.c_uint)]
    _lib = L
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


PARAM_KEYS = ("tstep", "tmin", "tmax", "omega0", "ionrate_denom", "neutral_density",
              "ionization_potential", "ponderomotive", "avalanche_cs", "recombination_tau",
              "raman_fraction", "n2", "omega_min", "omega_max", "max_tolerance")


class Propagator:
    """One pulse on one GPU behind the C ABI.  ``setup`` is a dict with the scalar
    parameters and FP64 tables (keys as in gs_params / gs_tables); see
    ``Setup(config).as_dict()`` for the product's own builder."""

    def __init__(self, setup: dict, precision: int = PREC_FP64, nonlinear: bool = True, device: int = 0):
        self.L = load_library()
        self.nr, self.nt = int(setup["n_r"]), int(setup["n_t"])
        p = Params()
        p.n_r, p.n_t, p.precision, p.nonlinear, p.device = self.nr, self.nt, int(precision), int(bool(nonlinear)), int(device)
        for k in PARAM_KEYS:
            setattr(p, k, float(setup[k]))
        p.rho0 = float(setup.get("rho0", 0.0))
        p.raman_tau = float(setup.get("raman_tau", 0.0))
        p.raman_omega = float(setup.get("raman_omega", 0.0))
        p.gas = int(setup.get("gas", 0))
        p.th_coeff = float(setup.get("th_coeff", 0.0))
        lv = int(setup.get("ion_levels", 1)) if p.gas else 1
        p.ion_levels = lv
        if lv > 1:
            pots = np.asarray(setup["ion_potentials"], dtype=np.float64)
            for i in range(lv):
                p.ion_potentials[i] = float(pots[i])
        self.params = p
        h = C.c_void_p()
        rc = self.L.gs_create(C.byref(p), C.byref(h))
        if rc:
            raise GsError(rc, self.L.gs_last_error(None).decode())
        self.h = h
        self.upload_tables(setup)
        if len(setup.get("aperture_z", ())) > 0:   # apertures of the config (propagator.cu:232-261)
            self.set_apertures(setup["aperture_z"], setup["aperture_r"], setup["qdht_x"], setup["r_max"])

    def upload_tables(self, setup: dict):
        """gs_upload_tables: the per-omega / per-k tables, the rate table and the QDHT matrix
        (cuda_load_const); may be called again on a live handle to replace them."""
        self._keep = {}
        t = Tables()
        for k, dt in (("rate_ln", np.float64), ("plasma_func", np.complex128), ("raman_func", np.complex128),
                      ("kerr", np.float64), ("omega", np.float64), ("wavenum", np.complex128),
                      ("ho_disp", np.float64), ("kt2", np.float64), ("qdht_m1", np.float64)):
            a = np.ascontiguousarray(setup[k], dtype=dt)
            self._keep[k] = a
            setattr(t, k, a.ctypes.data)
        cm = np.asfortranarray(np.asarray(setup["qdht_c"], dtype=np.float64))   # C[i + n_r*j]
        self._keep["qdht_c"] = cm
        t.qdht_c = cm.ctypes.data
        self._check(self.L.gs_upload_tables(self.h, C.byref(t)))

    def _check(self, rc):
        if rc:
            raise GsError(rc, self.L.gs_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.gs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _arr(self, a):
        a = np.ascontiguousarray(a, dtype=np.complex128)
        if a.shape != (self.nr, self.nt):
            raise ValueError(f"expected shape {(self.nr, self.nt)}, got {a.shape}")
        return a

    def set_field(self, field, spec=None):
        f = self._arr(field)
        s = self._arr(spec) if spec is not None else None
        self._check(self.L.gs_set_field(self.h, _ptr(f), _ptr(s)))

    def get_field(self, want_spec=True):
        f = np.empty((self.nr, self.nt), np.complex128)
        s = np.empty((self.nr, self.nt), np.complex128) if want_spec else None
        self._check(self.L.gs_get_field(self.h, _ptr(f), _ptr(s)))
        return (f, s) if want_spec else f

    def nl_step(self, dz):
        a2, n2 = C.c_double(), C.c_double()
        self._check(self.L.gs_nl_step(self.h, float(dz), C.byref(a2), C.byref(n2)))
        return a2.value, n2.value

    def get_nl(self):
        b = np.empty((self.nr, self.nt), np.complex128)
        self._check(self.L.gs_get_nl(self.h, _ptr(b)))
        return b

    def lstep(self, dz):
        self._check(self.L.gs_lstep(self.h, float(dz)))

    def qdht(self, data):
        d = np.array(self._arr(data), copy=True)
        self._check(self.L.gs_qdht(self.h, _ptr(d)))
        return d

    def step(self, current_z, znet_cur, znet_prev, zstep, step_n=0):
        dz = C.c_double(zstep)
        sn = C.c_uint(step_n)
        a2, n2 = C.c_double(), C.c_double()
        self._check(self.L.gs_step(self.h, float(current_z), float(znet_cur), float(znet_prev),
                                   C.byref(dz), C.byref(sn), C.byref(a2), C.byref(n2)))
        return dz.value, sn.value, a2.value, n2.value

    def step_host(self, field_ptr, spec_ptr, current_z, znet_cur, znet_prev, zstep, step_n=0):
        """gs_step_host: one propagator() call on host FIELD / BIGBUFFER2 buffers (raw pointers to
        [n_r][n_t] complex128, e.g. pinned), taken in and given back.  Returns (ZSTEP, STEP_N)."""
        dz = C.c_double(zstep)
        sn = C.c_uint(step_n)
        self._check(self.L.gs_step_host(self.h, C.c_void_p(field_ptr), C.c_void_p(spec_ptr), float(current_z),
                                        float(znet_cur), float(znet_prev), C.byref(dz), C.byref(sn), None, None))
        return dz.value, sn.value

    def advance(self, znet, n_z, current_z, zstep, step_n=0, max_calls=1 << 30):
        """gs_advance: up to max_calls propagator() calls from CURRENT_Z below ZNET[n_z], the step
        controller on the device.  Returns (CURRENT_Z, ZSTEP, STEP_N, calls, reached ZNET[n_z])."""
        zn = np.ascontiguousarray(znet, dtype=np.float64)
        cz, dz, sn = C.c_double(current_z), C.c_double(zstep), C.c_uint(step_n)
        calls, reached = C.c_int(), C.c_int()
        self._check(self.L.gs_advance(self.h, _ptr(zn), len(zn), int(n_z), C.byref(cz), C.byref(dz), C.byref(sn),
                                      int(max_calls), C.byref(calls), C.byref(reached)))
        return cz.value, dz.value, sn.value, calls.value, bool(reached.value)

    def stream_ptr(self):
        return int(self.L.gs_stream(self.h) or 0)

    def set_field_ptr(self, field_ptr, spec_ptr=None):
        """gs_set_field from raw host pointers (e.g. pinned buffers)."""
        self._check(self.L.gs_set_field(self.h, C.c_void_p(field_ptr), C.c_void_p(spec_ptr) if spec_ptr else None))

    def get_field_ptr(self, field_ptr, spec_ptr=None):
        self._check(self.L.gs_get_field(self.h, C.c_void_p(field_ptr) if field_ptr else None,
                                        C.c_void_p(spec_ptr) if spec_ptr else None))

    def dumps(self, qdht_x, r_max):
        """Device reductions of the current FIELD for the .udf dumps (gs_dump_reductions)."""
        nr, nt = self.nr, self.nt
        out = {"mI": np.empty(nr), "f": np.empty(nr), "pm": np.empty(nr), "fa": np.empty(nt, np.complex128),
               "s": np.empty(nt)}
        x = np.ascontiguousarray(qdht_x, dtype=np.float64)
        self._check(self.L.gs_dump_reductions(self.h, _ptr(x), float(r_max), _ptr(out["mI"]), _ptr(out["f"]),
                                              _ptr(out["pm"]), _ptr(out["fa"]), _ptr(out["s"])))
        return out

    def time_field(self):
        e = np.empty((self.nr, self.nt), np.complex128)
        self._check(self.L.gs_get_time_field(self.h, _ptr(e)))
        return e

    def launch_count(self):
        return int(self.L.gs_launch_count(self.h))

    def qdht_timing(self, enable=True):
        ms, n = C.c_double(), C.c_int()
        self._check(self.L.gs_qdht_timing(self.h, int(enable), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def nl_timing(self, enable=True):
        """CUDA-event time of the fused RK4-stage kernels since the previous call:
        (ms of their launches, RK4 stages timed, launches timed)."""
        f, n, k = C.c_double(), C.c_int(), C.c_int()
        self._check(self.L.gs_nl_timing(self.h, int(enable), C.byref(f), C.byref(n), C.byref(k)))
        return f.value, n.value, k.value

    def set_apertures(self, z, r, qdht_x, r_max):
        """Apertures in the reference's array order (the last entry is applied first); gs_step
        applies them after accepted steps (gs_set_apertures)."""
        z = np.ascontiguousarray(z, dtype=np.float64)
        r = np.ascontiguousarray(r, dtype=np.float64)
        x = np.ascontiguousarray(qdht_x, dtype=np.float64)
        self._check(self.L.gs_set_apertures(self.h, len(z), _ptr(z), _ptr(r), _ptr(x), float(r_max)))

    def energy(self, qdht_x, r_max):
        """(energy, photon number) of FIELD: the sum of the average spectrum and of it over omega
        (gs_energy, FP64 on the device)."""
        x = np.ascontiguousarray(qdht_x, dtype=np.float64)
        e, n = C.c_double(), C.c_double()
        self._check(self.L.gs_energy(self.h, _ptr(x), float(r_max), C.byref(e), C.byref(n)))
        return e.value, n.value

    def set_energy_tolerance(self, tol, qdht_x=None, r_max=0.0):
        """The photon-number check of step() (gs_set_energy_tolerance); 0 turns it off."""
        x = np.ascontiguousarray(qdht_x, dtype=np.float64) if qdht_x is not None else None
        self._check(self.L.gs_set_energy_tolerance(self.h, float(tol), _ptr(x), float(r_max)))

    def energy_stats(self):
        """(|N1/N0 - 1| of the last accepted step, rejections so far)."""
        r, k = C.c_double(), C.c_longlong()
        self._check(self.L.gs_energy_stats(self.h, C.byref(r), C.byref(k)))
        return r.value, k.value

    def checkpoint_save(self, path, current_z=0.0, zstep=0.0, n_z=0, step_n=0):
        self._check(self.L.gs_checkpoint_save(self.h, str(path).encode(), float(current_z), float(zstep), int(n_z),
                                              int(step_n)))

    def checkpoint_load(self, path):
        """Restore a saved state; returns the z-loop state {z, zstep, n_z, step_n}."""
        z, dz, nz, sn = C.c_double(), C.c_double(), C.c_int(), C.c_uint()
        self._check(self.L.gs_checkpoint_load(self.h, str(path).encode(), C.byref(z), C.byref(dz), C.byref(nz),
                                              C.byref(sn)))
        return {"z": z.value, "zstep": dz.value, "n_z": nz.value, "step_n": sn.value}

    def selftest_bounded_wait(self, limit_s=1e-3):
        """gs_selftest_bounded_wait: raises GsError (GS_ERR_CUDA, 'wait expired') when the bounded
        waits report as they should."""
        self._check(self.L.gs_selftest_bounded_wait(self.h, float(limit_s)))

    def selftest_bounds(self):
        """gs_selftest_bounds: raises GsError (GS_ERR_CUDA, 'index out of bounds') in a GS_CHECK
        build whose index test reports as it should (GS_ERR_UNSUPPORTED in other builds)."""
        self._check(self.L.gs_selftest_bounds(self.h))

    def nl_threads(self, threads=None):
        """Read, or set (0: default), the fused kernels' threads per row."""
        if threads is not None:
            self._check(self.L.gs_set_nl_threads(self.h, int(threads)))
        return self.L.gs_get_nl_threads(self.h)

    def autotune(self):
        """Pick the fused NL kernels' launch shape for this grid (gs_autotune); returns
        (threads per row, ms per RK4 stage)."""
        t, ms = C.c_int(), C.c_double()
        self._check(self.L.gs_autotune(self.h, C.byref(t), C.byref(ms)))
        return t.value, ms.value

    # -- gradients (gs_forward_fixed / gs_gradient / gs_adjoint_step) ---------------
    def _schedule(self, dz_rk, dz_lin):
        a = np.ascontiguousarray(dz_rk, dtype=np.float64)
        b = np.ascontiguousarray(dz_lin, dtype=np.float64)
        if a.shape != b.shape or a.ndim != 1:
            raise ValueError("dz_rk and dz_lin must be 1-D of equal length")
        return a, b

    def forward_fixed(self, field, dz_rk, dz_lin, weights):
        """propagator() calls with the given step sizes; returns (J, FIELD after) with
        J = sum(weights * |FIELD after|^2)."""
        f = np.ascontiguousarray(field, dtype=np.complex128)
        a, b = self._schedule(dz_rk, dz_lin)
        w = np.ascontiguousarray(weights, dtype=np.float64)
        out = np.empty_like(f)
        J = C.c_double()
        self._check(self.L.gs_forward_fixed(self.h, _ptr(f), len(a), _ptr(a), _ptr(b), _ptr(w), C.byref(J), _ptr(out)))
        return J.value, out

    def gradient(self, field, dz_rk, dz_lin, weights, checkpoint_stride=0):
        """(J, dJ/dRe(FIELD_0) + i dJ/dIm(FIELD_0)) by the adjoint."""
        f = np.ascontiguousarray(field, dtype=np.complex128)
        a, b = self._schedule(dz_rk, dz_lin)
        w = np.ascontiguousarray(weights, dtype=np.float64)
        g = np.empty_like(f)
        J = C.c_double()
        self._check(self.L.gs_gradient(self.h, _ptr(f), len(a), _ptr(a), _ptr(b), _ptr(w), int(checkpoint_stride),
                                       C.byref(J), _ptr(g)))
        return J.value, g

    def adjoint_stride(self):
        """Checkpoint stride of the last gradient() call (0 before the first)."""
        k = C.c_int()
        self._check(self.L.gs_adjoint_stride(self.h, C.byref(k)))
        return k.value

    def adjoint_step(self, dz_rk, dz_lin, field_bar, spec_bar):
        """Run one step forward from the current state and map the cotangents of (FIELD,
        BIGBUFFER2) after it to those before it."""
        fb = np.array(field_bar, dtype=np.complex128, order="C", copy=True)
        sb = np.array(spec_bar, dtype=np.complex128, order="C", copy=True)
        self._check(self.L.gs_adjoint_step(self.h, float(dz_rk), float(dz_lin), _ptr(fb), _ptr(sb)))
        return fb, sb

    def run(self, znet, dz0, steps=None, on_dump=None, device=False):
        """The z-loop of solver_main.cpp:202-225 over ZNET; on_dump(n_z, self) at each
        ZNET point.  Returns (final z, zstep, STEP_N, propagator calls).  device=True runs the
        calls between ZNET points through gs_advance (the step controller on the device)."""
        cz = float(znet[0]); n_z = 0; step_n = 0; zstep = float(dz0); calls = 0
        nz = len(znet)
        while True:
            if cz >= znet[n_z]:
                if on_dump:
                    on_dump(n_z, self)
                if n_z == nz - 1:
                    break
                n_z += 1
            if steps is not None and calls >= steps:
                break
            if device:
                left = (1 << 30) if steps is None else steps - calls
                cz, zstep, step_n, k, _ = self.advance(znet, n_z, cz, zstep, step_n, left)
                calls += k
                continue
            zstep, step_n, _, _ = self.step(cz, znet[n_z], znet[n_z - 1], zstep, step_n)
            step_n += 1
            calls += 1
            cz += zstep
        return cz, zstep, step_n, calls


# ----------------------------------------------------------------- host set-up --
class Setup:
    """Product set-up of one pulse from a reference-format config (include/gs_setup.h).

    ``as_dict()`` returns the same keys Propagator takes, built by the library's own C++
    (no oracle involved)."""

    def __init__(self, config_path: str, overrides: dict | None = None, noise_seed: int = 0,
                 noise_sigma: float = 0.0, device: int | None = None):
        """device: None builds everything on the host (gs_setup_from_config); a GPU ordinal
        builds the rate table, the QDHT matrix and the start field there
        (gs_setup_from_config_dev)."""
        L = load_library()
        V = C.c_void_p
        L.gs_setup_from_config.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p),
                                           C.c_ulonglong, C.c_double, C.POINTER(V)]
        L.gs_setup_from_config_dev.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p),
                                               C.c_ulonglong, C.c_double, C.c_int, C.POINTER(V)]
        L.gs_setup_last_error.restype = C.c_char_p
        L.gs_setup_grid.argtypes = [V, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.gs_setup_params.argtypes = [V, C.POINTER(Params)]
        L.gs_setup_tables.argtypes = [V, C.POINTER(Tables)]
        L.gs_setup_field.argtypes = [V, V]
        L.gs_setup_znet.argtypes = [V, V, C.POINTER(C.c_double), C.POINTER(C.c_double), V]
        L.gs_setup_destroy.argtypes = [V]
        self.L = L
        ov = overrides or {}
        keys = (C.c_char_p * max(1, len(ov)))(*[k.encode() for k in ov])
        vals = (C.c_char_p * max(1, len(ov)))(*[str(v).encode() for v in ov.values()])
        s = V()
        if device is None:
            rc = L.gs_setup_from_config(config_path.encode(), len(ov), keys, vals, int(noise_seed), float(noise_sigma),
                                        C.byref(s))
        else:
            rc = L.gs_setup_from_config_dev(config_path.encode(), len(ov), keys, vals, int(noise_seed),
                                            float(noise_sigma), int(device), C.byref(s))
        if rc:
            raise GsError(rc, L.gs_setup_last_error().decode())
        self.s = s

    def __del__(self):
        if getattr(self, "s", None):
            self.L.gs_setup_destroy(self.s)
            self.s = None

    def as_dict(self) -> dict:
        L = self.L
        nr, nt, nz = C.c_int(), C.c_int(), C.c_int()
        L.gs_setup_grid(self.s, C.byref(nr), C.byref(nt), C.byref(nz))
        nr, nt, nz = nr.value, nt.value, nz.value
        p = Params()
        L.gs_setup_params(self.s, C.byref(p))
        t = Tables()
        L.gs_setup_tables(self.s, C.byref(t))

        def grab(ptr, n, dt=np.float64):
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_double)), shape=(n,)).copy().view(dt)
        d = {k: getattr(p, k) for k in PARAM_KEYS}
        lv = max(1, p.ion_levels) if p.gas else 1
        pots = np.array(list(p.ion_potentials)[:lv]) if lv > 1 else np.array([p.ionization_potential])
        d.update(n_r=nr, n_t=nt, rho0=p.rho0, raman_tau=p.raman_tau, raman_omega=p.raman_omega,
                 gas=p.gas, th_coeff=p.th_coeff, ion_levels=lv, ion_potentials=pots)
        d["rate_ln"] = grab(t.rate_ln, 8192 * lv).reshape(lv, 8192) if lv > 1 else grab(t.rate_ln, 8192)
        d["plasma_func"] = grab(t.plasma_func, 2 * nt, np.complex128)
        d["raman_func"] = grab(t.raman_func, 2 * nt, np.complex128)
        d["kerr"] = grab(t.kerr, nt)
        d["omega"] = grab(t.omega, nt)
        d["wavenum"] = grab(t.wavenum, 2 * nt, np.complex128)
        d["ho_disp"] = grab(t.ho_disp, nt)
        d["kt2"] = grab(t.kt2, nr)
        d["qdht_c"] = grab(t.qdht_c, nr * nr).reshape(nr, nr, order="F")
        d["qdht_m1"] = grab(t.qdht_m1, nr)
        f = np.empty((nr, nt), np.complex128)
        L.gs_setup_field(self.s, f.ctypes.data_as(C.c_void_p))
        d["field"] = f
        nap = C.c_int()
        L.gs_setup_apertures(self.s, C.byref(nap), None, None)
        az, ar = np.empty(nap.value), np.empty(nap.value)
        L.gs_setup_apertures(self.s, C.byref(nap), _ptr(az), _ptr(ar))
        d["aperture_z"], d["aperture_r"] = az, ar
        zn = np.empty(nz)
        dz0, rmax = C.c_double(), C.c_double()
        x = np.empty(nr)
        L.gs_setup_znet(self.s, zn.ctypes.data_as(C.c_void_p), C.byref(dz0), C.byref(rmax), x.ctypes.data_as(C.c_void_p))
        d.update(znet=zn, init_zstep=dz0.value, r_max=rmax.value, qdht_x=x)
        return d


class Batch:
    """Independent pulses (Propagator objects on one device) advanced together: with fixed
    per-pulse step sizes, one CUDA graph launch per z-step (step), or with every pulse's
    adaptive controller on the device, one graph launch per attempt (advance)."""

    def __init__(self, pulses):
        self.L = load_library()
        self.pulses = list(pulses)   # kept alive: the batch uses their handles
        arr = (C.c_void_p * len(self.pulses))(*[p.h.value for p in self.pulses])
        b = C.c_void_p()
        rc = self.L.gs_batch_create(len(self.pulses), arr, C.byref(b))
        if rc:
            raise GsError(rc, self.L.gs_batch_last_error(None).decode())
        self.b = b

    def step(self, dz, n_steps=1, graph=True):
        d = np.ascontiguousarray(dz, dtype=np.float64)
        if d.shape != (len(self.pulses),):
            raise ValueError("one step size per pulse")
        rc = self.L.gs_batch_step(self.b, int(n_steps), _ptr(d), int(bool(graph)))
        if rc:
            raise GsError(rc, self.L.gs_batch_last_error(self.b).decode())

    def advance(self, znets, n_z, current_z, zstep, step_n, max_calls):
        """gs_batch_advance: up to max_calls propagator() calls of every pulse (gs_advance for
        each, all pulses' attempts in one graph launch).  znets: one ZNET array per pulse; n_z,
        current_z, zstep, step_n: per pulse.  Returns (current_z, zstep, step_n, calls, reached)
        as arrays."""
        n = len(self.pulses)
        zs = [np.ascontiguousarray(z, dtype=np.float64) for z in znets]
        if len(zs) != n:
            raise ValueError("one ZNET per pulse")
        zp = (C.c_void_p * n)(*[z.ctypes.data for z in zs])
        nz = np.array([len(z) for z in zs], np.int32)
        nzi = np.ascontiguousarray(n_z, dtype=np.int32)
        cz = np.ascontiguousarray(current_z, dtype=np.float64).copy()
        dz = np.ascontiguousarray(zstep, dtype=np.float64).copy()
        sn = np.ascontiguousarray(step_n, dtype=np.uint32).copy()
        calls = np.zeros(n, np.int32)
        reached = np.zeros(n, np.int32)
        rc = self.L.gs_batch_advance(self.b, zp, _ptr(nz), _ptr(nzi), _ptr(cz), _ptr(dz), _ptr(sn), int(max_calls),
                                     _ptr(calls), _ptr(reached))
        if rc:
            raise GsError(rc, self.L.gs_batch_last_error(self.b).decode())
        return cz, dz, sn, calls, reached.astype(bool)

    def autotune(self, dz):
        """Default vs per-grid tuned launch shapes for the batch as a whole (gs_batch_autotune);
        returns (ms per z-step default, ms tuned, chose tuned)."""
        d = np.ascontiguousarray(dz, dtype=np.float64)
        a, b, c = C.c_double(), C.c_double(), C.c_int()
        rc = self.L.gs_batch_autotune(self.b, _ptr(d), C.byref(a), C.byref(b), C.byref(c))
        if rc:
            raise GsError(rc, self.L.gs_batch_last_error(self.b).decode())
        return a.value, b.value, bool(c.value)

    def stream_ptr(self):
        return self.L.gs_batch_stream(self.b)

    def launch_count(self):
        return self.L.gs_batch_launch_count(self.b)

    def close(self):
        if getattr(self, "b", None):
            self.L.gs_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_config(config_path: str, out_dir: str = ".", overrides: dict | None = None, precision: int = PREC_FP64,
               device: int = 0, noise_seed: int = 0, noise_sigma: float = 0.0, max_calls: int = -1) -> dict:
    """The reference's whole run (main loop + .udf dumps) on one GPU (gs_run_config)."""
    L = load_library()
    ov = overrides or {}
    keys = (C.c_char_p * max(1, len(ov)))(*[k.encode() for k in ov])
    vals = (C.c_char_p * max(1, len(ov)))(*[str(v).encode() for v in ov.values()])
    st = RunStats()
    rc = L.gs_run_config(config_path.encode(), out_dir.encode(), len(ov), keys, vals, int(precision), int(device),
                         int(noise_seed), float(noise_sigma), int(max_calls), C.byref(st))
    if rc:
        raise GsError(rc, L.gs_run_last_error().decode())
    return {k: getattr(st, k) for k, _ in RunStats._fields_}
