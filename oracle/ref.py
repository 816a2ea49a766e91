"""Runs the reference solver itself, built in oracle/_ref by oracle/Makefile.ref (TEST
INFRASTRUCTURE).

Only tests/ (the oracle-against-reference checks) and tests/golden/make_ref_golden.py use this
module.  The binaries are the reference's own sources compiled against this project's
stand-ins for MPI, FFTW3 and GSL (oracle/ref_shim) with a command-line driver
(oracle/ref_harness.cpp); each call runs one process in the config's directory, so the
reference's global state starts fresh every time.  The reference checkout is needed only to
build them: where it is absent (and on machines the binaries were not built for) ``available()``
is False and the checks that need it are skipped.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# where the reference checkout lies in the container this project is developed in; the build
# reads its sources there, in place
DEFAULT_REFERENCE = "/root/reference"


def binary(build: str = "solid") -> str:
    return os.path.join(OUT, f"gsref_{build}")


def build(reference: str | None = None) -> bool:
    """Build both reference binaries if the checkout is present; True when they exist."""
    ref = reference or os.environ.get("GSOLVER_REFERENCE", DEFAULT_REFERENCE)
    if os.path.isfile(os.path.join(ref, "propagator.cu")):
        subprocess.run(["make", "-s", "-j8", "-f", os.path.join(HERE, "Makefile.ref"), f"REF={ref}"], check=True,
                       capture_output=True)
    return available()


def available() -> bool:
    for b in ("solid", "gas"):
        p = binary(b)
        if not os.access(p, os.X_OK):
            return False
    try:   # built for this machine?
        r = subprocess.run([binary("solid")], capture_output=True, timeout=30)
    except OSError:
        return False
    return r.returncode == 2


def read_records(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        b = f.read()
    o = 0
    while o < len(b):
        (nl,) = struct.unpack_from("<i", b, o)
        o += 4
        name = b[o:o + nl].decode()
        o += nl
        kind, count = struct.unpack_from("<iq", b, o)
        o += 12
        dt = np.complex128 if kind else np.float64
        a = np.frombuffer(b, dtype=dt, count=count, offset=o).copy()
        o += count * (16 if kind else 8)
        out[name] = a[0].item() if count == 1 and not kind else a
    return out


class RefError(RuntimeError):
    pass


class Reference:
    """The reference solver on one config (the reference's own start-up every call)."""

    def __init__(self, config_path: str, build: str = "solid", overrides: dict | None = None):
        self.cfg = os.path.abspath(config_path)
        self.build = build
        self.overrides = overrides or {}
        self._t = None

    def _call(self, mode, arrays=(), extra=()):
        d = os.path.dirname(self.cfg)
        with tempfile.TemporaryDirectory(prefix="gsref_") as tmp:
            ins = []
            for i, a in enumerate(arrays):
                p = os.path.join(tmp, f"in{i}.bin")
                np.ascontiguousarray(a, dtype=np.complex128).tofile(p)
                ins.append(p)
            outp = os.path.join(tmp, "out.bin")
            ov = [str(x) for kv in self.overrides.items() for x in kv]
            cmd = [binary(self.build), self.cfg] + ov + ["--", mode] + ins + [outp] + [str(x) for x in extra]
            r = subprocess.run(cmd, cwd=d, capture_output=True, text=True)
            if r.returncode != 0:
                raise RefError(f"reference {mode} failed ({r.returncode}): {r.stderr.strip()[-400:]}")
            return read_records(outp)

    def tables(self) -> dict:
        if self._t is None:
            t = self._call("tables")
            nr, nt = int(t["n_r"]), int(t["n_t"])
            t["field"] = t["field"].reshape(nr, nt)
            t["bb2"] = t["bb2"].reshape(nr, nt)
            self._t = t
        return self._t

    def _shape(self):
        t = self.tables()
        return int(t["n_r"]), int(t["n_t"])

    def run(self, field, steps=-1, dz0=None) -> dict:
        """process_input's restart from `field` and `steps` propagator() calls (-1: to the last
        ZNET point); returns the final FIELD, BIGBUFFER2, z, ZSTEP, STEP_N, n_Z."""
        extra = [int(steps)] + ([repr(float(dz0))] if dz0 is not None else [])
        r = self._call("run", [field], extra)
        nr, nt = self._shape()
        r["field"] = r["field"].reshape(nr, nt)
        r["bb2"] = r["bb2"].reshape(nr, nt)
        return r

    def nl_step(self, field, dz):
        r = self._call("nlstep", [field], [repr(float(dz))])
        return r["bb1"].reshape(self._shape()), r["max_a2"], r["max_nl2"]

    def nl_response(self, row):
        return self._call("nlresponse", [row])["nl"]

    def plasma(self, e_row):
        r = self._call("plasma", [e_row])
        return r["rho"], r["loss"]

    def qdht(self, data):
        return self._call("qdht", [data])["y"].reshape(self._shape())
