"""Generate golden vectors from the reference solver itself (oracle/_ref, built from the
reference checkout by oracle/Makefile.ref) for the GPU parity tests.

Run once in a container where the reference checkout exists:

    python tests/golden/make_ref_golden.py REFERENCE_CHECKOUT

It builds the reference binaries, then for each case writes the config text, the seeded start
field and the reference's outputs on it:
  ref_hot_solid.npz   fused silica, 16 x 1024, a tightly focused 20 P_cr pulse (Keldysh,
                      avalanche, loss and plasma defocusing all act): calculate_NLstep at the
                      first step size, the on-axis carrier density, and ten propagator() calls
                      through the reference's z-loop (gsolver_solid_qdht build)
  ref_argon_gas.npz   argon at 3.9 um, 8 x 2048, 6 P_cr (gsolver_gas_qdht build: PPT rates,
                      neutral depletion, third harmonic), with one ionization level and with
                      two (IONIZATION_LEVEL_N 2): calculate_NLstep and three propagator() calls
The start fields come from the oracle's seeded set-up (numpy PCG64), so the fixtures are
reproducible; the configs' dispersion tables are regenerated by gsolver_gb300.configs.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gsolver_gb300 import configs  # noqa: E402
from oracle import ref, tables  # noqa: E402

TWO_LEVELS = "IONIZATION_LEVEL_N 2\nIONIZATION_POTENTIAL1 15.76\nIONIZATION_POTENTIAL2 27.63\n"


def _text(p):
    with open(p) as f:
        return np.frombuffer(f.read().encode(), dtype=np.uint8)


def hot_solid():
    d = tempfile.mkdtemp(prefix="gs_refgold_")
    p = configs.hot_solid(d, n_r=16, n_t=1024, power_cr=20.0, tol=1e-2)
    T = tables.build(tables.Config.from_file(p), noise_seed=7, noise_sigma=1e-4)
    f = T["field"]
    R = ref.Reference(p)
    t = R.tables()
    run = R.run(f, 10)
    dz0 = run["init_zstep"]
    bb1, a2, n2 = R.nl_step(f, dz0)
    rho, _ = R.plasma(np.fft.ifft(f[0]))
    out = {"config": _text(p), "field0": f, "dz0": dz0, "bb1": bb1, "max_a2": a2, "max_nl2": n2,
           "rho_axis": rho, "steps": 10, "field": run["field"], "bb2": run["bb2"], "zstep": run["zstep"],
           "step_n": run["step_n"], "z": run["z"], "rate_ln": t["rate_ln"]}
    np.savez_compressed(os.path.join(HERE, "ref_hot_solid.npz"), **out)
    print("ref_hot_solid.npz: rho max %.3e, step_n %d" % (rho.max(), run["step_n"]))


def argon_gas():
    out = {}
    for levels in (1, 2):
        d = tempfile.mkdtemp(prefix="gs_refgold_ar_")
        p = configs.argon_c5(d, n_r=8, n_t=2048, build="gas_qdht", power_cr=6.0, w0=9e-4, r_max=3.6e-3)
        if levels == 2:
            with open(p, "a") as fh:
                fh.write(TWO_LEVELS)
        T = tables.build(tables.Config.from_file(p), noise_seed=1, noise_sigma=1e-4)
        f = T["field"]
        R = ref.Reference(p, build="gas")
        run = R.run(f, 3)
        bb1, a2, n2 = R.nl_step(f, run["init_zstep"])
        k = f"l{levels}_"
        out.update({k + "config": _text(p), k + "dz0": run["init_zstep"], k + "bb1": bb1, k + "max_a2": a2,
                    k + "max_nl2": n2, k + "field": run["field"], k + "bb2": run["bb2"], k + "zstep": run["zstep"],
                    k + "step_n": run["step_n"]})
        out["field0"] = f   # the same seeded start field for both
    np.savez_compressed(os.path.join(HERE, "ref_argon_gas.npz"), **out)
    print("ref_argon_gas.npz")


def main(reference):
    if not ref.build(reference):
        sys.exit("could not build the reference solver from " + reference)
    hot_solid()
    argon_gas()


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_ref_golden.py REFERENCE_CHECKOUT")
    main(sys.argv[1])
