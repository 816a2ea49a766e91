"""Generate the committed golden fixtures from the reference's own committed outputs.

Run once in a container where the reference checkout exists:

    python tests/golden/make_golden.py /path/to/reference

It reads, without modifying anything:
  bin/fil_SiO2_1d.txt              the config of the golden run
  bin/SiO2.rawdisp                 the RAW dispersion table it uses
  bin/fil_SiO2__{f,fa,mI,pm,s}.udf the reference's dumps of that run (N_R=512, N_T=512, N_Z=128)
  bin/omega.bin, bin/wavenum.bin   omega grid and k(omega) written by load_info
                                   (process_input.cpp:118-119) for the same N_T=512 grid
and writes tests/golden/fil_SiO2_1d.npz holding the config text, the dispersion table,
omega/k and a subset of z-slabs of every dump (every 16th slab and the last one).
"""
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_udf(path):
    with open(path, "rb") as f:
        b = f.read()
    assert b[:7] == b"UDF1.0\x00", path
    fsize, iscomplex, tN, xN, yN, zN = struct.unpack("6i", b[7:31])
    assert fsize == 8
    a = np.frombuffer(b, dtype=np.complex128 if iscomplex else np.float64, offset=31)
    return a.reshape(zN, -1), (iscomplex, tN, xN, yN, zN)


def main(ref):
    b = os.path.join(ref, "bin")
    with open(os.path.join(b, "fil_SiO2_1d.txt")) as f:
        cfg = f.read()
    with open(os.path.join(b, "SiO2.rawdisp"), "rb") as f:
        raw = f.read()
    typ, n = struct.unpack("ii", raw[:8])
    pw = np.frombuffer(raw, np.float64, n, 8)
    pn = np.frombuffer(raw, np.float64, 2 * n, 8 + 8 * n)
    out = {"config": np.frombuffer(cfg.encode(), dtype=np.uint8), "disp_omega": pw, "disp_n": pn,
           "disp_type": np.array([typ], dtype=np.int32)}
    out["omega_bin"] = np.fromfile(os.path.join(b, "omega.bin"), dtype=np.float64)
    out["wavenum_bin"] = np.fromfile(os.path.join(b, "wavenum.bin"), dtype=np.complex128)
    slabs = None
    for key in ("f", "fa", "mI", "pm", "s"):
        a, hdr = read_udf(os.path.join(b, f"fil_SiO2__{key}.udf"))
        zN = hdr[4]
        if slabs is None:
            slabs = np.array(sorted(set(list(range(0, zN, 16)) + [zN - 1])), dtype=np.int32)
        out["udf_" + key] = a[slabs]
        out["hdr_" + key] = np.array(hdr, dtype=np.int32)
    out["slabs"] = slabs
    np.savez_compressed(os.path.join(HERE, "fil_SiO2_1d.npz"), **out)
    print("wrote", os.path.join(HERE, "fil_SiO2_1d.npz"), "slabs", slabs.tolist())


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_CHECKOUT")
    main(sys.argv[1])
