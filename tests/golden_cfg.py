"""Helpers that turn the committed golden fixture into a runnable config."""
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "fil_SiO2_1d.npz")


def load_golden():
    return np.load(GOLDEN)


def write_rawdisp(path, omega, n, typ=3):
    with open(path, "wb") as f:
        f.write(np.array([typ, len(omega)], dtype=np.int32).tobytes())
        f.write(np.ascontiguousarray(omega, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(n, dtype=np.float64).tobytes())


def golden_config_dir():
    """Directory holding fil_SiO2_1d.txt and SiO2.rawdisp rebuilt from the fixture."""
    g = load_golden()
    d = tempfile.mkdtemp(prefix="gs_golden_")
    write_rawdisp(os.path.join(d, "SiO2.rawdisp"), g["disp_omega"], g["disp_n"])
    with open(os.path.join(d, "fil_SiO2_1d.txt"), "w") as f:
        f.write(bytes(g["config"]).decode())
    return d
