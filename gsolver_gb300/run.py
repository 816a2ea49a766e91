"""Command-line run of a reference-format config on one GPU, writing the .udf dumps:

    python -m gsolver_gb300.run CONFIG [KEY value ...] [--out DIR] [--mixed] [--device N]

the counterpart of ``mpirun -np N ./gsolver_solid_qdht CONFIG [KEY value ...]`` (the
trailing KEY value pairs override the config, as in process_input.cpp:297-482).
"""
import argparse
import json
import sys

import gsolver_gb300 as gs


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("config")
    ap.add_argument("pairs", nargs="*")
    ap.add_argument("--out", default=".")
    ap.add_argument("--mixed", action="store_true")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--max-calls", type=int, default=-1)
    a = ap.parse_args(argv)
    if len(a.pairs) % 2:
        ap.error("overrides come in KEY value pairs")
    ov = dict(zip(a.pairs[0::2], a.pairs[1::2]))
    st = gs.run_config(a.config, a.out, ov, gs.PREC_MIXED if a.mixed else gs.PREC_FP64, a.device,
                       max_calls=a.max_calls)
    print(json.dumps(st))


if __name__ == "__main__":
    sys.exit(main())
