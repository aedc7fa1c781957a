"""Regenerate the committed golden fixtures from the reference implementation itself.

Runs oracle/_ref/ref_driver (the reference's own Contract / ContractContiguousAxes /
ContractTailHeadContiguousAccumulate / SVD / QR, built from the
reference sources by oracle/ref/Makefile) on inputs from the deterministic workload
generator and stores inputs, task lists and outputs as compressed .npz files here.

    make -C oracle/ref && python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle.oracle import read_qtb  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")

# name -> (driver args, parity component of the QN type: -1 bosonic U1QN, 0 fermionic fU1U1QN)
CASES = {
    "cfg1": (["cfg1"], -1),
    "matvec_u1_small": (["matvec_u1", "4", "2.0", "40", "1"], -1),
    "matvec_f_small": (["matvec_f", "2", "24", "4"], 0),
    "ctrct_misc_u1": (["ctrct_misc", "7"], None),
    "ctrct_contig": (["ctrct_contig", "11"], None),
    # also writes tests/golden/qlten/<tag>.qlten with the reference's stream operator
    "qlten_io": (["qlten_io", "5", "{qlten_dir}"], None),
    "axis_ops": (["axis_ops", "3"], -1),
    "svd_u1_full": (["svd_u1", "4", "2.0", "40", "3", "1e-9", "1", "1000"], -1),
    "svd_u1_trunc": (["svd_u1", "4", "2.0", "40", "3", "1e-2", "1", "1000"], -1),
    "svd_u1_dmax": (["svd_u1", "4", "2.0", "40", "3", "1e-12", "1", "12"], -1),
    "svd_u1_dmin": (["svd_u1", "4", "2.0", "40", "3", "0.5", "20", "30"], -1),
    "svd_stress_small": (["svd_stress", "6", "3", "20", "3", "1e-3", "1", "40"], -1),
    "svd_f": (["svd_f", "2", "24", "4", "1e-3", "1", "30"], 0),
    "qr_u1": (["qr_u1", "4", "2.0", "40", "5"], -1),
    "qr_f": (["qr_f", "2", "24", "6"], 0),
}


def parity_for(name, key, default):
    if default is not None:
        return default
    return 0 if key.startswith("f_") else -1   # ctrct_misc / ctrct_contig: f_* cases are fermionic


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference driver first: make -C oracle/ref")
    only = set(sys.argv[1:])   # optional: regenerate only the named fixtures
    for name, (args, pc) in CASES.items():
        if only and name not in only:
            continue
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "out.qtb")
            qdir = os.path.join(HERE, "qlten")
            os.makedirs(qdir, exist_ok=True)
            run_args = [a.replace("{qlten_dir}", qdir) for a in args]
            subprocess.check_call([DRIVER, run_args[0], path] + run_args[1:])
            rec = read_qtb(path)
        prefixes = sorted({k.rsplit(".", 1)[0] for k in rec if k.endswith(".dirs")})
        for p in prefixes:
            rec[p + ".parity_comp"] = np.array([parity_for(name, p, pc)], np.int64)
        rec["__args__"] = np.array(" ".join(args))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
        print(name, os.path.getsize(os.path.join(HERE, name + ".npz")), "bytes")


if __name__ == "__main__":
    main()
