"""Regenerate the golden fixtures under tests/golden/ from the reference's
own regression tests (tests/0*/ inputs and tests/99_ref/ outputs of the
BraWl repository).

Run in a container that has the reference checked out:

    python tests/golden/make_golden.py [/path/to/BraWl]

Inputs (*.inp, *.vij) are copied verbatim; text outputs (*.dat, *.energies)
are stored gzip-compressed byte-for-byte; netCDF outputs are converted to
.npz with the variables' data (the reference's comparator, tests/ci_test.py,
compares variable data only).
"""
from __future__ import annotations

import gzip
import os
import shutil
import sys

import numpy as np
from scipy.io import netcdf_file

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = ["01_serial_metropolis", "02_parallel_metropolis", "03_serial_nested_sampling",
         "04_parallel_wang-landau"]


def main(ref_root: str) -> None:
    for t in TESTS:
        src_in = os.path.join(ref_root, "tests", t)
        src_out = os.path.join(ref_root, "tests", "99_ref", t)
        dst = os.path.join(HERE, t)
        os.makedirs(dst, exist_ok=True)
        for f in sorted(os.listdir(src_in)):
            if f.endswith((".inp", ".vij")):
                shutil.copyfile(os.path.join(src_in, f), os.path.join(dst, f))
        for f in sorted(os.listdir(src_out)):
            p = os.path.join(src_out, f)
            if f.endswith((".dat", ".energies")):
                with open(p, "rb") as fi, gzip.GzipFile(os.path.join(dst, f + ".gz"), "wb", mtime=0) as fo:
                    fo.write(fi.read())
            elif f.endswith(".nc"):
                d = netcdf_file(p, "r", mmap=False)
                arrays = {k.replace(" ", "_"): np.array(v.data) for k, v in d.variables.items()}
                d.close()
                np.savez_compressed(os.path.join(dst, f[:-3] + ".npz"), **arrays)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
