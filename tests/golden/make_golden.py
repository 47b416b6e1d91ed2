"""Regenerate the golden fixtures under tests/golden/ from the reference's
own regression tests (tests/0*/ inputs and tests/99_ref/ outputs of the
BraWl repository).

Run in a container that has the reference checked out:

    python tests/golden/make_golden.py [/path/to/BraWl]

Inputs (*.inp, *.vij) are copied verbatim; text outputs (*.dat, *.energies)
are stored gzip-compressed byte-for-byte; netCDF outputs are converted to
.npz with the variables' data (the reference's comparator, tests/ci_test.py,
compares variable data only), and a few are also kept verbatim under
netcdf/ for the file writer's byte-for-byte tests.
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
# netCDF outputs also kept verbatim, one of each kind the sampling path
# writes, for byte-for-byte checks of the file writer
RAW_NC = [("01_serial_metropolis", "proc_0000_final_config_at_0300.0.nc"),
          ("01_serial_metropolis", "proc_0000_rho_of_T.nc"),
          ("02_parallel_metropolis", "proc_0002_initial_config_at_0300.0.nc"),
          ("02_parallel_metropolis", "av_radial_density.nc"),
          ("04_parallel_wang-landau", "wl_dos.nc")]


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
    raw = os.path.join(HERE, "netcdf")
    os.makedirs(raw, exist_ok=True)
    for t, f in RAW_NC:
        shutil.copyfile(os.path.join(ref_root, "tests", "99_ref", t, f), os.path.join(raw, t[:2] + "_" + f))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    # the reference checkout: the first argument, else $BRAWL_REFERENCE_DIR
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BRAWL_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout>  (or set BRAWL_REFERENCE_DIR)")
    main(ref)
