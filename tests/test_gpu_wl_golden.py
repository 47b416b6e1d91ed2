"""Wang-Landau against the reference's own stored result: the full driver
(brawl_gb300.wang_landau: energy bins, windows and overlaps, main loop with
replica exchange, flatness, ln f halving, dos_average and dos_combine) on
the inputs of tests/04_parallel_wang-landau, to the same tolerance, and the
reference's own acceptance test (wl_test.py there): NRMSE of ln g below 1%.
The walk itself is pinned to the oracle trial by trial elsewhere; this
checks the assembled method end to end."""
import os

import numpy as np
import pytest

import brawl_gb300 as B
from brawl_gb300 import inputs as I, wang_landau as WLD

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden", "04_parallel_wang-landau")


@pytest.mark.parametrize("burn_in", ["temperature", "reference"])
def test_wang_landau_reproduces_the_reference_dos(burn_in):
    """burn_in "reference" enters the windows with enter_energy_window on
    the device and pre-samples, with the radial-density samples on, the
    per-bin configuration store, merge_configs, load_window_config at every
    ln f step and mpi_window_optimise (wl_input leaves performance at 0, so
    the reference's run resized its windows too); "temperature" enters with
    the temperature search and keeps the windows."""
    p = I.read_control_file(os.path.join(G, "brawl.inp"))
    wl = I.read_wl_file(os.path.join(G, "wl_input.inp"))
    V = I.read_exchange(os.path.join(G, "bcc_epi.vij"), p.n_species, p.interaction_range)
    setup = B.Setup.from_run_params(p)
    conc = np.asarray(p.species_concentrations, dtype=np.float64)
    radial = None
    if burn_in == "reference":
        # the run's radial-density samples too (wl_input radial_samples, wc_range)
        radial = dict(wc_range=p.wc_range, shells=B.Chain(setup, V).lattice_shells(p.wc_range),
                      radial_samples=wl.radial_samples)
    out = WLD.wang_landau(setup, V, conc, wl, burn_in=burn_in, numbers=p.numbers_or_none(), radial=radial,
                          pre_sample=burn_in == "reference")
    ver = np.load(os.path.join(G, "wl_dos.npz"))["grid_data"]
    run = out["lng"]
    assert out["window_sets"][0] == [[1, 128], [97, 256], [217, 384], [343, 512]]
    for ws in out["window_sets"]:        # every set covers the bins with overlaps
        assert ws[0][0] == 1 and ws[-1][1] == 512
        assert all(ws[i][0] <= ws[i - 1][1] and ws[i][1] > ws[i - 1][1] for i in range(1, len(ws)))
    assert len(out["window_sets"]) == (1 if burn_in == "temperature" else len(out["record"]) + 2)
    nrmse = np.sqrt(np.mean((ver - run) ** 2)) / np.mean(ver)
    assert nrmse < 0.01, nrmse
    if radial is not None:
        assert out["radial_min"] > 0.0
