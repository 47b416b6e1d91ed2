"""Host-side checks that need no GPU: the C-ABI library builds for sm_103a,
loads, and exports every entry point include/brawl_gpu.h declares; calls
fail with a status (not a crash) when there is no device; input readers."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import brawl_gb300 as B
from brawl_gb300 import inputs as I
from tests import golden_io as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "brawl_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(brawl_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = B.load()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    lib = B.load()
    for n in declared_functions():
        assert getattr(lib, n).restype is not None or n == "brawl_last_error"


def test_status_without_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = B.load()
    s = B.Setup("fcc", 2, 2, 2, 2, 2).c()
    V = np.zeros((2, 2, 2))
    h = C.c_void_p()
    rc = lib.brawl_ctx_create(C.byref(s), V.ctypes.data_as(C.c_void_p), C.byref(h))
    assert rc == 3  # BRAWL_ECUDA
    assert b"device" in lib.brawl_last_error()
    with pytest.raises(B.BrawlError):
        B.Chain(B.Setup("fcc", 2, 2, 2, 2, 2), V)


def test_read_reference_inputs():
    p = I.read_control_file(G.path("01_serial_metropolis", "brawl.inp"))
    assert (p.lattice, p.n_1, p.n_2, p.n_3, p.n_species, p.interaction_range, p.wc_range) == \
        ("fcc", 4, 4, 4, 5, 6, 3)
    assert list(p.species_numbers) == [51, 51, 51, 51, 52]
    assert p.numbers_or_none() is not None and p.static_seed
    m = I.read_metropolis_file(G.path("01_serial_metropolis", "metropolis.inp"))
    assert (m.n_mc_steps, m.n_sample_steps, m.n_sample_steps_asro, m.T, m.T_steps) == (256, 1, 256, 300.0, 1)
    assert m.write_trajectory_energy and not m.nbr_swap
    p2 = I.read_control_file(G.path("02_parallel_metropolis", "brawl.inp"))
    assert p2.numbers_or_none() is None
    assert list(p2.species_concentrations) == [0.0, 0.25, 0.25, 0.25, 0.25]
    wl = I.read_wl_file(G.path("04_parallel_wang-landau", "wl_input.inp"))
    assert (wl.bins, wl.num_windows, wl.mc_sweeps) == (512, 4, 100)
    assert wl.bin_overlap == float(np.float32(0.25)) and wl.tolerance == float(np.float32(5e-5))
    ns = I.read_ns_file(G.path("03_serial_nested_sampling", "ns_input.inp"))
    assert (ns.n_walkers, ns.n_steps, ns.n_iter) == (100, 500, 1000)


def test_metropolis_input_quirk(tmp_path):
    """n_sample_steps_asro is reset to n_sample_steps when n_sample_steps_alro
    is zero (the reference tests the wrong variable, src/io.f90:654-656)."""
    f = tmp_path / "metropolis.inp"
    f.write_text("mode=simulated_annealing\nn_mc_steps=100\nn_sample_steps=10\n"
                 "n_sample_steps_asro=50\nT=300\n")
    m = I.read_metropolis_file(str(f))
    assert m.n_sample_steps_asro == 10 and m.n_sample_steps_alro == 10
    f.write_text("mode=simulated_annealing\nn_mc_steps=100\nn_sample_steps=10\n"
                 "n_sample_steps_asro=50\nn_sample_steps_alro=20\nT=300\nburn_in=T\n")
    m = I.read_metropolis_file(str(f))
    assert m.n_sample_steps_asro == 50 and m.burn_in_start


def test_exchange_is_column_major():
    p, V = G.load_inputs("02_parallel_metropolis")
    raw = open(G.path("02_parallel_metropolis", p.interaction_file)).read().split()
    assert V[1, 0, 0] == float(raw[1]) and V[0, 1, 0] == float(raw[4])
    assert V.shape == (4, 4, 6)
