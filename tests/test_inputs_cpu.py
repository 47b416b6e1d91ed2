"""The input readers (brawl_gb300/inputs.py) against the reference's read
rules (src/io.f90): label = everything before the first '=' with trailing
blanks dropped (leading blanks leave it unmatched), lines without '='
ignored, Fortran-style values (d exponents, .true./T, quoted strings,
comma or blank separated lists), the metropolis reader's reset of
n_sample_steps_asro when n_sample_steps_alro is zero (:654-656), the
single-precision reals of wl_input, the column-major V_ex fill (:389-402),
and the missing-label stops as exceptions."""
from __future__ import annotations

import numpy as np
import pytest

from brawl_gb300 import inputs as I

from . import golden_io as G


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_golden_inputs_read_as_written():
    p = I.read_control_file(G.path("01_serial_metropolis", "brawl.inp"))
    assert (p.mode, p.lattice, p.n_1, p.n_2, p.n_3, p.n_species) == (301, "fcc", 4, 4, 4, 5)
    assert p.lattice_parameter == 3.568 and p.interaction_range == 6 and p.wc_range == 3
    assert p.interaction_file == "fcc_epi.vij" and p.static_seed is True
    assert p.species_names == ["A", "B", "C", "D", "E"]
    assert list(p.species_numbers) == [51, 51, 51, 51, 52] and p.n_atoms == 256
    assert np.array_equal(p.numbers_or_none(), p.species_numbers)
    m = I.read_metropolis_file(G.path("01_serial_metropolis", "metropolis.inp"))
    assert m.mode == "simulated_annealing" and m.n_mc_steps == 256 and m.n_sample_steps == 1
    assert m.calculate_energies and m.calculate_asro and not m.burn_in
    ns = I.read_ns_file(G.path("03_serial_nested_sampling", "ns_input.inp"))
    assert (ns.n_walkers, ns.n_steps, ns.n_iter, ns.traj_freq) == (100, 500, 1000, 100)
    assert ns.outfile_ener == "fcc_al_1.00_crfeconi_K100.energies"
    wl = I.read_wl_file(G.path("04_parallel_wang-landau", "wl_input.inp"))
    assert (wl.mc_sweeps, wl.bins, wl.num_windows, wl.radial_samples, wl.performance) == (100, 512, 4, 8, 0)
    assert wl.flatness == float(np.float32(0.90)) and wl.bin_overlap == float(np.float32(0.25))
    assert wl.tolerance == float(np.float32(5e-5)) and wl.energy_min == -96.0


CONTROL = """# comment line without an equals sign
mode=301
lattice = bcc
lattice_parameter = 2.87d0
n_1 = 3
n_2=4
 n_3 = 9
n_3 = 5
n_species = 3
species_names = Fe, Cr  Ni
species_concentrations = 0.5d0, 0.25 0.25
interaction_range = 2
interaction_file = "V.vij"  ! trailing text
static_seed = T
"""


def test_control_file_rules(tmp_path):
    p = I.read_control_file(_write(tmp_path, "brawl.inp", CONTROL))
    assert p.lattice == "bcc" and p.lattice_parameter == 2.87
    assert (p.n_1, p.n_2, p.n_3) == (3, 4, 5)            # " n_3" (leading blank) is not the label
    assert p.species_names == ["Fe", "Cr", "Ni"]
    assert list(p.species_concentrations) == [0.0, 0.5, 0.25, 0.25]
    assert p.interaction_file == "V.vij" and p.static_seed is True
    assert p.numbers_or_none() is None                     # species_numbers absent
    with pytest.raises(ValueError, match="Missing 'mode' in system file"):
        I.read_control_file(_write(tmp_path, "b2.inp", CONTROL.replace("mode=301", "")))
    with pytest.raises(FileNotFoundError):
        I.read_control_file(str(tmp_path / "absent.inp"))


METRO = """mode = simulated_annealing
n_mc_steps = 1000
n_sample_steps = 10
n_sample_steps_asro = 50
burn_in = .true.
T = 1.5d3
delta_T = -100
T_steps = 4
nbr_swap = F
"""


def test_metropolis_file_rules(tmp_path):
    m = I.read_metropolis_file(_write(tmp_path, "m.inp", METRO))
    assert m.T == 1500.0 and m.delta_T == -100.0 and m.T_steps == 4
    # n_sample_steps_alro = 0 resets n_sample_steps_asro too (src/io.f90:654-656)
    assert m.n_sample_steps_asro == 10 and m.n_sample_steps_alro == 10
    assert m.n_sample_steps_trajectory == 10
    assert m.burn_in and m.burn_in_start                   # burn_in implies burn_in_start
    m2 = I.read_metropolis_file(_write(tmp_path, "m2.inp", METRO + "n_sample_steps_alro = 20\n"))
    assert m2.n_sample_steps_asro == 50 and m2.n_sample_steps_alro == 20
    with pytest.raises(ValueError, match="Missing 'T' in Metropolis input file"):
        I.read_metropolis_file(_write(tmp_path, "m3.inp", METRO.replace("T = 1.5d3\n", "")))


def test_exchange_file_fills_column_major(tmp_path):
    text = "1 2 3 4\n5.0d0, 6 7 8\n"
    V = I.read_exchange(_write(tmp_path, "v.vij", text), 2, 2)
    assert V.shape == (2, 2, 2)
    assert V[1, 0, 0] == 2.0 and V[0, 1, 0] == 3.0 and V[0, 0, 1] == 5.0 and V[1, 1, 1] == 8.0
    with pytest.raises(ValueError, match="expected 8 values"):
        I.read_exchange(_write(tmp_path, "short.vij", "1 2 3"), 2, 2)


def test_lattice_codes():
    assert [I.lattice_id(x) for x in ("simple_cubic", "bcc", "fcc")] == [0, 1, 2]
    with pytest.raises(ValueError, match="not yet implemented"):
        I.lattice_id("hcp")
