"""The netCDF writer and reader against the reference's own output files
(tests/99_ref of the reference, kept verbatim under tests/golden/netcdf/):
the same data and attributes give the same bytes, and the readers apply the
reference's checks (src/netcdf_io.f90:1368-1516)."""
from __future__ import annotations

import copy
import os

import numpy as np
import pytest

from brawl_gb300 import inputs as I
from brawl_gb300 import netcdf_io as N
from oracle import oracle as O

from . import golden_io as G

RAW = os.path.join(G.GOLDEN, "netcdf")
TESTS = {"01": "01_serial_metropolis", "02": "02_parallel_metropolis", "04": "04_parallel_wang-landau"}


def _raw(name: str) -> bytes:
    with open(os.path.join(RAW, name), "rb") as f:
        return f.read()


def _params(prefix: str):
    p = I.read_control_file(G.path(TESTS[prefix], "brawl.inp"))
    if prefix == "01":
        # Test 01 gives species_numbers (51 51 51 51 52).  Its stored files
        # carry Concentrations 0.2 each, from an earlier build of the
        # reference; the current initial_setup writes 51/256 and so on
        # (src/initialise.F90:471).  The attribute is taken from the file.
        p.species_concentrations = np.array([0.0, 0.2, 0.2, 0.2, 0.2, 0.2])
    return p


@pytest.mark.parametrize("name", ["01_proc_0000_final_config_at_0300.0.nc",
                                  "02_proc_0002_initial_config_at_0300.0.nc"])
def test_config_writer_matches_reference_bytes(tmp_path, name):
    prefix, rest = name[:2], name[3:]
    p = _params(prefix)
    cfg = G.config_zyx(TESTS[prefix], rest[:-3] + ".npz")
    out = tmp_path / "c.nc"
    N.write_config(str(out), cfg, p)
    assert out.read_bytes() == _raw(name)
    assert np.array_equal(N.read_config(str(out), p), cfg)


@pytest.mark.parametrize("name", ["01_proc_0000_rho_of_T.nc", "02_av_radial_density.nc"])
def test_radial_density_writer_matches_reference_bytes(tmp_path, name):
    prefix, rest = name[:2], name[3:]
    p = _params(prefix)
    ref = G.npz(TESTS[prefix], rest[:-3] + ".npz")
    out = tmp_path / "r.nc"
    N.write_radial_density(str(out), ref["rho_data"], ref["r_data"], ref["T_data"], ref["U_data"], p)
    assert out.read_bytes() == _raw(name)
    rho, U = N.read_radial_density(str(out), p, n_steps=ref["T_data"].size)
    assert np.array_equal(rho, ref["rho_data"]) and np.array_equal(U, ref["U_data"])


def test_dos_writer_matches_reference_bytes(tmp_path):
    ref = G.npz(TESTS["04"], "wl_dos.npz")["grid_data"]
    out = tmp_path / "d.nc"
    N.write_grid_1d(str(out), ref)
    assert out.read_bytes() == _raw("04_wl_dos.nc")
    d = N.read_file(str(out))
    assert d["dims"] == {"x": ref.size} and np.array_equal(d["vars"]["grid data"][1], ref)


def test_read_file_structure():
    d = N.read_file(os.path.join(RAW, "01_proc_0000_rho_of_T.nc"))
    assert d["dims"] == {"i": 5, "j": 5, "r": 3, "T": 1, "r_i": 3, "T_i": 1, "U_i": 1}
    assert d["attrs"]["Lattice Type"] == "fcc" and d["attrs"]["Interaction file"] == "fcc_epi.vij"
    assert int(d["attrs"]["Warren-Cowley Range"][0]) == 3
    assert d["vars"]["rho data"][0] == ("T", "r", "j", "i")


def test_reader_checks_like_the_reference():
    name = os.path.join(RAW, "02_proc_0002_initial_config_at_0300.0.nc")
    p = _params("02")
    for field, value, msg in (("n_1", 5, "n_1 values"), ("n_basis", 2, "n_basis values"),
                              ("lattice", "fcc", "Lattice types")):
        q = copy.deepcopy(p)
        setattr(q, field, value)
        with pytest.raises(ValueError, match=msg + " do not match in ncdf_config_reader"):
            N.read_config(name, q)
    q = copy.deepcopy(p)
    q.wc_range = p.wc_range + 1
    with pytest.raises(ValueError, match="wc_range values do not match"):
        N.read_radial_density(os.path.join(RAW, "02_av_radial_density.nc"), q, n_steps=1)
    with pytest.raises(ValueError, match="n_steps values do not match"):
        N.read_radial_density(os.path.join(RAW, "02_av_radial_density.nc"), p, n_steps=2)


def test_oracle_run_written_byte_for_byte(tmp_path):
    """Rank 2 of test 02 from the inputs alone: initial_setup on the oracle,
    then the file writer, gives the reference's file."""
    p, V = G.load_inputs(TESTS["02"])
    mod = O.OracleModel(p.lattice, p.n_1, p.n_2, p.n_3, V)
    rng = O.OracleRng(O.lib().bo_static_seed(2))
    cfg, _ = mod.initial_setup(rng, p.species_concentrations, p.numbers_or_none())
    out = tmp_path / "init.nc"
    N.write_config(str(out), cfg, p)
    assert out.read_bytes() == _raw("02_proc_0002_initial_config_at_0300.0.nc")


def test_order_writer_reads_back_with_scipy(tmp_path):
    """ncdf_order_writer's layout, checked with scipy's independent reader."""
    from scipy.io import netcdf_file
    p = _params("02")
    rng = np.random.default_rng(4)
    order = rng.uniform(0, 1, (3, 8, 8, 8, 1, p.n_species))
    T = np.array([300.0, 250.0, 200.0])
    out = tmp_path / "alro.nc"
    N.write_order(str(out), order, T, p)
    f = netcdf_file(str(out), "r", mmap=False)
    assert f.dimensions == {"b": p.n_species, "x": 1, "y": 8, "z": 8, "s": 8, "t": 3, "temp": 3}
    assert f.variables["grid data"].dimensions == ("t", "s", "z", "y", "x", "b")
    assert np.array_equal(np.array(f.variables["grid data"].data), order)
    assert np.array_equal(np.array(f.variables["temperature data"].data), T)
    assert int(f.N_Basis) == 1 and f._attributes["Lattice Type"] == b"bcc"
    f.close()
