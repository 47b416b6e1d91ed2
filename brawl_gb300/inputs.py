"""Readers for BraWl's key=value input files and interaction files.

The files are read exactly as the reference reads them, so existing inputs
work unchanged:

* ``brawl.inp``      -- read_control_file (src/io.f90:135-330)
* ``metropolis.inp`` -- read_metropolis_file (src/io.f90:519-686), including
  its reset of n_sample_steps_asro when n_sample_steps_alro is zero
  (src/io.f90:654-656)
* ``ns_input.inp``   -- read_ns_file (src/io.f90:740-817)
* ``wl_input.inp``   -- read_wl_file (src/io.f90:951-1086)
* ``*.vij``          -- read_exchange (src/io.f90:389-402): one list-directed
  read of all values into V_ex(n_species, n_species, interaction_range),
  column-major, in Ry.

A line is ``label=value``; the label is everything before the first '='
with trailing blanks ignored (leading blanks make it unmatched, as in the
reference), and lines without '=' are ignored.
"""
from __future__ import annotations

import dataclasses
import os
import re

import numpy as np


def _split(line: str):
    pos = line.find("=")
    if pos < 0:
        return None, None
    return line[:pos].rstrip(), line[pos + 1:]


def _first_token(value: str) -> str:
    v = value.strip()
    if not v:
        raise ValueError("empty value")
    if v[0] in "'\"":
        q = v[0]
        end = v.find(q, 1)
        return v[1:end] if end > 0 else v[1:]
    return re.split(r"[\s,]+", v)[0]


def _fortran_int(value: str) -> int:
    return int(_first_token(value))


def _fortran_real(value: str) -> float:
    tok = _first_token(value).lower().replace("d", "e")
    return float(tok)


def _fortran_logical(value: str) -> bool:
    tok = _first_token(value).lstrip(".").lower()
    if tok.startswith("t"):
        return True
    if tok.startswith("f"):
        return False
    raise ValueError(f"not a logical: {value!r}")


def _fortran_list(value: str, conv, n: int):
    toks = [t for t in re.split(r"[\s,]+", value.strip()) if t]
    if len(toks) < n:
        raise ValueError(f"expected {n} values, got {len(toks)}")
    return [conv(t) for t in toks[:n]]


def _f32(x: float) -> float:
    return float(np.float32(x))


@dataclasses.dataclass
class RunParams:
    """run_params (src/derived_types.f90:56-100), after read_control_file."""
    mode: int = 301
    lattice: str = "fcc"
    lattice_parameter: float = 3.57
    n_1: int = 4
    n_2: int = 4
    n_3: int = 4
    n_basis: int = 1
    n_species: int = 4
    interaction_file: str = "V_ijs.txt"
    interaction_range: int = 0
    wc_range: int = 2
    static_seed: bool = False
    species_names: list = dataclasses.field(default_factory=list)
    # index 0..n_species with entry 0 == 0.0, as allocated at src/io.f90:242
    species_concentrations: np.ndarray = None
    species_numbers: np.ndarray = None

    @property
    def n_atoms(self) -> int:
        cells = self.n_1 * self.n_2 * self.n_3
        return {"simple_cubic": 8, "bcc": 2, "fcc": 4}[self.lattice] * cells

    def numbers_or_none(self):
        """species_numbers when they define the composition (they sum to
        n_atoms, src/initialise.F90:468), else None."""
        if self.species_numbers is not None and int(self.species_numbers.sum()) == self.n_atoms:
            return self.species_numbers
        return None


def read_control_file(path: str) -> RunParams:
    if not os.path.exists(path):
        raise FileNotFoundError(f"Could not find input file {path}")
    p = RunParams()
    lines = open(path).read().splitlines()
    seen = set()
    for line in lines:
        label, value = _split(line)
        if label is None:
            continue
        try:
            if label == "mode":
                p.mode = _fortran_int(value)
            elif label == "lattice":
                p.lattice = _first_token(value)
            elif label == "lattice_parameter":
                p.lattice_parameter = _fortran_real(value)
            elif label in ("n_1", "n_2", "n_3", "n_species", "interaction_range", "wc_range"):
                setattr(p, label, _fortran_int(value))
            elif label == "interaction_file":
                p.interaction_file = _first_token(value)
            elif label == "static_seed":
                p.static_seed = _fortran_logical(value)
            else:
                continue
            seen.add(label)
        except ValueError:
            continue
    # second pass once n_species is known (src/io.f90:238-290)
    p.species_concentrations = np.zeros(p.n_species + 1, dtype=np.float64)
    p.species_numbers = np.zeros(p.n_species, dtype=np.int64)
    for line in lines:
        label, value = _split(line)
        if label == "species_names":
            p.species_names = [t for t in re.split(r"[\s,]+", value.strip()) if t][: p.n_species]
            seen.add(label)
        elif label == "species_concentrations":
            p.species_concentrations[1:] = _fortran_list(value, _fortran_real, p.n_species)
        elif label == "species_numbers":
            p.species_numbers[:] = _fortran_list(value, _fortran_int, p.n_species)
    required = ["mode", "lattice", "lattice_parameter", "n_1", "n_2", "n_3", "n_species",
                "interaction_file", "interaction_range", "species_names"]
    missing = [r for r in required if r not in seen]
    if missing:
        raise ValueError(f"Missing '{missing[0]}' in system file")
    return p


@dataclasses.dataclass
class MetropolisParams:
    """metropolis_params (src/derived_types.f90:141-226)."""
    mode: str = ""
    n_mc_steps: int = 0
    burn_in_start: bool = False
    burn_in: bool = False
    n_burn_in_steps: int = 0
    n_sample_steps: int = 0
    calculate_energies: bool = True
    write_trajectory_energy: bool = False
    calculate_asro: bool = True
    write_trajectory_asro: bool = False
    n_sample_steps_asro: int = 0
    calculate_alro: bool = False
    n_sample_steps_alro: int = 0
    write_trajectory_xyz: bool = False
    n_sample_steps_trajectory: int = 0
    write_initial_config_xyz: bool = False
    write_initial_config_nc: bool = False
    write_final_config_xyz: bool = False
    write_final_config_nc: bool = False
    read_start_config_nc: bool = False
    start_config_file: str = ""
    T: float = 0.0
    T_steps: int = 1
    delta_T: float = 1.0
    nbr_swap: bool = False


_MET_INT = {"n_mc_steps", "n_burn_in_steps", "n_sample_steps", "n_sample_steps_asro",
            "n_sample_steps_alro", "n_sample_steps_trajectory", "T_steps"}
_MET_LOG = {"burn_in_start", "burn_in", "calculate_energies", "write_trajectory_energy",
            "calculate_asro", "write_trajectory_asro", "calculate_alro", "write_trajectory_xyz",
            "write_initial_config_xyz", "write_initial_config_nc", "write_final_config_xyz",
            "write_final_config_nc", "read_start_config_nc", "nbr_swap"}
_MET_REAL = {"T", "delta_T"}


def read_metropolis_file(path: str) -> MetropolisParams:
    if not os.path.exists(path):
        raise FileNotFoundError(f"Could not find input file {path}")
    m = MetropolisParams()
    seen = set()
    for line in open(path).read().splitlines():
        label, value = _split(line)
        if label is None:
            continue
        try:
            if label == "mode":
                m.mode = _first_token(value)
            elif label in _MET_INT:
                setattr(m, label, _fortran_int(value))
            elif label in _MET_LOG:
                setattr(m, label, _fortran_logical(value))
            elif label in _MET_REAL:
                setattr(m, label, _fortran_real(value))
            elif label == "start_config_file":
                m.start_config_file = _first_token(value)
            else:
                continue
            seen.add(label)
        except ValueError:
            continue
    # src/io.f90:654-662 (the first test checks n_sample_steps_alro)
    if m.n_sample_steps_alro == 0:
        m.n_sample_steps_asro = m.n_sample_steps
    if m.n_sample_steps_alro == 0:
        m.n_sample_steps_alro = m.n_sample_steps
    if m.n_sample_steps_trajectory == 0:
        m.n_sample_steps_trajectory = m.n_sample_steps
    for key, msg in (("mode", "mode"), ("n_mc_steps", "n_mc_steps"),
                     ("n_sample_steps", "n_sample_steps"), ("T", "T")):
        if key not in seen:
            raise ValueError(f"Missing '{msg}' in Metropolis input file")
    if m.burn_in:
        m.burn_in_start = True
    return m


@dataclasses.dataclass
class NSParams:
    """ns_params (src/derived_types.f90:242-255)."""
    n_walkers: int = 0
    n_steps: int = 0
    n_iter: int = 0
    traj_freq: int = 0
    outfile_ener: str = ""
    outfile_traj: str = ""


def read_ns_file(path: str) -> NSParams:
    p = NSParams()
    for line in open(path).read().splitlines():
        label, value = _split(line)
        if label in ("n_walkers", "n_steps", "n_iter", "traj_freq"):
            setattr(p, label, _fortran_int(value))
        elif label in ("outfile_ener", "outfile_traj"):
            setattr(p, label, _first_token(value))
    return p


@dataclasses.dataclass
class WLParams:
    """wl_params (src/derived_types.f90:322-350).  The real fields are
    single precision in the reference and are kept rounded to float32."""
    mc_sweeps: int = 0
    bins: int = 0
    num_windows: int = 0
    bin_overlap: float = 0.0
    tolerance: float = 0.0
    flatness: float = 0.0
    wl_f: float = 0.0
    energy_min: float = 0.0
    energy_max: float = 0.0
    radial_samples: int = 0
    performance: int = 0
    nbr_swap: bool = False


def read_wl_file(path: str) -> WLParams:
    p = WLParams()
    for line in open(path).read().splitlines():
        label, value = _split(line)
        if label in ("mc_sweeps", "bins", "num_windows", "radial_samples", "performance"):
            setattr(p, label, _fortran_int(value))
        elif label in ("bin_overlap", "tolerance", "flatness", "wl_f", "energy_min", "energy_max"):
            setattr(p, label, _f32(_fortran_real(value)))
        elif label == "nbr_swap":
            p.nbr_swap = _fortran_logical(value)
    return p


def read_exchange(path: str, n_species: int, interaction_range: int) -> np.ndarray:
    """V_ex(n_species, n_species, interaction_range) in Ry, Fortran order."""
    toks = open(path).read().replace(",", " ").split()
    need = n_species * n_species * interaction_range
    if len(toks) < need:
        raise ValueError(f"{path}: expected {need} values, found {len(toks)}")
    vals = np.array([float(t.lower().replace("d", "e")) for t in toks[:need]], dtype=np.float64)
    return vals.reshape((n_species, n_species, interaction_range), order="F")


def lattice_id(name: str) -> int:
    """0 simple cubic, 1 bcc, 2 fcc -- the C-ABI's lattice codes."""
    try:
        return {"simple_cubic": 0, "sc": 0, "bcc": 1, "fcc": 2}[name]
    except KeyError:
        raise ValueError("Lattice type not yet implemented!") from None
