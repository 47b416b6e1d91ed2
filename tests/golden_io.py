"""Loaders for the committed golden fixtures (tests/golden/) and helpers that
drive a run from the reference's own input files."""
from __future__ import annotations

import gzip
import os

import numpy as np

from brawl_gb300 import inputs as I

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def path(test: str, name: str) -> str:
    return os.path.join(GOLDEN, test, name)


def text(test: str, name: str) -> list[str]:
    with gzip.open(path(test, name + ".gz"), "rt") as f:
        return f.readlines()


def npz(test: str, name: str) -> dict:
    with np.load(path(test, name)) as d:
        return {k: d[k] for k in d.files}


def config_zyx(test: str, name: str) -> np.ndarray:
    """configuration(b, x, y, z) as int8, viewed C-ordered as (z, y, x)."""
    c = npz(test, name)["configuration"]
    return np.ascontiguousarray(c[:, :, :, 0].astype(np.int8))


def load_inputs(test: str):
    p = I.read_control_file(path(test, "brawl.inp"))
    V = I.read_exchange(path(test, p.interaction_file), p.n_species, p.interaction_range)
    return p, V


def anneal_params(p, m) -> dict:
    return dict(T=m.T, delta_T=m.delta_T, T_steps=m.T_steps, n_mc_steps=m.n_mc_steps,
                n_burn_in_steps=m.n_burn_in_steps, n_sample_steps=m.n_sample_steps,
                n_sample_steps_asro=m.n_sample_steps_asro,
                n_sample_steps_alro=m.n_sample_steps_alro,
                n_sample_steps_trajectory=m.n_sample_steps_trajectory,
                burn_in=int(m.burn_in), burn_in_start=int(m.burn_in_start),
                calculate_energies=int(m.calculate_energies),
                calculate_asro=int(m.calculate_asro), nbr_swap=int(m.nbr_swap),
                wc_range=p.wc_range)
