"""GPU nested sampling against the oracle: walker initialisation, every
iteration's ceiling, the final walkers and energies, bit for bit."""
import numpy as np
import pytest

import brawl_gb300 as B
from brawl_gb300 import inputs as I
from oracle import oracle as O
from tests import golden_io as G
from tests.test_gpu_metropolis import conc_vector, equi_numbers, random_V

pytestmark = pytest.mark.gpu

CASES = [
    # lattice, n, ns, nsh, K, n_steps, n_iter, seed
    ("fcc", (3, 3, 3), 5, 4, 20, 40, 120, 7),
    ("bcc", (3, 4, 3), 3, 6, 16, 30, 90, 8),
    ("simple_cubic", (2, 2, 3), 2, 2, 10, 25, 60, 9),
    ("fcc", (2, 2, 2), 4, 6, 12, 20, 50, 10),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}-K{c[4]}")
def test_nested_sampling_matches_oracle(case):
    lattice, n, ns, nsh, K, n_steps, n_iter, seed = case
    rng = np.random.default_rng(seed)
    V = random_V(rng, ns, nsh, 0.08)
    setup = B.Setup(lattice, *n, ns, nsh)
    nums = equi_numbers(setup.n_atoms, ns)
    mod = O.OracleModel(lattice, *n, V)
    r = O.OracleRng(seed)
    limits_o, walkers_o, energies_o, _ = mod.ns_run(r, conc_vector(ns), nums, K, n_steps, n_iter)
    run = dict(setup=setup, V=V, seed=seed, n_walkers=K, n_steps=n_steps,
               species_concentrations=conc_vector(ns), species_numbers=nums)
    nsg = B.NestedSampling([run, run])
    a = n_iter // 3
    lim = np.concatenate([nsg.iterate(a), nsg.iterate(n_iter - a)], axis=1)
    for k in range(2):
        assert np.array_equal(lim[k], limits_o)
        assert np.array_equal(nsg.energies(k), energies_o)
    for w in range(K):
        assert np.array_equal(nsg.walker_config(1, w), walkers_o[w])


def test_nested_sampling_golden_configuration():
    """The reference's own nested-sampling test inputs (fcc 3^3, 5 species,
    4 shells, K = 100, 500 steps, 1000 iterations): the GPU reproduces the
    oracle's ceilings exactly."""
    test = "03_serial_nested_sampling"
    p, V = G.load_inputs(test)
    nsp = I.read_ns_file(G.path(test, "ns_input.inp"))
    mod = O.OracleModel(p.lattice, p.n_1, p.n_2, p.n_3, V)
    r = O.OracleRng(110179)
    limits_o, _, energies_o, _ = mod.ns_run(r, p.species_concentrations, p.numbers_or_none(),
                                            nsp.n_walkers, nsp.n_steps, nsp.n_iter)
    run = dict(setup=B.Setup.from_run_params(p), V=V, seed=110179, n_walkers=nsp.n_walkers,
               n_steps=nsp.n_steps, species_concentrations=p.species_concentrations,
               species_numbers=p.numbers_or_none())
    nsg = B.NestedSampling([run])
    lim = nsg.iterate(nsp.n_iter)[0]
    assert np.array_equal(lim, limits_o)
    assert np.array_equal(nsg.energies(0), energies_o)


# The nested-sampling workload's own shape (fcc 6^3, 5 species, 3 shells,
# V uniform +-0.08 eV, K = 1024 walkers, 2000-step walks), for 20
# iterations; and a small-K run on the same lattice that reaches the
# adaptive extra_steps branch (src/nested_sampling.f90:129-144): with
# n_at * 0.05 = 54 and 20-step walks, every check at i_iter = K/2, K, ...
# finds fewer than 54 accepted steps and lengthens the walks.
SHAPE_CASES = [
    # lattice, n, ns, nsh, K, n_steps, n_iter, seed
    ("fcc", (6, 6, 6), 5, 3, 1024, 2000, 20, 31),
    ("fcc", (6, 6, 6), 5, 3, 8, 20, 120, 32),
]


@pytest.mark.parametrize("case", SHAPE_CASES, ids=lambda c: f"{c[0]}-{c[1]}-K{c[4]}")
def test_nested_sampling_workload_shape_matches_oracle(case):
    lattice, n, ns, nsh, K, n_steps, n_iter, seed = case
    rng = np.random.default_rng(seed)
    V = random_V(rng, ns, nsh, 0.08)
    setup = B.Setup(lattice, *n, ns, nsh)
    nums = equi_numbers(setup.n_atoms, ns)
    mod = O.OracleModel(lattice, *n, V)
    r = O.OracleRng(seed)
    limits_o, walkers_o, energies_o, acc_o = mod.ns_run(r, conc_vector(ns), nums, K, n_steps,
                                                        n_iter)
    run = dict(setup=setup, V=V, seed=seed, n_walkers=K, n_steps=n_steps,
               species_concentrations=conc_vector(ns), species_numbers=nums)
    nsg = B.NestedSampling([run])
    lim = nsg.iterate(n_iter)[0]
    assert np.array_equal(lim, limits_o)
    assert np.array_equal(nsg.energies(0), energies_o)
    for w in range(0, K, max(1, K // 64)):
        assert np.array_equal(nsg.walker_config(0, w), walkers_o[w])
    c = nsg.counters(0)
    if K < 2 * n_iter:
        # the walks were lengthened: more steps than n_iter * n_steps
        assert c["trials"] > n_iter * n_steps


def test_nested_sampling_rare_species_redraws_match_oracle():
    """A composition with a few atoms of one species (the mixed serving
    stream's Dirichlet draws give such lattices): site 2 is redrawn many
    times per step, and the warp tries ten redraws at once; the stream,
    the walks and the ceilings must stay the oracle's bit for bit."""
    lattice, n, ns, nsh, K, n_steps, n_iter, seed = "bcc", (4, 3, 5), 2, 3, 8, 30, 40, 41
    rng = np.random.default_rng(seed)
    V = random_V(rng, ns, nsh, 0.05)
    setup = B.Setup(lattice, *n, ns, nsh)
    nums = np.array([setup.n_atoms - 3, 3], dtype=np.int64)
    conc = np.concatenate([[0.0], nums / setup.n_atoms])
    mod = O.OracleModel(lattice, *n, V)
    r = O.OracleRng(seed)
    limits_o, walkers_o, energies_o, _ = mod.ns_run(r, conc, nums, K, n_steps, n_iter)
    run = dict(setup=setup, V=V, seed=seed, n_walkers=K, n_steps=n_steps,
               species_concentrations=conc, species_numbers=nums)
    nsg = B.NestedSampling([run])
    lim = nsg.iterate(n_iter)[0]
    assert np.array_equal(lim, limits_o)
    assert np.array_equal(nsg.energies(0), energies_o)
    for w in range(K):
        assert np.array_equal(nsg.walker_config(0, w), walkers_o[w])
