"""The oracle against the reference's own golden outputs
(tests/99_ref of the BraWl repository, committed under tests/golden/)."""
import numpy as np
import pytest

from brawl_gb300 import inputs as I
from brawl_gb300 import output as OUT
from oracle import oracle as O
from tests import golden_io as G

MET = [("01_serial_metropolis", 0)] + [("02_parallel_metropolis", r) for r in range(4)]


def test_mt19937_matches_reference_source():
    """The restated generator emits the same words as the reference's own
    src/mt19937ar.c (compiled from source into oracle/_ref when the reference
    is present), and the published MT19937 check value."""
    import os
    r = O.OracleRng(5489)
    words = [r.u32() for _ in range(10000)]
    assert words[9999] == 4123659995  # 10000th output for seed 5489
    O.build(ref=True)
    if os.path.exists(O.REF_MT_PATH):
        for seed in (110179, 110190, 5489, 1):
            ref = O.reference_mt_words(seed, 3000)
            r = O.OracleRng(seed)
            assert np.array_equal(ref, np.array([r.u32() for _ in range(3000)], dtype=np.uint32))


def _run_anneal(test, rank):
    p, V = G.load_inputs(test)
    m = I.read_metropolis_file(G.path(test, "metropolis.inp"))
    mod = O.OracleModel(p.lattice, p.n_1, p.n_2, p.n_3, V)
    rng = O.OracleRng(O.lib().bo_static_seed(rank))
    cfg, _ = mod.initial_setup(rng, p.species_concentrations, p.numbers_or_none())
    out = mod.anneal(cfg, rng, G.anneal_params(p, m))
    return p, out


@pytest.mark.parametrize("test,rank", MET)
def test_anneal_golden(test, rank):
    p, out = _run_anneal(test, rank)
    tag = "proc_%04d" % rank
    assert np.array_equal(out["initial_configs"][0],
                          G.config_zyx(test, tag + "_initial_config_at_0300.0.npz"))
    assert np.array_equal(out["final_configs"][0],
                          G.config_zyx(test, tag + "_final_config_at_0300.0.npz"))
    lines = [OUT.energy_trajectory_header()] + [
        OUT.energy_trajectory_line(s, e) for s, e in zip(out["traj_step"], out["traj_energy"])]
    assert lines == G.text(test, tag + "_energy_trajectory_at_T_0300.0.dat")
    lines = [OUT.asro_trajectory_header()] + [
        OUT.asro_trajectory_line(s, a) for s, a in zip(out["traj_step"], out["traj_asro"])]
    assert lines == G.text(test, tag + "_asro_trajectory_at_T_0300.0.dat")
    rho = G.npz(test, tag + "_rho_of_T.npz")
    assert np.array_equal(rho["rho_data"], out["rho_of_T"])
    assert np.array_equal(rho["r_data"], out["shells"])
    assert np.array_equal(rho["T_data"], out["temperature"])
    assert np.array_equal(rho["U_data"], out["energies_of_T"])
    if test.startswith("02"):
        diag = OUT.diagnostics_lines(out["temperature"], out["energies_of_T"], out["C_of_T"],
                                     out["acceptance_of_T"])
        assert diag == G.text(test, tag + "_energy_diagnostics.dat")


def test_ensemble_average_golden():
    """comms_reduce_metropolis_results (src/comms.F90:122-160): the rank sum
    in rank order, divided by the number of ranks."""
    test = "02_parallel_metropolis"
    outs = [_run_anneal(test, r)[1] for r in range(4)]
    av = {}
    for k in ("energies_of_T", "C_of_T", "acceptance_of_T", "rho_of_T"):
        s = outs[0][k]
        for o in outs[1:]:
            s = s + o[k]
        av[k] = s / 4.0
    diag = OUT.diagnostics_lines(outs[0]["temperature"], av["energies_of_T"], av["C_of_T"],
                                 av["acceptance_of_T"])
    assert diag == G.text(test, "av_energy_diagnostics.dat")
    ref = G.npz(test, "av_radial_density.npz")
    assert np.array_equal(ref["rho_data"], av["rho_of_T"])
    assert np.array_equal(ref["U_data"], av["energies_of_T"])


def test_total_energy_matches_golden_configs():
    """The first and last trajectory energies recompute from the golden
    configurations alone."""
    for test, rank in MET:
        p, V = G.load_inputs(test)
        mod = O.OracleModel(p.lattice, p.n_1, p.n_2, p.n_3, V)
        tag = "proc_%04d" % rank
        traj = G.text(test, tag + "_energy_trajectory_at_T_0300.0.dat")
        for name, line in (("_initial_config_at_0300.0.npz", traj[1]),
                           ("_final_config_at_0300.0.npz", traj[-1])):
            e = mod.total_energy(G.config_zyx(test, tag + name))
            assert OUT.energy_trajectory_line(int(line.split()[0]), e) == line


def test_nested_sampling_golden_statistical():
    """The committed .energies fixture of tests/99_ref/03_serial_nested_sampling
    is not reproduced bit-for-bit by the current reference source (its first
    line already differs for every seed and input reading tried; the
    reference's CI does not check it).  The oracle's NS is checked here for
    format and statistical agreement of the ceiling trajectory; its primitives
    are pinned bit-exactly by the Metropolis goldens."""
    test = "03_serial_nested_sampling"
    p, V = G.load_inputs(test)
    ns = I.read_ns_file(G.path(test, "ns_input.inp"))
    mod = O.OracleModel(p.lattice, p.n_1, p.n_2, p.n_3, V)
    rng = O.OracleRng(O.lib().bo_static_seed(0))
    limits, _, _, _ = mod.ns_run(rng, p.species_concentrations, p.numbers_or_none(), ns.n_walkers,
                                 ns.n_steps, ns.n_iter)
    golden = G.text(test, "fcc_al_1.00_crfeconi_K100.energies")
    n_at = p.n_1 * p.n_2 * p.n_3 * 1 * p.n_species
    assert golden[0] == OUT.ns_energies_header(ns.n_walkers, n_at)
    g = np.array([float(l.split()[1]) for l in golden[1:]])
    assert all(OUT.ns_energies_line(i + 1, v) == golden[i + 1] for i, v in enumerate(g))
    assert len(limits) == len(g)
    assert np.all(np.diff(limits) <= 0)           # the ceiling never rises
    for lo, hi in ((100, 200), (400, 500), (900, 1000)):
        a, b = limits[lo:hi].mean(), g[lo:hi].mean()
        assert abs(a - b) <= 0.05 * abs(b) + 0.01
